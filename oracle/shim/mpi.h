/* Oracle test infrastructure: a type-only stand-in for <mpi.h> so that the
 * reference's serial build (L_BUILD_FOR_MPI undefined) compiles without an
 * MPI installation.  The reference names these types in declarations even in
 * serial builds (inc/MpiManager.h, inc/definitions.h:40); no MPI call is
 * reachable serially. */
#ifndef LUMA_ORACLE_MPI_SHIM_H
#define LUMA_ORACLE_MPI_SHIM_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
static inline int MPI_Finalize(void) { return 0; }
#endif
