/*
 * luma_gpu.h — C ABI of the GB300 lattice-Boltzmann time step.
 *
 * This is the drop-in boundary for LUMA's hot path.  The reference has no
 * plugin or FFI layer: its seam is the C++ member functions
 *   void GridObj::LBM_multi_opt(int subcycle = 0)      (LUMA inc/GridObj.h:188,
 *        body src/GridObj_ops_lbm_optimised.cpp:36-193, called from
 *        src/main_lbm.cpp:441 and recursively from :45-49)
 *   void ObjectManager::ibm_apply(GridObj*, bool)      (LUMA inc/ObjectManager.h:142,
 *        body src/ObjectManager_ops_ibm.cpp:33-54)
 * whose state is the GridObj members f, fNew, u, rho, force_xyz, LatTyp,
 * omega, dt, dh, ux_in/uy_in/uz_in, CoarseLims and the sub-grid tree
 * (LUMA inc/GridObj.h:54-127).  A host shim compiled into those member
 * functions forwards to the entry points below.
 *
 * Conventions
 *  - Every entry point returns an int status: LUMA_OK (0) or a negative
 *    LUMA_E_* code; none throws or exits.  luma_gpu_last_error_string()
 *    describes the most recent failure on the calling thread.
 *  - Host arrays passed in or out use the reference's layout: site index
 *    id = k + j*K + i*K*M (src/GridObj_ops_lbm_optimised.cpp:79); per-site
 *    vectors are interleaved, f[v + id*Q], u[d + id*dims]
 *    (LUMA inc/IVector.h:94-101).  The device keeps its own layout
 *    (structure of arrays, FP64 or shifted FP32) and converts on transfer.
 *  - Plain C types only; handles are opaque.
 */
#ifndef LUMA_GPU_H
#define LUMA_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LUMA_GPU_ABI_VERSION 2

/* Status codes. */
#define LUMA_OK 0
#define LUMA_E_INVALID (-1)     /* bad argument or unsupported configuration */
#define LUMA_E_CUDA (-2)        /* a CUDA runtime call failed */
#define LUMA_E_NOMEM (-3)       /* device or host allocation failed */
#define LUMA_E_STATE (-4)       /* call not valid in the handle's current state */
#define LUMA_E_TIMEOUT (-5)     /* a bounded device-side wait gave up */
#define LUMA_E_NUMERIC (-6)     /* watchdog found a non-finite or drifting value */
#define LUMA_E_DOMAIN (-7)      /* e.g. an IBM marker left the grid */

/* Site labels: the values of the reference's eType
 * (LUMA inc/Enumerations.h:84-96). */
enum {
    LUMA_SITE_SOLID = 0,
    LUMA_SITE_FLUID = 1,
    LUMA_SITE_REFINED = 2,
    LUMA_SITE_TL_TO_COARSER = 3,
    LUMA_SITE_TL_TO_FINER = 4,
    LUMA_SITE_BFL = 5,
    LUMA_SITE_VELOCITY = 6,
    LUMA_SITE_PRESSURE = 7,
    LUMA_SITE_SLIP = 8,
    LUMA_SITE_EXTRAPOLATE_RIGHT = 9
};

/* Storage / arithmetic precision of the populations. */
enum {
    LUMA_PREC_FP64 = 0,          /* the reference's arithmetic */
    LUMA_PREC_FP32_SHIFTED = 1   /* stores f_i - w_i*rho0 in FP32, collides in FP32 */
};

/* Collision operator (definitions.h L_USE_KBC_COLLISION / L_USE_BGKSMAG). */
enum {
    LUMA_COLL_BGK = 0,           /* _LBM_collide_opt, :765-790 */
    LUMA_COLL_BGK_SMAG = 1,      /* _LBM_collide_opt with _LBM_smag, :717-756 */
    LUMA_COLL_KBC = 2            /* _LBM_kbcCollide_opt, :1122-1305 */
};

/* Feature flags (compile-time switches of the reference's definitions.h). */
#define LUMA_FLAG_REGULARISED 0x1   /* L_REGULARISED_BOUNDARIES */
#define LUMA_FLAG_IBM 0x2           /* L_IBM_ON: split loop, Guo forcing, IBM pass */
#define LUMA_FLAG_GRAVITY 0x4       /* L_GRAVITY_ON */
#define LUMA_FLAG_FIX_MACRO3D 0x8   /* add 0.5*F_z to z-momentum (the reference adds it
                                       to x, src/GridObj_ops_lbm_optimised.cpp:833) */
#define LUMA_FLAG_FIX_KBC 0x10      /* KBC relaxes the streamed populations (the reference
                                       relaxes the pre-stream f, :1147,1296) */
#define LUMA_FLAG_TWO_BUFFER 0x20   /* keep the two-buffer step even where the in-place
                                       (AA-pattern) step applies */
#define LUMA_FLAG_TIME_AVERAGES 0x80 /* L_COMPUTE_TIME_AVERAGED_QUANTITIES: running means of rho, u_p
                                        and u_p u_q (p <= q) updated by every macroscopic update
                                        (_LBM_macro_opt, :895-917); not with regularised BCs or
                                        flexible bodies (LUMA_E_INVALID) */
#define LUMA_FLAG_UNIVERSAL_EPSILON 0x100 /* L_UNIVERSAL_EPSILON_CALC: one epsilon system over all IB
                                              bodies of the grid's level (rigid bodies, one region per
                                              level) */
#define LUMA_FLAG_SPLIT_INTERIOR 0x40 /* two-buffer step: run interior fluid sites in their
                                       own kernel at any grid size (by default only grids
                                       of 2^14 sites or more split) */

/* Description of one grid (one level/region of the hierarchy).  Mirrors the
 * GridObj members it is filled from; arrays are read during create only. */
typedef struct luma_grid_desc {
    int abi_version;            /* LUMA_GPU_ABI_VERSION */
    int level, region;          /* GridObj::level, region_number */
    int dims, Q;                /* L_DIMS, L_NUM_VELS: (2,9), (3,19) or (3,27) */
    int N, M, K;                /* N_lim, M_lim, K_lim (K = 1 in 2D) */
    int precision;              /* LUMA_PREC_* */
    int collision;              /* LUMA_COLL_* */
    int flags;                  /* LUMA_FLAG_* */
    double omega, dt, dh;       /* GridObj::omega, dt, dh */
    double refinement_ratio;    /* GridObj::refinement_ratio = 2^-level */
    double rho_in;              /* L_RHOIN */
    double velocity_ramp;       /* L_VELOCITY_RAMP (dimensionless time); 0 = no ramp */
    double pressure_delta;      /* GridUnits::pd2dlbm(L_PRESSURE_DELTA) (lattice units) */
    double gravity;             /* GridObj::gravity (lattice units) */
    int gravity_dir;            /* L_GRAVITY_DIRECTION (0,1,2) */
    double csmag;               /* L_CSMAG */
    double global_edges[6];     /* GridManager global edges of L0: xmin,xmax,ymin,ymax,zmin,zmax */
    double wall_thickness[6];   /* L_WALL_THICKNESS_{LEFT,RIGHT,BOTTOM,TOP,FRONT,BACK} */
    int coarse_lims[6];         /* CoarseLimsX/Y/Z [min,max] on the parent (level > 0) */
    const int32_t *lattyp;      /* N*M*K site labels (LUMA_SITE_*) */
    const double *xpos, *ypos, *zpos;    /* XPos[N], YPos[M], ZPos[K] */
    const double *ux_in, *uy_in, *uz_in; /* inlet profile, length M */
    double reynolds_ramp;       /* L_REYNOLDS_RAMP (dimensionless time); 0 = no ramp.  With a ramp every
                                   step of the grid first sets omega from Re = re * ramp coefficient of
                                   (t+1)*dt (GridObj::_LBM_updateReynolds, src/GridObj_ops_lbm_optimised.cpp:
                                   39-42, 1313-1321) */
    double re;                  /* L_RE (used by the Reynolds ramp only) */
} luma_grid_desc;

typedef struct luma_gpu_grid luma_gpu_grid;

/* Reductions over the fluid-updated sites of one grid, accumulated in FP64. */
typedef struct luma_reduction {
    double mass;                /* sum rho */
    double momentum[3];         /* sum rho*u_d */
    double kinetic_energy;      /* sum 0.5*rho*|u|^2 */
    double max_speed;           /* max |u| */
    int64_t nonfinite;          /* count of non-finite rho/u values */
} luma_reduction;

/* ---- version / errors -------------------------------------------------- */
/* No counterpart in the reference: its failures go through L_ERROR
 * (inc/stdafx.h:127-149), which logs and exits; here the ABI version and
 * the calling thread's last error message. */
int luma_gpu_abi_version(void);
const char *luma_gpu_last_error_string(void);

/* ---- grid lifetime ------------------------------------------------------ */
/* Replaces GridObj(int level) / GridObj(int region, GridObj& parent) and
 * LBM_addSubGrid (LUMA src/GridObj.cpp:51-118): allocates device state for
 * one grid; `parent` is NULL for level 0, else the parent's handle (the new
 * grid becomes its next sub-grid, in region order). */
int luma_gpu_grid_create(const luma_grid_desc *desc, luma_gpu_grid *parent, luma_gpu_grid **out);
/* Destroys a grid and its sub-grids: GridObj::~GridObj
 * (src/GridObj.cpp:39) over the tree, as `delete Grids` (src/main_lbm.cpp:667). */
int luma_gpu_grid_destroy(luma_gpu_grid *grid);
/* No counterpart in the reference (its step runs on the calling host
 * thread).  Selects the CUDA stream (a cudaStream_t, may be NULL for the
 * legacy stream) used by every subsequent call on this grid tree. */
int luma_gpu_set_stream(luma_gpu_grid *root, void *cuda_stream);

/* ---- state transfer ------------------------------------------------------ */
/* The state the reference keeps in GridObj::f, u, rho, force_xyz
 * (inc/GridObj.h:54-127).
 * Host -> device: f (N*M*K*Q), u (N*M*K*dims), rho (N*M*K); force_xyz may be
 * NULL and is ignored on grids without IBM or gravity forcing.  Arrays in the reference layout (post-collision f, as GridObj::f
 * holds between time steps).  Sets the grid's step counter to t. */
int luma_gpu_upload_state(luma_gpu_grid *grid, const double *f, const double *u,
                          const double *rho, const double *force_xyz, int t);
/* Device -> host into the GridObj members' layout (inc/GridObj.h:54-127);
 * any pointer may be NULL to skip it. */
int luma_gpu_download_state(luma_gpu_grid *grid, double *f, double *u, double *rho,
                            double *force_xyz);
/* Running means of a grid created with LUMA_FLAG_TIME_AVERAGES
 * (GridObj::rho_timeav, ui_timeav, uiuj_timeav, inc/GridObj.h:93-95;
 * reference layout: N*M*K,
 * N*M*K*dims, N*M*K*(3*dims-3) with the (p, q >= p) pairs in order). */
int luma_gpu_download_time_averages(luma_gpu_grid *grid, double *rho_ta, double *ui_ta, double *uiuj_ta);
/* Step counter of a grid (GridObj::t, inc/GridObj.h:111). */
int luma_gpu_get_time(const luma_gpu_grid *grid, int *t);

/* ---- the time step ------------------------------------------------------ */
/* Runs `nsteps` calls of GridObj::LBM_multi_opt()
 * (src/GridObj_ops_lbm_optimised.cpp:36-193, as src/main_lbm.cpp:441 calls it) on the root grid: each
 * recursively advances every sub-grid two sub-steps, then this grid one
 * step (explode/coalesce, IBM pass and collision included).  Asynchronous
 * on the grid's stream.  Inside a step, work forks onto streams the library
 * owns (each grid's sub-grid stream and listed-site stream, of the highest
 * priority) and joins back into the grid's stream before the step ends, so
 * the grid's stream orders everything a step does. */
int luma_gpu_step(luma_gpu_grid *root, int nsteps);
/* No counterpart in the reference (its step is synchronous).  Blocks until
 * all work queued on the grid's stream has finished; reports a site that
 * needed an operation outside the GPU path (LUMA_E_INVALID) or a filament
 * marker that left its grid during the steps (LUMA_E_DOMAIN), for the first
 * grid of the tree with one, and clears that record. */
int luma_gpu_synchronize(luma_gpu_grid *root);

/* ---- decomposed grids: halo planes ----------------------------------------- */
/* A grid cut into slabs along x, one per GPU (or several on one), each slab
 * a grid of its own with one ghost x-plane on each side that holds a copy of
 * the neighbouring slab's edge plane.  After every step each slab exports
 * its first and last real planes and imports its neighbours' into its
 * ghost planes: the exchange MpiManager::mpi_communicate performs with
 * mpi_buffer_pack / mpi_buffer_unpack after every step of a grid
 * (src/MpiManager.cpp:631-820, src/Mpi_buffer_pack.cpp,
 * src/Mpi_buffer_unpk.cpp; called from src/GridObj_ops_lbm_optimised.cpp:189).
 * The planes are the grid's current populations, all Q directions, in the
 * device's storage (FP64, or shifted FP32), direction-major: direction v's
 * nplanes*M*K values, then v+1's.  `buf` is device memory of this or a peer
 * GPU, or pinned host memory.  Stream-ordered on the grid's stream.  Grids
 * created with LUMA_FLAG_TWO_BUFFER only (the in-place step keeps two
 * storage layouts); LUMA_E_INVALID otherwise or for planes off the grid. */
int luma_gpu_planes_bytes(const luma_gpu_grid *grid, int nplanes, size_t *bytes);
int luma_gpu_planes_export(luma_gpu_grid *grid, int i0, int nplanes, void *buf);
int luma_gpu_planes_import(luma_gpu_grid *grid, int i0, int nplanes, const void *buf);

/* ---- reductions / watchdog ----------------------------------------------- */
/* No counterpart in the reference (it keeps no running sums).  FP64 sums
 * over the grid's fluid-updated sites (see luma_reduction), deterministic:
 * the same state gives the same bits.  Blocks until the result is on the
 * host. */
int luma_gpu_reduce(luma_gpu_grid *grid, luma_reduction *out);

/* No counterpart in the reference.  The FP64 reduction of luma_gpu_reduce
 * for callers that cannot allocate device memory — hosts that give the
 * GPU's memory to a fixed pool at start-up and forbid later allocations,
 * real-time loops that cannot afford an allocation's latency or failure —
 * over SoA device arrays they own: typ[n] site labels (uint8, LUMA_SITE_*),
 * rho[n], u[d*n + id] (FP64).  It allocates nothing: its scratch is a fixed
 * 64 KiB device array held by every GPU that loads the library.  At most
 * 16,777,216 sites (larger n is rejected with LUMA_E_INVALID).  The first
 * call on a device sets up that device's scratch address; the address is
 * cached for the process, so the call is
 * not valid after cudaDeviceReset.  Calls share the scratch: calls whose
 * kernels overlap on the GPU race.  Blocks until the result is on the host,
 * so a stream under capture is refused (LUMA_E_INVALID, nothing recorded). */
int luma_gpu_reduce_fields_noalloc(const uint8_t *typ, const double *rho, const double *u, int64_t n,
                                   int dims, void *cuda_stream, luma_reduction *out);

/* ---- immersed-boundary bodies (grids created with LUMA_FLAG_IBM) -------- */
/* Host-only: the set-up luma_gpu_ibm_initialise runs for rigid bodies on one
 * grid (support search, marker spacing ds, epsilon system; the reference's
 * ObjectManager::ibm_initialise, src/ObjectManager_ops_ibm.cpp:190-246),
 * for `nbodies` bodies of nmarkers[b] markers at positions[3*m + d]
 * (bodies concatenated), on the grid `desc` describes (sizes, dh, level,
 * site positions and global_edges read).  universal != 0 solves one
 * epsilon system over all the bodies (L_UNIVERSAL_EPSILON_CALC, :773-920
 * with :1067-1142).  Writes eps, ds and (if not NULL) each marker's
 * support count, per marker.  No device call. */
int luma_ibm_setup_host(const luma_grid_desc *desc, int nbodies, const int *nmarkers, const double *positions,
                        int universal, double *eps, double *ds, int *nsupports);
/* Adds a rigid body of `nmarkers` Lagrangian markers to the grid that owns
 * it: positions[3*m + d] in the reference's length units, optional marker
 * velocities (lattice units, NULL = stationary).  Replaces the body
 * construction of ObjectManager::io_readInGeomConfig / IBBody
 * (LUMA src/ObjectManager_ops_io.cpp:322-800, src/IBBody.cpp:58-91). */
int luma_gpu_ibm_add_body(luma_gpu_grid *grid, int nmarkers, const double *positions,
                          const double *velocities, int *body_index);
/* Support stencils, marker spacing and epsilon for every body of the tree:
 * ObjectManager::ibm_initialise (src/ObjectManager_ops_ibm.cpp:190-246).
 * Call after all bodies are added and before stepping. */
int luma_gpu_ibm_initialise(luma_gpu_grid *root);
/* Adds a flexible filament as the reference's FILAMENT_ARRAY geometry
 * reader builds one (LUMA src/ObjectManager_ops_io.cpp:455-567): IB markers
 * every dh along the filament (inc/Body.h:143-187) and a co-rotational
 * Euler-Bernoulli FEM beam of `nel` elements (src/FEMBody.cpp:48-130),
 * clamped or simply supported at `start` (already shifted by the wall
 * thickness where the reader shifts it); angle_v in degrees; dm =
 * GridObj::dm; fsi_vel_scale = L_UX0*dt/dh (the FSI residual's scale,
 * src/ObjectManager_ops_ibm.cpp:1007).  The beam is planar (x-y plane, 3
 * DOF per node) as the reference's FEM is; on a 3D grid the reference aborts
 * on a matrix-size mismatch in FEMElement::loadVector and
 * FEMBody::updateIBMarkers (src/FEMElement.cpp:153-157,
 * src/FEMBody.cpp:356-361), which here take the x and y components and keep
 * the markers' z (the only change), with the element depth `depth` (2D: dh,
 * src/FEMBody.cpp:103-105).  The FEM (Newmark-beta + Newton-Raphson) and
 * the FSI sub-iterations run on the device. */
int luma_gpu_ibm_add_filament(luma_gpu_grid *grid, const double start[3], double length, double height,
                              double depth, double angle_v, int nel, int clamped, double density,
                              double youngs_modulus, double dm, double fsi_vel_scale, int *body_index);
/* IBMarker state (inc/IBMarker.h:33-74) of one body of the grid,
 * 9 doubles per marker: x y z Fx Fy Fz epsilon ds nsupport
 * (F = the last IBM force of ibm_computeForce, lattice units). */
int luma_gpu_ibm_get_markers(luma_gpu_grid *grid, int body, double *out);
/* FP64 sum over a body's markers of F*epsilon*ds (*ds in 3D): the force the
 * body exerts in lattice units, as io_writeLiftDrag scales it per marker
 * (src/ObjectManager_ops_io.cpp:65-128) before its physical scaling. */
int luma_gpu_ibm_body_force(luma_gpu_grid *grid, int body, double force[3]);

/* ---- bounce-back bodies ---------------------------------------------------- */
/* Momentum-exchange force of the grid's solid sites (bounce-back bodies and,
 * as in the reference, walls): ObjectManager::computeLiftDrag
 * (src/ObjectManager.cpp:93-165), which the reference accumulates during a
 * step under L_LD_OUT from the populations that step streams; here it is
 * computed from the grid's current state (the populations the next step
 * streams), in FP64, in lattice units.  Blocks until the result is on the
 * host. */
int luma_gpu_momex_force(luma_gpu_grid *grid, double force[3]);

/* ---- BFL bodies ------------------------------------------------------------ */
/* Attach BFL body 0 of a grid (ObjectManager::pBody[0], set up by BFLBody:
 * labels, surface closure and link distances, src/BFLBody.cpp:49-142):
 * site_marker[N*M*K] is, per site in id order, the marker
 * Body::getMarkerData finds for the site's position (inc/Body.h:581-614;
 * -1 for none) and q[Q*nmarkers] is BFLBody::Q (q[v + Q*m]; -1 where no wall
 * cuts the link).  The grid's stream then applies _LBM_applyBFL_opt
 * (src/GridObj_ops_lbm_optimised.cpp:1010-1113) on every link it names.
 * A grid whose labels hold LUMA_SITE_BFL sites refuses to step
 * (LUMA_E_STATE) until this is called.  Replaces the per-link position
 * lookups of _LBM_applyBFL_opt. */
int luma_gpu_bfl_set(luma_gpu_grid *grid, const int32_t *site_marker, int nmarkers, const double *q);
/* Per-marker momentum-exchange force (forces[3*m + d], FP64, lattice units)
 * of the latest step: ObjectManager::computeLiftDrag(v, id, g, markerID)
 * (src/ObjectManager.cpp:176-189) summed in the reference's loop order.
 * Blocks until the result is on the host. */
int luma_gpu_bfl_forces(luma_gpu_grid *grid, double *forces);

/* ---- output in the reference's formats ------------------------------------ */
/* GridObj::io_lite(tval, "") (src/GridObj_ops_io.cpp:706-810) for every grid
 * of the tree: <dir>/io_lite.Lev<l>.Reg<r>.Rnk<rank>.<(int)tval>.dat, doubles
 * in fixed notation with `precision` digits (L_OUTPUT_PRECISION).  The state
 * is copied to the host before the call returns; the files are formatted
 * and written by a host thread while the caller steps on (luma_gpu_io_wait
 * joins it).  fNew is the state before the latest step, as the reference's
 * fNew after its swap (on the in-place all-fluid path, f). */
int luma_gpu_io_lite(luma_gpu_grid *root, const char *dir, double tval, int precision, int rank);
/* GridObj::io_restart(eWrite) (src/GridObj_ops_io.cpp:406-490) for the tree:
 * <dir>/restart_LBM_Rnk<rank>.out, level 0 then each sub-grid after its
 * parent; on a tree created with LUMA_FLAG_IBM also, as level 0's call has
 * the ObjectManager do (ObjectManager::io_restart(eWrite),
 * src/ObjectManager_ops_io.cpp:136-190), <dir>/restart_IBBody_Rnk<rank>.out
 * with every IB body of the tree in creation order (a filament's markers
 * where the FEM has moved them, then their initial positions); same
 * snapshot and host-thread scheme as luma_gpu_io_lite. */
int luma_gpu_io_restart(luma_gpu_grid *root, const char *dir, int rank);
/* No counterpart in the reference (its writers are synchronous).  Waits
 * for the tree's pending writers; returns the first error they met. */
int luma_gpu_io_wait(luma_gpu_grid *root);
/* GridObj::io_lite and io_restart(eWrite) (src/GridObj_ops_io.cpp:406-490,
 * 706-810), the two formats from host arrays in the reference layout (f, fnew: N*M*K*Q;
 * u: N*M*K*dims; rho: N*M*K), with the labels, positions, dt, dh and omega
 * of `desc`: the formatting alone, for callers that hold the state.
 * fnew may be NULL (f is written in its place); the three time averages
 * (layout of luma_gpu_download_time_averages) are all NULL or all given and
 * then add the columns the reference writes when it keeps them; `append`
 * adds to an existing restart file, as the reference's sub-grids do. */
int luma_io_lite_write(const luma_grid_desc *desc, const double *f, const double *fnew, const double *u,
                       const double *rho, const double *rho_ta, const double *ui_ta, const double *uiuj_ta,
                       const char *dir, double tval, int precision, int rank);
int luma_io_restart_write(const luma_grid_desc *desc, const double *f, const double *u, const double *rho,
                          const char *path, int append);
/* The IB-body part of the restart (ObjectManager::io_restart(eWrite),
 * src/ObjectManager_ops_io.cpp:136-190; restart_IBBody_Rnk<rank>.out):
 * nmarkers[b] markers per body, positions (3 per marker, bodies in order,
 * e.g. from luma_gpu_ibm_get_markers), flexible[b] non-zero for bodies that
 * also write their old positions (positions0, same layout). */
int luma_io_ibbody_restart_write(const char *path, int nbodies, const int *nmarkers, const int *flexible,
                                 const double *positions, const double *positions0);
/* GridObj::io_restart(eRead) (src/GridObj_ops_io.cpp:490-580) on host
 * arrays: descs[0..ngrids) are the tree's grids with level 0 first (labels
 * not needed; positions, dt, dh, omega, global_edges used), f/u/rho their
 * reference-layout state, overwritten at every site the file names (then
 * upload with luma_gpu_upload_state).  As the reference does, each line's
 * f = feq (1 + dt f_neq / omega) takes feq from level 0's rho and u at the
 * level-0 index of the line's (i, j, k), and level 0's omega. */
int luma_io_restart_read(const char *path, int ngrids, const luma_grid_desc *const *descs, double *const *f,
                         double *const *u, double *const *rho);

/* ---- discrete adjoint of the time-averaged drag ------------------------- */
/* No counterpart in the reference (its objective is the drag that
 * io_writeLiftDrag writes, src/ObjectManager_ops_io.cpp:105-121).
 * Forward: runs `nsteps` ordinary steps from the current state, saving the
 * population state every `checkpoint_every` steps, and returns
 * J = (1/nsteps) sum over the steps of sum over the body's markers of
 * F_x * epsilon * ds (* ds in 3D), lattice units.  Single grid, BGK, rigid
 * bodies; site types fluid, solid, velocity, extrapolate-right; no
 * regularised BCs, gravity or ramp (LUMA_E_INVALID otherwise). */
int luma_gpu_adj_forward(luma_gpu_grid *grid, int nsteps, int checkpoint_every, int body, double *J);
/* No counterpart in the reference.  Backward: once per forward.  Recomputes each checkpoint segment, runs the
 * reverse steps and returns dJ * dJ/ds for the scale s of the velocity of
 * every velocity site (u = s * u_uploaded, at s = 1) and dJ * dJ/dX for the
 * body's marker positions (dims doubles per marker, reference length
 * units; through the supports' delta values, epsilon and ds).  Either
 * output may be NULL.  The grid is left in the state after the forward. */
int luma_gpu_adj_backward(luma_gpu_grid *grid, double dJ, double *grad_inlet_scale, double *grad_markers);
/* No counterpart in the reference.  Device bytes held by the checkpoints
 * and the tape of the last forward. */
int luma_gpu_adj_memory(const luma_gpu_grid *grid, size_t *bytes);

#ifdef __cplusplus
}
#endif
#endif /* LUMA_GPU_H */
