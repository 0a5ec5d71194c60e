/* Oracle test infrastructure.  Shared tail of every per-case configuration
 * header used to build the reference's serial oracle.
 *
 * A case header defines LUMA_VERSION and the guard LBM_DEFINITIONS_H (so the
 * reference's own inc/definitions.h is skipped when this header is
 * pre-included with -include), sets the case switches, then includes this
 * file.  The macro names are the reference's configuration interface
 * (inc/definitions.h:1-352); this tail derives the quantities that file
 * derives: cell counts L_N/L_M/L_K (definitions.h:46-48), the coarse site
 * width, the lattice size per dimensionality (definitions.h:300-318), the 2D
 * overrides, and the default single-region refinement arrays. */
#ifndef LUMA_ORACLE_CASE_TAIL_H
#define LUMA_ORACLE_CASE_TAIL_H

#include <time.h>
#include <iostream>
#include <fstream>
#include <vector>
#include <iomanip>
#include <math.h>
#include <string>
#include <limits>
#include <mpi.h>

#define L_N static_cast<int>((L_BX) * L_RESOLUTION)
#define L_M static_cast<int>((L_BY) * L_RESOLUTION)
#define L_K static_cast<int>((L_BZ) * L_RESOLUTION)
#define L_COARSE_SITE_WIDTH (1.0 / static_cast<double>(L_RESOLUTION))

/* Output / IO switches the oracle never uses but the sources name. */
#ifndef L_GRID_OUT_FREQ
#define L_GRID_OUT_FREQ 1000000
#endif
#define L_EXTRA_OUT_FREQ 1000000
#define L_OUTPUT_PRECISION 10
#define L_RESTART_OUT_FREQ 100000000
#define L_PROBE_OUT_FREQ 100000000
#define L_PROBE_NUM_X 0
#define L_PROBE_NUM_Y 0
#define L_PROBE_NUM_Z 0
#define L_PROBE_MIN_X 0.0
#define L_PROBE_MIN_Y 0.0
#define L_PROBE_MIN_Z 0.0
#define L_PROBE_MAX_X 0.0
#define L_PROBE_MAX_Y 0.0
#define L_PROBE_MAX_Z 0.0
#ifndef L_GRAVITY_FORCE
#define L_GRAVITY_FORCE 0.0
#endif
#ifndef L_GRAVITY_DIRECTION
#define L_GRAVITY_DIRECTION eXDirection
#endif
#define L_CSMAG 0.3
#define L_TOTAL_TIMESTEPS 1000000
#define L_MPI_XCORES 1
#define L_MPI_YCORES 1
#define L_MPI_ZCORES 1
#define L_MPI_SD_MAX_ITER 1
#define L_MPI_TOP_XCORES 1
#define L_MPI_TOP_YCORES 1
#define L_MPI_TOP_ZCORES 1
#define L_PHYSICAL_U 1.0
#define L_PHYSICAL_RHO 1000.0
#ifndef L_UY0
#define L_UY0 0.0
#endif
#ifndef L_UZ0
#define L_UZ0 0.0
#endif
#define L_RHOIN 1
#define L_NB_ALPHA 0.25
#define L_NB_DELTA 0.5
#define L_RELAX 0.5
#define L_PRESSURE_DELTA 0.0
#define L_PADDING_X_MIN (-2.0 * dh)
#define L_PADDING_X_MAX (2.0 * dh)
#define L_PADDING_Y_MIN (-2.0 * dh)
#define L_PADDING_Y_MAX (2.0 * dh)
#define L_PADDING_Z_MIN (-2.0 * dh)
#define L_PADDING_Z_MAX (2.0 * dh)
#ifndef L_WALL_THICKNESS_BOTTOM
#define L_WALL_THICKNESS_BOTTOM (1.0 * L_COARSE_SITE_WIDTH)
#define L_WALL_THICKNESS_TOP (1.0 * L_COARSE_SITE_WIDTH)
#define L_WALL_THICKNESS_LEFT (1.0 * L_COARSE_SITE_WIDTH)
#define L_WALL_THICKNESS_RIGHT (1.0 * L_COARSE_SITE_WIDTH)
#define L_WALL_THICKNESS_FRONT (1.0 * L_COARSE_SITE_WIDTH)
#define L_WALL_THICKNESS_BACK (1.0 * L_COARSE_SITE_WIDTH)
#endif

#if L_NUM_LEVELS != 0
static double cRefStartX[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_START_X };
static double cRefEndX[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_END_X };
static double cRefStartY[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_START_Y };
static double cRefEndY[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_END_Y };
static double cRefStartZ[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_START_Z };
static double cRefEndZ[L_NUM_LEVELS][L_NUM_REGIONS] = { LUMA_CASE_REF_END_Z };
#endif

const static int cNumProbes[3] = { L_PROBE_NUM_X, L_PROBE_NUM_Y, L_PROBE_NUM_Z };
const static double cProbeLimsX[2] = { L_PROBE_MIN_X, L_PROBE_MAX_X };
const static double cProbeLimsY[2] = { L_PROBE_MIN_Y, L_PROBE_MAX_Y };
const static double cProbeLimsZ[2] = { L_PROBE_MIN_Z, L_PROBE_MAX_Z };

#if (L_DIMS == 3)
# ifdef L_USE_KBC_COLLISION
#  define L_NUM_VELS 27
# else
#  define L_NUM_VELS 19
# endif
# define L_MPI_DIRS 26
#else
# define L_NUM_VELS 9
# define L_MPI_DIRS 8
# undef L_BZ
# define L_BZ 0
# undef L_K
# define L_K 1
# undef L_UZ0
# define L_UZ0 0.0
# define L_BLOCK_MIN_Z 0.0
# define L_BLOCK_MAX_Z 0.0
#endif

#if L_NUM_LEVELS == 0
static double cRefStartX[1][1] = { {0.0} };
static double cRefEndX[1][1] = { {0.0} };
static double cRefStartY[1][1] = { {0.0} };
static double cRefEndY[1][1] = { {0.0} };
static double cRefStartZ[1][1] = { {0.0} };
static double cRefEndZ[1][1] = { {0.0} };
# undef L_NUM_REGIONS
# define L_NUM_REGIONS 1
#endif

#endif
