/* Oracle case: D2Q9 LBGK channel, 48 x 24 nodes, forced-equilibrium
 * velocity inlet with a uniform profile ramped over 0.3 dimensionless time
 * units, extrapolate-right outlet, solid bottom/top walls. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 24
#define L_TIMESTEP (1.0 / 480.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 40
#define L_NO_FLOW
#define L_VELOCITY_RAMP 0.3
#define L_WALL_LEFT eVelocity
#define L_WALL_RIGHT eExtrapolateRight
#define L_WALL_BOTTOM eSolid
#define L_WALL_TOP eSolid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 0
#define L_NUM_REGIONS 0
#include "luma_case_tail.h"
#endif
