/* Oracle case (with L_COMPUTE_TIME_AVERAGED_QUANTITIES): D2Q9 LBGK channel 160 x 64 with a rigid IBM circle (64
 * injected markers, seeded radii around 10 lu), forced-equilibrium uniform
 * inlet u = 0.04 lu, extrapolate-right outlet, solid bottom/top walls. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 32
#define L_TIMESTEP (1.0 / 800.0)
#define L_BX 5.0
#define L_BY 2.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 160
#define L_NO_FLOW
#define L_IBM_ON
#define L_COMPUTE_TIME_AVERAGED_QUANTITIES
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
