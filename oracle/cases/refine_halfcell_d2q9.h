/* Oracle case: D2Q9 LBGK channel 16 x 8 with one embedded refined region
 * (level 1) whose limits fall on half coarse cells (x in [0.625, 2.125], y in
 * [0.375, 1.625]: std::round takes them away from zero): forced-equilibrium
 * uniform inlet, extrapolate-right outlet, solid bottom/top walls. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 4
#define L_TIMESTEP (1.0 / 80.0)
#define L_BX 4.0
#define L_BY 2.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 50
#define L_NO_FLOW
#define L_WALL_LEFT eVelocity
#define L_WALL_RIGHT eExtrapolateRight
#define L_WALL_BOTTOM eSolid
#define L_WALL_TOP eSolid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 1
#define L_NUM_REGIONS 1
#define LUMA_CASE_REF_START_X {0.625}
#define LUMA_CASE_REF_END_X {2.125}
#define LUMA_CASE_REF_START_Y {0.375}
#define LUMA_CASE_REF_END_Y {1.625}
#define LUMA_CASE_REF_START_Z {0.0}
#define LUMA_CASE_REF_END_Z {0.0}
#include "luma_case_tail.h"
#endif
