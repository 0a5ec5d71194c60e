/* Oracle case: D2Q9 LBGK channel 80 x 40 with one embedded refined region
 * (level 1) over x in [0.5, 1.0], y in [0.25, 0.75], whose inlet profile is
 * read from input/inlet_profile.in (L_USE_INLET_PROFILE) and which starts
 * from that profile everywhere: extrapolate-right outlet, solid bottom/top
 * walls. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 40
#define L_TIMESTEP (1.0 / 800.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 50
#define L_USE_INLET_PROFILE
#define L_WALL_LEFT eVelocity
#define L_WALL_RIGHT eExtrapolateRight
#define L_WALL_BOTTOM eSolid
#define L_WALL_TOP eSolid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 1
#define L_NUM_REGIONS 1
#define LUMA_CASE_REF_START_X {0.5}
#define LUMA_CASE_REF_END_X {1.0}
#define LUMA_CASE_REF_START_Y {0.25}
#define LUMA_CASE_REF_END_Y {0.75}
#define LUMA_CASE_REF_START_Z {0.0}
#define LUMA_CASE_REF_END_Z {0.0}
#include "luma_case_tail.h"
#endif
