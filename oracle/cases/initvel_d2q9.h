/* Oracle case: D2Q9 LBGK channel 40 x 20 whose level-0 velocity is read from
 * input/initial_velocity.in (L_INIT_VELOCITY_FROM_FILE): uniform inlet,
 * extrapolate-right outlet, solid bottom/top walls. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 20
#define L_TIMESTEP (1.0 / 400.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 50
#define L_INIT_VELOCITY_FROM_FILE
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
