/* Oracle case: D3Q19 LBGK periodic box 12 x 8 x 6 whose velocity is read from
 * input/initial_velocity.in (L_INIT_VELOCITY_FROM_FILE). */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 4
#define L_TIMESTEP (1.0 / 80.0)
#define L_BX 3.0
#define L_BY 2.0
#define L_BZ 1.5
#define L_UX0 0.0
#define L_RE 10
#define L_INIT_VELOCITY_FROM_FILE
#define L_WALL_LEFT eFluid
#define L_WALL_RIGHT eFluid
#define L_WALL_BOTTOM eFluid
#define L_WALL_TOP eFluid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 0
#define L_NUM_REGIONS 0
#include "luma_case_tail.h"
#endif
