/* Oracle case: D2Q9 KBC periodic box 64 x 64, tau = 0.505
 * (dt = dh/16, L_RE = 2400).  The harness injects the velocity field. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 64
#define L_TIMESTEP (1.0 / 1024.0)
#define L_BX 1.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 0.0
#define L_RE 2400
#define L_NO_FLOW
#define L_USE_KBC_COLLISION
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
