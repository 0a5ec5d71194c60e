/* Oracle case: D3Q27 KBC-N4 periodic box 16^3, tau = 0.51
 * (dt = dh/16, L_RE = 300).  The harness injects the velocity field. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 16
#define L_TIMESTEP (1.0 / 256.0)
#define L_BX 1.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 0.0
#define L_RE 300
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
