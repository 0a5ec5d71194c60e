/* Oracle case: D3Q19 LBGK periodic box 32^3, tau = 0.55
 * (nu_lbm = (1/L_RE) dt/dh^2 = 1/60 with dt = dh/16).  The harness injects the
 * Taylor-Green + noise velocity field. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 32
#define L_TIMESTEP (1.0 / 512.0)
#define L_BX 1.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 0.0
#define L_RE 120
#define L_NO_FLOW
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
