/* Oracle case: D3Q19 LBGK periodic box 32^3 with two nested refined regions
 * (levels 1 and 2) centred in the box.  The harness injects a Taylor-Green
 * field on level 0; sub-grids start from rest (L_NO_FLOW). */
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
#define L_NUM_LEVELS 2
#define L_NUM_REGIONS 1
#define LUMA_CASE_REF_START_X {0.25}, {0.375}
#define LUMA_CASE_REF_END_X {0.75}, {0.625}
#define LUMA_CASE_REF_START_Y {0.25}, {0.375}
#define LUMA_CASE_REF_END_Y {0.75}, {0.625}
#define LUMA_CASE_REF_START_Z {0.25}, {0.375}
#define LUMA_CASE_REF_END_Z {0.75}, {0.625}
#include "luma_case_tail.h"
#endif
