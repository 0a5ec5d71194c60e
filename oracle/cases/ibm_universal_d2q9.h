/* Oracle case: D2Q9 LBGK channel 80 x 40 with IB bodies read from
 * input/geometry.config and one epsilon system over all of them
 * (L_UNIVERSAL_EPSILON_CALC);
 * forced-equilibrium uniform inlet u = 0.04 lu, extrapolate-right outlet. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 40
#define L_TIMESTEP (1.0 / 1000.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 100
#define L_NO_FLOW
#define L_IBM_ON
#define L_GEOMETRY_FILE
#define L_UNIVERSAL_EPSILON_CALC
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
