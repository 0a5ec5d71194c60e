/* Oracle case: D3Q19 LBGK channel 48 x 24 x 24 with a rigid IBM sphere
 * (Fibonacci layout, injected markers), forced-equilibrium uniform inlet
 * u = 0.04 lu, extrapolate-right outlet, solid bottom/top walls, periodic
 * front/back. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 16
#define L_TIMESTEP (1.0 / 400.0)
#define L_BX 3.0
#define L_BY 1.5
#define L_BZ 1.5
#define L_UX0 1.0
#define L_RE 40
#define L_NO_FLOW
#define L_IBM_ON
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
