/* Oracle case: D3Q19 LBGK channel 40 x 20 x 20 with a rigid BFL sphere (the
 * reference's CIRCLE_SPHERE BFL prefab in 3D: Fibonacci points, radius
 * 0.15 = 3 lu, centred at (0.6, 0.5, 0.5) before the wall shift) read from
 * input/geometry.config, with L_LD_OUT for the per-marker momentum-exchange
 * force.  Forced-equilibrium uniform inlet u = 0.04 lu, extrapolate-right
 * outlet, solid bottom/top, periodic front/back; Re 10 (tau 0.74). */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 20
#define L_TIMESTEP (1.0 / 500.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 10
#define L_NO_FLOW
#define L_LD_OUT
#define L_GEOMETRY_FILE
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
