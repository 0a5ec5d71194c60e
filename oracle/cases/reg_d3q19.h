/* Oracle case: D3Q19 LBGK channel 24 x 12 x 12 nodes, regularised uniform
 * velocity inlet (ramped over 0.2 dimensionless time units) and regularised
 * pressure outlet, solid bottom/top walls (the inlet and outlet faces meet
 * them in edges, whose density is extrapolated), periodic front/back. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 12
#define L_TIMESTEP (1.0 / 300.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_UX0 1.0
#define L_RE 20
#define L_NO_FLOW
#define L_REGULARISED_BOUNDARIES
#define L_VELOCITY_RAMP 0.2
#define L_WALL_LEFT eVelocity
#define L_WALL_RIGHT ePressure
#define L_WALL_BOTTOM eSolid
#define L_WALL_TOP eSolid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 0
#define L_NUM_REGIONS 0
#include "luma_case_tail.h"
#endif
