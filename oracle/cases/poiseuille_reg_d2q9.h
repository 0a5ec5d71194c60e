/* Oracle case: D2Q9 LBGK channel, 60 x 30 nodes, regularised velocity inlet
 * (parabolic, ramped over 0.5 dimensionless time units) and regularised
 * pressure outlet, solid bottom/top walls, tau = 0.6. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 30
#define L_TIMESTEP (1.0 / 900.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_PARABOLIC_INLET
#define L_UX0 1.0
#define L_RE 30
#define L_NO_FLOW
#define L_REGULARISED_BOUNDARIES
#define L_VELOCITY_RAMP 0.5
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
