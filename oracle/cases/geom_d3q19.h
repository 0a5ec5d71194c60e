/* Oracle case: D3Q19 LBGK channel 40 x 20 x 20 with IBM and the geometry
 * reader on, for checking the reader's prefab bodies (sphere, cube, plate,
 * rigid filaments) against the restatement; uniform inlet, extrapolate-right
 * outlet, solid bottom/top. */
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
#define L_RE 100
#define L_NO_FLOW
#define L_IBM_ON
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
