/* Oracle case: D3Q19 LBGK 16^3 with gravity along z (periodic in z),
 * solid bottom/top walls in y and specular-slip walls in x.  Exercises Guo
 * forcing and the 3D macroscopic step's handling of F_z. */
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
#define L_RE 60
#define L_NO_FLOW
#define L_GRAVITY_ON
#define L_GRAVITY_FORCE 0.04
#define L_GRAVITY_DIRECTION eZDirection
#define L_WALL_LEFT eSlip
#define L_WALL_RIGHT eSlip
#define L_WALL_BOTTOM eSolid
#define L_WALL_TOP eSolid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 0
#define L_NUM_REGIONS 0
#include "luma_case_tail.h"
#endif
