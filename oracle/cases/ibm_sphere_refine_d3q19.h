/* Oracle case: scaled copy of the refined-sphere workload.  D3Q19 LBGK
 * channel 48 x 24 x 24 (L0) with two nested refined regions centred on a
 * rigid IBM sphere: level 1 over 12^3 base cells (24^3 sites), level 2 over
 * 2^3 base cells (8^3 sites) inside the sphere.  The sphere (diameter 6 base
 * lattice units, 12 on level 1; Fibonacci layout, injected markers) lives on
 * level 1, as in the workload.  Uniform inlet u = 0.04 lu (forced
 * equilibrium), the same velocity everywhere at t = 0, extrapolate-right
 * outlet, periodic lateral faces; tau = 0.548 on L0. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 3
#define L_RESOLUTION 8
#define L_TIMESTEP (0.005)
#define L_BX 6.0
#define L_BY 3.0
#define L_BZ 3.0
#define L_UX0 1.0
#define L_RE 20
#define L_IBM_ON
#define L_WALL_LEFT eVelocity
#define L_WALL_RIGHT eExtrapolateRight
#define L_WALL_BOTTOM eFluid
#define L_WALL_TOP eFluid
#define L_WALL_FRONT eFluid
#define L_WALL_BACK eFluid
#define L_NUM_LEVELS 2
#define L_NUM_REGIONS 1
#define LUMA_CASE_REF_START_X {0.75}, {1.375}
#define LUMA_CASE_REF_END_X {2.25}, {1.625}
#define LUMA_CASE_REF_START_Y {0.75}, {1.375}
#define LUMA_CASE_REF_END_Y {2.25}, {1.625}
#define LUMA_CASE_REF_START_Z {0.75}, {1.375}
#define LUMA_CASE_REF_END_Z {2.25}, {1.625}
#include "luma_case_tail.h"
#endif
