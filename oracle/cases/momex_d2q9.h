/* Oracle case: D2Q9 LBGK Poiseuille channel with L_LD_OUT (the
 * momentum-exchange force of the solid sites), 200 x 100 nodes including the
 * one-cell solid walls at the bottom and top.  Left face: forced-equilibrium
 * velocity inlet with a parabolic profile of peak 1.5*L_UX0*dt/dh = 0.05 lu;
 * right face: zero-gradient (extrapolate-right) outlet.  tau = 0.6
 * (nu_lbm = (1/L_RE)*dt/dh^2 = 1/30).  No ramp, no regularisation. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 100
#define L_TIMESTEP (1.0 / 3000.0)
#define L_BX 2.0
#define L_BY 1.0
#define L_BZ 1.0
#define L_PARABOLIC_INLET
#define L_UX0 1.0
#define L_RE 100
#define L_NO_FLOW
#define L_LD_OUT
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
