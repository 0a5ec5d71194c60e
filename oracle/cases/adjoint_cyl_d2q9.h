/* Oracle case: the adjoint workload.  D2Q9 LBGK channel 400 x 160 nodes
 * (one-cell solid walls at the bottom and top), parabolic forced-equilibrium
 * inlet of peak 1.5*L_UX0*dt/dh = 0.05 lu, extrapolate-right outlet, fluid
 * at rest initially; a rigid IBM cylinder of 64 injected markers (diameter
 * 20 lu, seeded radius perturbations) centred 80 lu from the inlet on the
 * centre line.  nu_lbm = (1/L_RE)*dt/dh^2 = 2/75.  No ramp, no
 * regularisation. */
#define LUMA_VERSION "1.7.12"
#ifndef LBM_DEFINITIONS_H
#define LBM_DEFINITIONS_H
#define L_DIMS 2
#define L_RESOLUTION 80
#define L_TIMESTEP (1.0 / 2400.0)
#define L_BX 5.0
#define L_BY 2.0
#define L_BZ 1.0
#define L_PARABOLIC_INLET
#define L_UX0 1.0
#define L_RE 100
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
