/* Oracle build of the reference for the 1D GSPH gradient check: the Sod
 * constants of cfg_sod.h with h = 2 m/rho, so that every particle of a
 * ghost-free tube has more than 20 neighbours inside its CUTOFF2*h box and
 * the reference's calc_gradients (calculate_gradient.cc:162-164) never
 * takes its small-neighbourhood branch.  Force-included after
 * src/plume/parameters.h, which stays untouched. */
#ifndef ORACLE_CFG_GSPH_GRAD_H
#define ORACLE_CFG_GSPH_GRAD_H
static const double oracle_eta_smooth_P = 2.0;
static const double oracle_CFL_P = 0.3;
static const double oracle_Cva_P = 717.5;
#define eta_smooth_P oracle_eta_smooth_P
#define CFL_P oracle_CFL_P
#define Cva_P oracle_Cva_P
#endif
