/* Oracle build of the reference for the 1D Sod workload: constants that the
 * workload sets differently from src/plume/parameters.h:1225-1448.  The
 * reference header is left untouched; this header is force-included after it
 * and redirects the names used by the hot-path sources to new constants. */
#ifndef ORACLE_CFG_SOD_H
#define ORACLE_CFG_SOD_H
static const double oracle_eta_smooth_P = 1.3; /* h = 1.3 m/rho            */
static const double oracle_CFL_P = 0.3;        /* CFL 0.3                   */
static const double oracle_Cva_P = 717.5;      /* gamma = 1 + 287/717.5 = 1.4 */
#define eta_smooth_P oracle_eta_smooth_P
#define CFL_P oracle_CFL_P
#define Cva_P oracle_Cva_P
#endif
