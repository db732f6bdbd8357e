/* Oracle build of the reference for the 3D plume workload: constants that the
 * workload sets differently from src/plume/parameters.h:862-1041 (air with
 * cp = 998 and R = 287, ash mass fraction 0.95 of the erupted material, vent
 * plane at z = 0).  Force-included after parameters.h; the reference header
 * is left untouched. */
#ifndef ORACLE_CFG_PLUME_H
#define ORACLE_CFG_PLUME_H
static const double oracle_Cva_P = 711.0;
static const double oracle_ng0_P = 0.05;
static const double oracle_Ll_P[3] = { -1.0e4, -1.0e4, 0.0 };
#define Cva_P oracle_Cva_P
#define ng0_P oracle_ng0_P
#define Ll_P oracle_Ll_P
#endif
