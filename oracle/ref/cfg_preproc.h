/* Oracle build of the reference's preprocessor (src/preproc/preprocess.cc):
 * the original domain Ll_P / Lu_P of parameters.h is read at run time from
 * ORACLE_DOMAIN (six numbers: lo x y z, hi x y z) by ref/preproc_dump.cc, so
 * that one build covers every grid the tests compare.  Force-included
 * after parameters.h; the reference header is left untouched. */
#ifndef ORACLE_CFG_PREPROC_H
#define ORACLE_CFG_PREPROC_H
extern double oracle_pre_Ll[3];
extern double oracle_pre_Lu[3];
#define Ll_P oracle_pre_Ll
#define Lu_P oracle_pre_Lu
#endif
