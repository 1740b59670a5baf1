/* Level-3 routines called by the extracted Level-3 tester: the routines under
 * test (ATL_?gemm/trsm/trmm/syrk, bound to the GPU library by
 * tester_glue.c), ATL_?symm/syr2k (reference BLAS, not part of the GPU
 * library) and the recursive routines the tester trusts (ATL_?*_APR, bound
 * to the reference BLAS).  TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_TESTER_LEVEL3_H
#define REFSHIM_TESTER_LEVEL3_H
#include "atlas_misc.h"
#define DECL_L3(T, P, SUF) \
void ATL_##P##gemm##SUF(const enum ATLAS_TRANS, const enum ATLAS_TRANS, const int, const int, const int, \
   const T, const T*, const int, const T*, const int, const T, T*, const int); \
void ATL_##P##trsm##SUF(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##trmm##SUF(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##syrk##SUF(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const int, const int, const T, \
   const T*, const int, const T, T*, const int); \
void ATL_##P##syr2k##SUF(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const int, const int, const T, \
   const T*, const int, const T*, const int, const T, T*, const int); \
void ATL_##P##symm##SUF(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const int, const int, const T, \
   const T*, const int, const T*, const int, const T, T*, const int);
DECL_L3(double, d, )
DECL_L3(double, d, _APR)
#undef DECL_L3
#endif
