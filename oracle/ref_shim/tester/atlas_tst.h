/* The stand-in test-library header of the reference build, plus the
 * test-library routines only the tester programs call.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_TESTER_TST_H
#define REFSHIM_TESTER_TST_H
#include "../atlas_tst.h"
TYPE Mjoin(PATL,synrm)(const enum ATLAS_UPLO Uplo, const int N, const TYPE *A, const int lda);
TYPE Mjoin(PATL,trnrm1)(const enum ATLAS_UPLO Uplo, const enum ATLAS_DIAG Diag, const int N,
                        const TYPE *A, const int lda);
void *Mjoin(PATL,gecmpBV)(int verb, double ferr, int M, int N, const TYPE *A, int lda,
                          const TYPE *B, int ldb);
void *Mjoin(PATL,trcmpBV)(int verb, double tol, const enum ATLAS_UPLO Uplo, int M, int N,
                          const TYPE *A, int lda, const TYPE *B, int ldb);
void ATL_print2dBV(int M, int N, void *bv);
#endif
