/* Test-library interface used by the extracted generator routines (same macro
 * names as the reference's test header, written for this build).
 * TEST INFRASTRUCTURE ONLY. */
#ifndef REFSHIM_TST_H
#define REFSHIM_TST_H
#include "atlas_misc.h"
void ATL_srand(int iseed);
int  ATL_rand(void);
#define dumb_seed(iseed_) ATL_srand(iseed_)
#define dumb_rand() (0.5 - ((double)ATL_rand())/(2147483648.0))
void ATL_dset(const int, const double, double*, const int);
void ATL_sset(const int, const float, float*, const int);
/* test-library routines the extracted tester programs call */
double time00(void);
double ATL_flushcache(long long size);
TYPE Mjoin(PATL,epsilon)(void);
void Mjoin(PATL,gegen)(const int M, const int N, TYPE *A, const int lda, const int seed);
TYPE Mjoin(PATL,genrm1)(const int M, const int N, const TYPE *A, const int lda);
TYPE Mjoin(PATL,gediffnrm1)(const int M, const int N, const TYPE *A, const int lda, const TYPE *B,
                            const int ldb);
#endif
