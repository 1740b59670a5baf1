/*
 * Link glue for the reference's own tester programs (xdlutst from
 * AtlasBase/Clint/atlas-tlp.base `lutst`, xdl3blastst from
 * AtlasBase/Antoine/atlbinblas.base `l3blastst`), extracted by
 * oracle/ref_build.sh and linked against the GPU library.  TEST
 * INFRASTRUCTURE ONLY.
 *
 * The testers call ATLAS-internal names.  In the reference they resolve to
 * the ATLAS build under test; here:
 *  - the routines under test (ATL_dgemm, ATL_dtrsm, ATL_dtrmm, ATL_dsyrk;
 *    clapack_dgetrf and cblas_dtrmm are called by their public names) go to
 *    the GPU library's cblas entry points, ColMajor, so each tester call is a
 *    host-pointer call through the drop-in C ABI;
 *  - the "trusted" side is the reference's C reference BLAS (ATL_dref*):
 *    gemm by the tester's own -DUSE_L3_REFERENCE switch, and the recursive
 *    ATL_*_APR routines the tester would otherwise trust (ATLAS's recursive
 *    Level 3 on its tuned kernels, which only the tuned build provides) are
 *    bound to the reference BLAS too;
 *  - ATL_dsymm / ATL_dsyr2k are not part of the GPU library: they are bound
 *    to the reference BLAS, so the tester's SYMM/SYR2K cases check nothing
 *    of this repository and are not run by the tests;
 *  - Level-1 helpers (asum, copy) are the reference BLAS; zero and gecopy are
 *    plain loops.
 * The ATLAS enum values are the cblas ones (AtlasNoTrans = CblasNoTrans = 111,
 * ...), so the enums pass through unchanged.
 */
#include <stddef.h>
#include "atlas_enum.h"

#define DECL_REF(T, P) \
void ATL_##P##refgemm(const enum ATLAS_TRANS, const enum ATLAS_TRANS, const int, const int, const int, \
   const T, const T*, const int, const T*, const int, const T, T*, const int); \
void ATL_##P##reftrsm(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##reftrmm(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##refsyrk(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const int, const int, const T, \
   const T*, const int, const T, T*, const int); \
void ATL_##P##refsyr2k(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const int, const int, const T, \
   const T*, const int, const T*, const int, const T, T*, const int); \
void ATL_##P##refsymm(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const int, const int, const T, \
   const T*, const int, const T*, const int, const T, T*, const int); \
T    ATL_##P##refasum(const int, const T*, const int); \
void ATL_##P##refcopy(const int, const T*, const int, T*, const int);

DECL_REF(double, d)
DECL_REF(float, s)

/* the library under test: its cblas entry points (include/atlas_gb300.h) */
void cblas_dgemm(const enum CBLAS_ORDER, const enum CBLAS_TRANSPOSE, const enum CBLAS_TRANSPOSE,
                 const int, const int, const int, const double, const double*, const int,
                 const double*, const int, const double, double*, const int);
void cblas_dtrsm(const enum CBLAS_ORDER, const enum CBLAS_SIDE, const enum CBLAS_UPLO,
                 const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG, const int, const int,
                 const double, const double*, const int, double*, const int);
void cblas_dtrmm(const enum CBLAS_ORDER, const enum CBLAS_SIDE, const enum CBLAS_UPLO,
                 const enum CBLAS_TRANSPOSE, const enum CBLAS_DIAG, const int, const int,
                 const double, const double*, const int, double*, const int);
void cblas_dsyrk(const enum CBLAS_ORDER, const enum CBLAS_UPLO, const enum CBLAS_TRANSPOSE,
                 const int, const int, const double, const double*, const int, const double,
                 double*, const int);

void ATL_dgemm(const enum ATLAS_TRANS TA, const enum ATLAS_TRANS TB, const int M, const int N,
               const int K, const double al, const double *A, const int lda, const double *B,
               const int ldb, const double be, double *C, const int ldc)
{
   cblas_dgemm(CblasColMajor, (enum CBLAS_TRANSPOSE)TA, (enum CBLAS_TRANSPOSE)TB, M, N, K, al, A, lda,
               B, ldb, be, C, ldc);
}
void ATL_dtrsm(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const enum ATLAS_TRANS TA,
               const enum ATLAS_DIAG D, const int M, const int N, const double al, const double *A,
               const int lda, double *B, const int ldb)
{
   cblas_dtrsm(CblasColMajor, (enum CBLAS_SIDE)S, (enum CBLAS_UPLO)U, (enum CBLAS_TRANSPOSE)TA,
               (enum CBLAS_DIAG)D, M, N, al, A, lda, B, ldb);
}
void ATL_dtrmm(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const enum ATLAS_TRANS TA,
               const enum ATLAS_DIAG D, const int M, const int N, const double al, const double *A,
               const int lda, double *B, const int ldb)
{
   cblas_dtrmm(CblasColMajor, (enum CBLAS_SIDE)S, (enum CBLAS_UPLO)U, (enum CBLAS_TRANSPOSE)TA,
               (enum CBLAS_DIAG)D, M, N, al, A, lda, B, ldb);
}
void ATL_dsyrk(const enum ATLAS_UPLO U, const enum ATLAS_TRANS T, const int N, const int K,
               const double al, const double *A, const int lda, const double be, double *C,
               const int ldc)
{
   cblas_dsyrk(CblasColMajor, (enum CBLAS_UPLO)U, (enum CBLAS_TRANSPOSE)T, N, K, al, A, lda, be, C, ldc);
}
/* not part of the GPU library: reference BLAS */
void ATL_dsymm(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const int M, const int N,
               const double al, const double *A, const int lda, const double *B, const int ldb,
               const double be, double *C, const int ldc)
{ ATL_drefsymm(S, U, M, N, al, A, lda, B, ldb, be, C, ldc); }
void ATL_dsyr2k(const enum ATLAS_UPLO U, const enum ATLAS_TRANS T, const int N, const int K,
                const double al, const double *A, const int lda, const double *B, const int ldb,
                const double be, double *C, const int ldc)
{ ATL_drefsyr2k(U, T, N, K, al, A, lda, B, ldb, be, C, ldc); }

/* the tester's trusted recursive routines, bound to the reference BLAS */
void ATL_dtrsm_APR(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const enum ATLAS_TRANS TA,
                   const enum ATLAS_DIAG D, const int M, const int N, const double al,
                   const double *A, const int lda, double *B, const int ldb)
{ ATL_dreftrsm(S, U, TA, D, M, N, al, A, lda, B, ldb); }
void ATL_dtrmm_APR(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const enum ATLAS_TRANS TA,
                   const enum ATLAS_DIAG D, const int M, const int N, const double al,
                   const double *A, const int lda, double *B, const int ldb)
{ ATL_dreftrmm(S, U, TA, D, M, N, al, A, lda, B, ldb); }
void ATL_dsyrk_APR(const enum ATLAS_UPLO U, const enum ATLAS_TRANS T, const int N, const int K,
                   const double al, const double *A, const int lda, const double be, double *C,
                   const int ldc)
{ ATL_drefsyrk(U, T, N, K, al, A, lda, be, C, ldc); }
void ATL_dsyr2k_APR(const enum ATLAS_UPLO U, const enum ATLAS_TRANS T, const int N, const int K,
                    const double al, const double *A, const int lda, const double *B,
                    const int ldb, const double be, double *C, const int ldc)
{ ATL_drefsyr2k(U, T, N, K, al, A, lda, B, ldb, be, C, ldc); }
void ATL_dsymm_APR(const enum ATLAS_SIDE S, const enum ATLAS_UPLO U, const int M, const int N,
                   const double al, const double *A, const int lda, const double *B,
                   const int ldb, const double be, double *C, const int ldc)
{ ATL_drefsymm(S, U, M, N, al, A, lda, B, ldb, be, C, ldc); }

/* Level-1 helpers of the test library */
double ATL_dasum(const int N, const double *X, const int incX) { return ATL_drefasum(N, X, incX); }
float  ATL_sasum(const int N, const float *X, const int incX) { return ATL_srefasum(N, X, incX); }
void ATL_dcopy(const int N, const double *X, const int incX, double *Y, const int incY)
{ ATL_drefcopy(N, X, incX, Y, incY); }
void ATL_scopy(const int N, const float *X, const int incX, float *Y, const int incY)
{ ATL_srefcopy(N, X, incX, Y, incY); }
void ATL_dzero(const int N, double *X, const int incX)
{
   int i;
   for (i = 0; i < N; i++) X[(size_t)i * incX] = 0.0;
}
void ATL_szero(const int N, float *X, const int incX)
{
   int i;
   for (i = 0; i < N; i++) X[(size_t)i * incX] = 0.0f;
}
void ATL_dgecopy(const int M, const int N, const double *A, const int lda, double *C, const int ldc)
{
   int i, j;
   for (j = 0; j < N; j++)
      for (i = 0; i < M; i++) C[i + (size_t)j * ldc] = A[i + (size_t)j * lda];
}
void ATL_sgecopy(const int M, const int N, const float *A, const int lda, float *C, const int ldc)
{
   int i, j;
   for (j = 0; j < N; j++)
      for (i = 0; i < M; i++) C[i + (size_t)j * ldc] = A[i + (size_t)j * lda];
}
