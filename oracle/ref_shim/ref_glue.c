/*
 * Glue for the oracle's reference build: routes the generic BLAS calls of
 * the reference's extracted LU routines to the reference's own C reference
 * BLAS (ATL_?ref*, extracted from AtlasBase/Antoine/atlrefblas.base), and
 * exports a flat atlref_* API for the parity fixtures.  TEST INFRASTRUCTURE
 * ONLY: compiled by oracle/ref_build.sh into oracle/_ref/libatlref.so.
 */
#include <stdio.h>
#include <stdlib.h>
#include "atlas_enum.h"
#include "refshim_cblas.h"

#define DEF_REF(T, P) \
void ATL_##P##refgemm(const enum ATLAS_TRANS, const enum ATLAS_TRANS, const int, const int, \
   const int, const T, const T*, const int, const T*, const int, const T, T*, const int); \
void ATL_##P##reftrsm(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##refger(const int, const int, const T, const T*, const int, const T*, const int, \
   T*, const int); \
void ATL_##P##refscal(const int, const T, T*, const int); \
void ATL_##P##refswap(const int, T*, const int, T*, const int); \
int  ATL_i##P##refamax(const int, const T*, const int); \
int  ATL_##P##getrfC(const int, const int, T*, const int, int*); \
int  ATL_##P##getrfR(const int, const int, T*, const int, int*); \
void ATL_##P##laswp(const int, T*, const int, const int, const int, const int*, const int); \
void ATL_##P##getrs(const enum CBLAS_ORDER, const enum CBLAS_TRANSPOSE, const int, const int, \
   const T*, const int, const int*, T*, const int); \
void ATL_##P##gegen(const int, const int, T*, const int, const int); \
void ATL_##P##refsyrk(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const int, const int, const T, \
   const T*, const int, const T, T*, const int); \
void ATL_##P##reftrmm(const enum ATLAS_SIDE, const enum ATLAS_UPLO, const enum ATLAS_TRANS, \
   const enum ATLAS_DIAG, const int, const int, const T, const T*, const int, T*, const int); \
void ATL_##P##refgemv(const enum ATLAS_TRANS, const int, const int, const T, const T*, const int, \
   const T*, const int, const T, T*, const int); \
void ATL_##P##reftrsv(const enum ATLAS_UPLO, const enum ATLAS_TRANS, const enum ATLAS_DIAG, const int, \
   const T*, const int, T*, const int); \
int  ATL_##P##potrf(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const int, T*, const int); \
void ATL_##P##potrs(const enum CBLAS_ORDER, const enum CBLAS_UPLO, const int, const int, const T*, \
   const int, T*, const int); \
\
void refshim_##P##gemm(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, \
   int M, int N, int K, T al, const T *A, int lda, const T *B, int ldb, T be, T *C, int ldc) \
{ \
   if (o == CblasColMajor) \
      ATL_##P##refgemm((enum ATLAS_TRANS)ta, (enum ATLAS_TRANS)tb, M, N, K, al, A, lda, B, ldb, be, C, ldc); \
   else \
      ATL_##P##refgemm((enum ATLAS_TRANS)tb, (enum ATLAS_TRANS)ta, N, M, K, al, B, ldb, A, lda, be, C, ldc); \
} \
void refshim_##P##trsm(enum CBLAS_ORDER o, enum CBLAS_SIDE s, enum CBLAS_UPLO u, \
   enum CBLAS_TRANSPOSE t, enum CBLAS_DIAG d, int M, int N, T al, const T *A, int lda, T *B, int ldb) \
{ \
   if (o == CblasColMajor) \
      ATL_##P##reftrsm((enum ATLAS_SIDE)s, (enum ATLAS_UPLO)u, (enum ATLAS_TRANS)t, (enum ATLAS_DIAG)d, \
                       M, N, al, A, lda, B, ldb); \
   else \
      ATL_##P##reftrsm(s == CblasLeft ? AtlasRight : AtlasLeft, u == CblasUpper ? AtlasLower : AtlasUpper, \
                       (enum ATLAS_TRANS)t, (enum ATLAS_DIAG)d, N, M, al, A, lda, B, ldb); \
} \
void refshim_##P##trsv(enum CBLAS_ORDER o, enum CBLAS_UPLO u, enum CBLAS_TRANSPOSE t, \
   enum CBLAS_DIAG d, int N, const T *A, int lda, T *X, int incx) \
{ \
   if (incx != 1) abort(); \
   refshim_##P##trsm(o, CblasLeft, u, t, d, N, 1, (T)1, A, lda, X, N); \
} \
void refshim_##P##gemv(enum CBLAS_ORDER o, enum CBLAS_TRANSPOSE t, int M, int N, T al, \
   const T *A, int lda, const T *X, int incx, T be, T *Y, int incy) \
{ \
   if (incx != 1 || incy != 1) abort(); \
   if (t == CblasNoTrans) refshim_##P##gemm(o, CblasNoTrans, CblasNoTrans, M, 1, N, al, A, lda, X, N, be, Y, M); \
   else refshim_##P##gemm(o, CblasTrans, CblasNoTrans, N, 1, M, al, A, lda, X, M, be, Y, N); \
} \
int  refshim_i##P##amax(int N, const T *X, int incx) { return ATL_i##P##refamax(N, X, incx); } \
void refshim_##P##scal(int N, T al, T *X, int incx) { ATL_##P##refscal(N, al, X, incx); } \
void refshim_##P##swap(int N, T *X, int incx, T *Y, int incy) { ATL_##P##refswap(N, X, incx, Y, incy); } \
void ATL_##P##ger(const int M, const int N, const T al, const T *X, const int incx, const T *Y, \
   const int incy, T *A, const int lda) { ATL_##P##refger(M, N, al, X, incx, Y, incy, A, lda); } \
void ATL_##P##set(const int N, const T al, T *X, const int incx) \
{ int i; for (i = 0; i < N; i++) X[(size_t)i*incx] = al; } \
/* flat API */ \
int  atlref_##P##getrf(int order, int M, int N, T *A, int lda, int *ipiv) \
{ \
   if (M <= 0 || N <= 0) return 0; \
   return (order == CblasColMajor) ? ATL_##P##getrfC(M, N, A, lda, ipiv) \
                                   : ATL_##P##getrfR(M, N, A, lda, ipiv); \
} \
void atlref_##P##getrs(int order, int trans, int N, int NRHS, const T *A, int lda, \
   const int *ipiv, T *B, int ldb) \
{ ATL_##P##getrs((enum CBLAS_ORDER)order, (enum CBLAS_TRANSPOSE)trans, N, NRHS, A, lda, ipiv, B, ldb); } \
void atlref_##P##laswp(int N, T *A, int lda, int K1, int K2, const int *ipiv, int inci) \
{ ATL_##P##laswp(N, A, lda, K1, K2, ipiv, inci); } \
void atlref_##P##gegen(int M, int N, T *A, int lda, int seed) { ATL_##P##gegen(M, N, A, lda, seed); } \
void atlref_##P##gemm(int order, int ta, int tb, int M, int N, int K, T al, const T *A, int lda, \
   const T *B, int ldb, T be, T *C, int ldc) \
{ refshim_##P##gemm((enum CBLAS_ORDER)order, (enum CBLAS_TRANSPOSE)ta, (enum CBLAS_TRANSPOSE)tb, M, N, K, \
                    al, A, lda, B, ldb, be, C, ldc); } \
void atlref_##P##trsm(int order, int s, int u, int t, int d, int M, int N, T al, const T *A, int lda, \
   T *B, int ldb) \
{ refshim_##P##trsm((enum CBLAS_ORDER)order, (enum CBLAS_SIDE)s, (enum CBLAS_UPLO)u, \
                    (enum CBLAS_TRANSPOSE)t, (enum CBLAS_DIAG)d, M, N, al, A, lda, B, ldb); } \
int atlref_i##P##amax(int N, const T *X, int incx) { return ATL_i##P##refamax(N, X, incx); } \
long ATL_i##P##amax(long, const T*, long); \
int atlref_cblas_i##P##amax(int N, const T *X, int incx) \
{ return (N > 0 && incx > 0) ? (int)ATL_i##P##amax(N, X, incx) : 0; } \
/* cblas_syrk's RowMajor flip of Uplo and Trans (AtlasBase/Clint/cblas.base:440-448) */ \
void refshim_##P##syrk(enum CBLAS_ORDER o, enum CBLAS_UPLO u, enum CBLAS_TRANSPOSE t, int N, int K, \
   T al, const T *A, int lda, T be, T *C, int ldc) \
{ \
   if (o == CblasColMajor) \
      ATL_##P##refsyrk((enum ATLAS_UPLO)u, (enum ATLAS_TRANS)t, N, K, al, A, lda, be, C, ldc); \
   else \
      ATL_##P##refsyrk(u == CblasUpper ? AtlasLower : AtlasUpper, \
                       t == CblasNoTrans ? AtlasTrans : AtlasNoTrans, N, K, al, A, lda, be, C, ldc); \
} \
void atlref_##P##syrk(int order, int u, int t, int N, int K, T al, const T *A, int lda, T be, T *C, \
   int ldc) \
{ refshim_##P##syrk((enum CBLAS_ORDER)order, (enum CBLAS_UPLO)u, (enum CBLAS_TRANSPOSE)t, N, K, al, A, lda, \
                    be, C, ldc); } \
int  atlref_##P##potrf(int order, int u, int N, T *A, int lda) \
{ return ATL_##P##potrf((enum ATLAS_ORDER)order, (enum ATLAS_UPLO)u, N, A, lda); } \
/* cblas order mappings of trmm (as trsm), gemv and trsv: AtlasBase/Clint/cblas.base \
 * TRSM/TRMM section and AtlasBase/Clint/cblas-lvl2.base; negative increments start \
 * at the far end as the cblas wrappers arrange */ \
void atlref_##P##trmm(int order, int s, int u, int t, int d, int M, int N, T al, const T *A, int lda, \
   T *B, int ldb) \
{ \
   if (order == CblasColMajor) \
      ATL_##P##reftrmm((enum ATLAS_SIDE)s, (enum ATLAS_UPLO)u, (enum ATLAS_TRANS)t, (enum ATLAS_DIAG)d, \
                       M, N, al, A, lda, B, ldb); \
   else \
      ATL_##P##reftrmm(s == CblasLeft ? AtlasRight : AtlasLeft, u == CblasUpper ? AtlasLower : AtlasUpper, \
                       (enum ATLAS_TRANS)t, (enum ATLAS_DIAG)d, N, M, al, A, lda, B, ldb); \
} \
void atlref_##P##gemv(int order, int ta, int M, int N, T al, const T *A, int lda, const T *X, int incx, \
   T be, T *Y, int incy) \
{ \
   const int lx = (ta == CblasNoTrans) ? N : M, ly = (ta == CblasNoTrans) ? M : N; \
   if (incx < 0) X += (1 - lx) * incx; \
   if (incy < 0) Y += (1 - ly) * incy; \
   /* ATL_refgemv takes the dimensions of op(A): y has ly entries, x has lx */ \
   if (order == CblasColMajor) \
      ATL_##P##refgemv((enum ATLAS_TRANS)ta, ly, lx, al, A, lda, X, incx, be, Y, incy); \
   else \
      ATL_##P##refgemv(ta == CblasNoTrans ? AtlasTrans : AtlasNoTrans, ly, lx, al, A, lda, X, incx, be, Y, incy); \
} \
void atlref_##P##trsv(int order, int u, int t, int d, int N, const T *A, int lda, T *X, int incx) \
{ \
   if (incx < 0) X += (1 - N) * incx; \
   if (order == CblasColMajor) \
      ATL_##P##reftrsv((enum ATLAS_UPLO)u, (enum ATLAS_TRANS)t, (enum ATLAS_DIAG)d, N, A, lda, X, incx); \
   else \
      ATL_##P##reftrsv(u == CblasUpper ? AtlasLower : AtlasUpper, t == CblasNoTrans ? AtlasTrans : AtlasNoTrans, \
                       (enum ATLAS_DIAG)d, N, A, lda, X, incx); \
} \
/* stand-in for the tuned blocking factor: 64 columns */ \
int ATL_##P##laGetB(int M, int N, int K, int hint) { (void)M; (void)N; (void)K; (void)hint; return 64; } \
int  ATL_##P##trtri(const enum ATLAS_ORDER, const enum ATLAS_UPLO, const enum ATLAS_DIAG, const int, T*, \
   const int); \
int  ATL_##P##getri(const enum CBLAS_ORDER, const int, T*, const int, const int*, T*, int*); \
int  atlref_##P##trtri(int order, int u, int d, int N, T *A, int lda) \
{ return ATL_##P##trtri((enum ATLAS_ORDER)order, (enum ATLAS_UPLO)u, (enum ATLAS_DIAG)d, N, A, lda); } \
/* clapack_getri's workspace: laGetB * N entries (AtlasBase/Clint/atlas-clp.base:115-139) */ \
int  atlref_##P##getri(int order, int N, T *A, int lda, const int *ipiv) \
{ \
   int lwrk = ATL_##P##laGetB(N, 0, N, 0), ierr; \
   T *w; \
   lwrk = (lwrk <= N) ? lwrk * N : N * N; \
   w = (T*)malloc(sizeof(T) * (size_t)(lwrk > 0 ? lwrk : 1)); \
   ierr = ATL_##P##getri((enum CBLAS_ORDER)order, N, A, lda, ipiv, w, &lwrk); \
   free(w); \
   return ierr; \
} \
void atlref_##P##potrs(int order, int u, int N, int NRHS, const T *A, int lda, T *B, int ldb) \
{ ATL_##P##potrs((enum CBLAS_ORDER)order, (enum CBLAS_UPLO)u, N, NRHS, A, lda, B, ldb); }

DEF_REF(double, d)
DEF_REF(float, s)

void ATL_srand(int);
int ATL_rand(void);
double ATL_depsilon(void);
void atlref_srand(int seed) { ATL_srand(seed); }
int  atlref_rand(void) { return ATL_rand(); }
double atlref_depsilon(void) { return ATL_depsilon(); }
