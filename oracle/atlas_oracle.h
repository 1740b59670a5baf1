/*
 * atlas_oracle.h -- CPU restatement of ATLAS 3.11.42's Level-3 / LU path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300
 * implementation in math-atlas_gb300/: the parity tests, the smoke test and the
 * bench's CPU baseline call it.  The product library never links, loads or
 * calls it.
 *
 * Parity pin: the random generator, laswp, pivot order, Cholesky info and
 * the LU / Cholesky / GEMM / SYRK / TRSM / TRMM / GEMV / TRSV results of this
 * restatement are
 * checked against routines extracted from the reference's own basefiles (oracle/ref_build.sh builds them into
 * oracle/_ref/) and against the fixtures in tests/golden/ that were generated
 * from that build (tests/golden/make_golden.py).
 *
 * Conventions follow the reference C interfaces: column-major storage unless
 * an Order argument says otherwise, cblas enum values (RowMajor=101,
 * ColMajor=102, NoTrans=111, Trans=112, ConjTrans=113, Upper=121, Lower=122,
 * NonUnit=131, Unit=132, Left=141, Right=142; AtlasBase/Clint/atlas.base:19800),
 * 0-based ipiv.
 */
#ifndef ATLAS_ORACLE_H
#define ATLAS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* --- test-library generator (AtlasBase/Clint/atlas-tst.base:5353-5560, 2949) */
void   ora_srand(int seed);
int    ora_rand(void);
void   ora_dgegen(int M, int N, double *A, int lda, int seed);
void   ora_sgegen(int M, int N, float *A, int lda, int seed);
void   ora_dgefillgap(int M, int N, double *A, int lda);
int    ora_dgechkgap(int M, int N, const double *A, int lda);
double ora_depsilon(void);
float  ora_sepsilon(void);
double ora_dgenrm1(int M, int N, const double *A, int lda);
double ora_dgediffnrm1(int M, int N, const double *A, int lda,
                       const double *B, int ldb);
float  ora_sgenrm1(int M, int N, const float *A, int lda);
float  ora_sgediffnrm1(int M, int N, const float *A, int lda,
                       const float *B, int ldb);

/* --- Level 3 (column-major cores + cblas-order wrappers) --------------- */
void ora_dgemm(int TA, int TB, int M, int N, int K, double alpha,
               const double *A, int lda, const double *B, int ldb,
               double beta, double *C, int ldc);
void ora_sgemm(int TA, int TB, int M, int N, int K, float alpha,
               const float *A, int lda, const float *B, int ldb,
               float beta, float *C, int ldc);
void ora_dcblas_gemm(int Order, int TA, int TB, int M, int N, int K,
                     double alpha, const double *A, int lda, const double *B,
                     int ldb, double beta, double *C, int ldc);
void ora_scblas_gemm(int Order, int TA, int TB, int M, int N, int K,
                     float alpha, const float *A, int lda, const float *B,
                     int ldb, float beta, float *C, int ldc);
void ora_dtrsm(int Side, int Uplo, int TA, int Diag, int M, int N,
               double alpha, const double *A, int lda, double *B, int ldb);
void ora_strsm(int Side, int Uplo, int TA, int Diag, int M, int N,
               float alpha, const float *A, int lda, float *B, int ldb);
void ora_dcblas_trsm(int Order, int Side, int Uplo, int TA, int Diag, int M,
                     int N, double alpha, const double *A, int lda,
                     double *B, int ldb);
void ora_scblas_trsm(int Order, int Side, int Uplo, int TA, int Diag, int M,
                     int N, float alpha, const float *A, int lda,
                     float *B, int ldb);

/* --- Level 1 used by the factorization --------------------------------- */
int  ora_idamax(int N, const double *X, int incX);
int  ora_isamax(int N, const float *X, int incX);

/* --- LAPACK LU path (AtlasBase/Clint/atlas-lp.base:1053-1717, 5204) --- */
/* cblas_i?amax: ATL_i?amax's comparison sequence, NaNs included */
int ora_dcblas_iamax(int N, const double *X, int incX);
int ora_scblas_iamax(int N, const float *X, int incX);
void ora_dlaswp(int N, double *A, int lda, int K1, int K2, const int *ipiv,
                int inci);
void ora_slaswp(int N, float *A, int lda, int K1, int K2, const int *ipiv,
                int inci);
/* Tuning knobs that the reference takes from install-generated headers:
 * L1C_ELTS (getf2 cut-off, elements) and ATL_VWipgen_100LCMMN (split
 * rounding; 0 = not defined).  Defaults: 4096 and 0. */
void ora_set_lu_params(long l1c_elts, int lcmmn);
int  ora_dgetrf(int Order, int M, int N, double *A, int lda, int *ipiv);
int  ora_sgetrf(int Order, int M, int N, float *A, int lda, int *ipiv);
void ora_dgetrs(int Order, int Trans, int N, int NRHS, const double *A,
                int lda, const int *ipiv, double *B, int ldb);
void ora_sgetrs(int Order, int Trans, int N, int NRHS, const float *A,
                int lda, const int *ipiv, float *B, int ldb);
int  ora_dgesv(int Order, int N, int NRHS, double *A, int lda, int *ipiv,
               double *B, int ldb);

/* --- SYRK and Cholesky ---------------------------------------------------- */
/* reference-BLAS SYRK (AtlasBase/Antoine/atlrefblas.base:7573-8100) */
void ora_dsyrk(int Uplo, int Trans, int N, int K, double alpha, const double *A,
               int lda, double beta, double *C, int ldc);
void ora_ssyrk(int Uplo, int Trans, int N, int K, float alpha, const float *A,
               int lda, float beta, float *C, int ldc);
/* cblas_syrk order handling (AtlasBase/Clint/cblas.base:440-448) */
void ora_dcblas_syrk(int Order, int Uplo, int Trans, int N, int K, double alpha,
                     const double *A, int lda, double beta, double *C, int ldc);
void ora_scblas_syrk(int Order, int Uplo, int Trans, int N, int K, float alpha,
                     const float *A, int lda, float beta, float *C, int ldc);
/* ATL_potrf with the recursive ATL_potrfU / ATL_potrfL
 * (AtlasBase/Clint/atlas-lp.base:332-968); returns 0 or the 1-based index of
 * the first non-positive pivot. */
int  ora_dpotrf(int Order, int Uplo, int N, double *A, int lda);
int  ora_spotrf(int Order, int Uplo, int N, float *A, int lda);
/* ATL_potrs (AtlasBase/Clint/atlas-lp.base:969-1052) */
void ora_dpotrs(int Order, int Uplo, int N, int NRHS, const double *A, int lda,
                double *B, int ldb);
void ora_spotrs(int Order, int Uplo, int N, int NRHS, const float *A, int lda,
                float *B, int ldb);
/* clapack_posv (AtlasBase/Clint/atlas-clp.base:266-315) */
int  ora_dposv(int Order, int Uplo, int N, int NRHS, double *A, int lda,
               double *B, int ldb);
int  ora_sposv(int Order, int Uplo, int N, int NRHS, float *A, int lda,
               float *B, int ldb);

/* --- TRMM, GEMV, TRSV --------------------------------------------------- */
/* reference-BLAS trmm (AtlasBase/Antoine/atlrefblas.base:8406) and the cblas
 * order mapping shared with TRSM (AtlasBase/Clint/cblas.base:587-692) */
void ora_dtrmm(int Side, int Uplo, int TA, int Diag, int M, int N, double alpha,
               const double *A, int lda, double *B, int ldb);
void ora_strmm(int Side, int Uplo, int TA, int Diag, int M, int N, float alpha,
               const float *A, int lda, float *B, int ldb);
void ora_dcblas_trmm(int Order, int Side, int Uplo, int TA, int Diag, int M,
                     int N, double alpha, const double *A, int lda, double *B,
                     int ldb);
void ora_scblas_trmm(int Order, int Side, int Uplo, int TA, int Diag, int M,
                     int N, float alpha, const float *A, int lda, float *B,
                     int ldb);
/* cblas_gemv / cblas_trsv (AtlasBase/Clint/cblas-lvl2.base:21-93, 273-357),
 * negative increments counted from the far end */
void ora_dcblas_gemv(int Order, int TA, int M, int N, double alpha,
                     const double *A, int lda, const double *X, int incX,
                     double beta, double *Y, int incY);
void ora_scblas_gemv(int Order, int TA, int M, int N, float alpha,
                     const float *A, int lda, const float *X, int incX,
                     float beta, float *Y, int incY);
void ora_dcblas_trsv(int Order, int Uplo, int TA, int Diag, int N,
                     const double *A, int lda, double *X, int incX);
void ora_scblas_trsv(int Order, int Uplo, int TA, int Diag, int N,
                     const float *A, int lda, float *X, int incX);

/* --- inverses -------------------------------------------------------------- */
/* ATL_trtri (AtlasBase/Clint/atlas-lp.base:1718-2380): 0, or the 1-based index
 * of the first exact zero on a non-unit diagonal (A untouched then). */
int  ora_dtrtri(int Order, int Uplo, int Diag, int N, double *A, int lda);
int  ora_strtri(int Order, int Uplo, int Diag, int N, float *A, int lda);
/* clapack_getri / ATL_getriC (AtlasBase/Clint/atlas-clp.base:115-139,
 * atlas-lp.base:104-199) on the factors and 0-based pivots of getrf */
int  ora_dgetri(int Order, int N, double *A, int lda, const int *ipiv);
int  ora_sgetri(int Order, int N, float *A, int lda, const int *ipiv);

/* --- tester residuals ---------------------------------------------------- */
/* xdlutst residual (AtlasBase/Clint/atlas-tlp.base:1992-2058) for a
 * column-major factorization held in LU/ipiv of the matrix gegen(M,N,lda,seed). */
double ora_dlu_resid(int M, int N, const double *LU, int lda, const int *ipiv,
                     int seed);
float  ora_slu_resid(int M, int N, const float *LU, int lda, const int *ipiv,
                     int seed);
/* xdl3blastst gemm residual (AtlasBase/Antoine/atlbinblas.base:11910-11930). */
double ora_dgemm_resid(int TA, int TB, int M, int N, int K, double alpha,
                       const double *A, int lda, const double *B, int ldb,
                       double beta, const double *Cin, const double *Ctest,
                       const double *Ctrust, int ldc);
/* xdslvtst residual ||X-Xc||_inf / (N eps ||A||_1 ||Xc||_inf)
 * (AtlasBase/Clint/atlas-tlp.base:574-600). */
double ora_dslv_resid(int N, int NRHS, const double *A, int lda,
                      const double *X, int ldx, const double *Xc, int ldxc);

/* --- new methods: double-double oracle and backward error --------------- */
/* C(i,j) of op(A)*op(B) in double-double (Dekker/Knuth error-free
 * transformations), for nsamp sampled (i,j); returns hi and lo parts. */
void ora_dgemm_dd_samples(int TA, int TB, int M, int N, int K,
                          const double *A, int lda, const double *B, int ldb,
                          int nsamp, const int *ii, const int *jj,
                          double *hi, double *lo);
/* Normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
 * with the residual accumulated in double-double. */
double ora_dbackward_error(int N, const double *A, int lda, const double *x,
                           const double *b);

/* Threads the oracle uses (OpenMP); returns the count in effect. */
int ora_set_threads(int n);
int ora_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
