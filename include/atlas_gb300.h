/*
 * atlas_gb300.h -- C ABI of the GB300 (sm_103a) implementation of ATLAS's
 * Level-3 / LU path.
 *
 * The cblas_* and clapack_* entry points have the reference's names,
 * prototypes, enum values, argument checks and return conventions, so a
 * program built against ATLAS's cblas.h / clapack.h links against
 * libatlas_gb300.so unchanged.  Each declaration cites the reference
 * interface it replaces (paths inside the ATLAS source tree).
 *
 * Conventions (as in the reference):
 *  - the caller owns every array; A and B are overwritten in place;
 *  - ipiv is caller allocated, min(M,N) ints, 0-based row indices;
 *  - an invalid argument prints "Parameter %d to routine %s was incorrect"
 *    on stderr and exits with status -1 (cblas_xerbla);
 *  - clapack_*getrf returns i > 0 when U(i-1,i-1) is exactly zero (the
 *    factorization is completed);
 *  - every host-pointer call is synchronous and must be made from one host
 *    thread at a time.
 * The atlg_*_dev variants take device pointers and a CUDA stream (NULL:
 * the library's stream), are asynchronous, and return 0 or -1 for a bad size.
 */
#ifndef ATLAS_GB300_H
#define ATLAS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* AtlasBase/Clint/atlas.base:19800-19806 (cblas.h enums) */
#ifndef CBLAS_ENUM_DEFINED_H
#define CBLAS_ENUM_DEFINED_H
enum CBLAS_ORDER {CblasRowMajor=101, CblasColMajor=102};
enum CBLAS_TRANSPOSE {CblasNoTrans=111, CblasTrans=112, CblasConjTrans=113, AtlasConj=114};
enum CBLAS_UPLO {CblasUpper=121, CblasLower=122};
enum CBLAS_DIAG {CblasNonUnit=131, CblasUnit=132};
enum CBLAS_SIDE {CblasLeft=141, CblasRight=142};
#endif
/* AtlasBase/Clint/atlas-clp.base:624-630 (clapack.h aliases) */
#ifndef ATLAS_ORDER
#define ATLAS_ORDER CBLAS_ORDER
#endif
#ifndef ATLAS_UPLO
#define ATLAS_UPLO CBLAS_UPLO
#endif
#ifndef ATLAS_DIAG
#define ATLAS_DIAG CBLAS_DIAG
#endif

/* ---- error reporting: AtlasBase/Clint/cblas.base:14 (cblas_errprn), :42 (cblas_xerbla) */
int  cblas_errprn(int ierr, int info, const char *form, ...);
void cblas_xerbla(int p, const char *rout, const char *form, ...);

/* ---- Level 3: AtlasBase/Clint/cblas.base:110-236 (GEMM template, d and s) */
void cblas_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_TRANSPOSE TB, const int M, const int N, const int K,
                 const double alpha, const double *A, const int lda, const double *B,
                 const int ldb, const double beta, double *C, const int ldc);
void cblas_sgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_TRANSPOSE TB, const int M, const int N, const int K,
                 const float alpha, const float *A, const int lda, const float *B,
                 const int ldb, const float beta, float *C, const int ldc);

/* ---- Level 3: AtlasBase/Clint/cblas.base:600-692 (TRSM template, d and s) */
void cblas_dtrsm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side,
                 const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int M, const int N, const double alpha,
                 const double *A, const int lda, double *B, const int ldb);
void cblas_strsm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side,
                 const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int M, const int N, const float alpha,
                 const float *A, const int lda, float *B, const int ldb);

/* ---- Level 3: AtlasBase/Clint/cblas.base:587-692 (TRMM, the TRSM template's
 *      twin: same checks and RowMajor mapping; d and s) */
void cblas_dtrmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side,
                 const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int M, const int N, const double alpha,
                 const double *A, const int lda, double *B, const int ldb);
void cblas_strmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side,
                 const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_DIAG Diag, const int M, const int N, const float alpha,
                 const float *A, const int lda, float *B, const int ldb);

/* ---- Level 1: AtlasBase/Clint/cblas-lvl1.base:408-420 (I?AMAX, CBLAS_INDEX = int):
 * 0-based index of the first element of largest magnitude, ATL_i?amax's
 * comparison sequence (AtlasBase/Clint/atlas-lvl1.base:1148-1340) including
 * its NaN behaviour; 0 when N < 2 or incX <= 0. */
int cblas_idamax(const int N, const double *X, const int incX);
int cblas_isamax(const int N, const float *X, const int incX);
/* ---- Level 2: AtlasBase/Clint/cblas-lvl2.base:21-93 (GEMV, d and s) */
void cblas_dgemv(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const int M,
                 const int N, const double alpha, const double *A, const int lda,
                 const double *X, const int incX, const double beta, double *Y,
                 const int incY);
void cblas_sgemv(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA, const int M,
                 const int N, const float alpha, const float *A, const int lda,
                 const float *X, const int incX, const float beta, float *Y, const int incY);
/* ---- Level 2: AtlasBase/Clint/cblas-lvl2.base:273-357 (TRSV, d and s) */
void cblas_dtrsv(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int N,
                 const double *A, const int lda, double *X, const int incX);
void cblas_strsv(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE TA, const enum CBLAS_DIAG Diag, const int N,
                 const float *A, const int lda, float *X, const int incX);

/* ---- Level 3: AtlasBase/Clint/cblas.base:339-450 (SYRK template, d and s) */
void cblas_dsyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE Trans, const int N, const int K,
                 const double alpha, const double *A, const int lda, const double beta,
                 double *C, const int ldc);
void cblas_ssyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo,
                 const enum CBLAS_TRANSPOSE Trans, const int N, const int K,
                 const float alpha, const float *A, const int lda, const float beta,
                 float *C, const int ldc);

/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:140 (clapack_getrf, d and s) */
int clapack_dgetrf(const enum CBLAS_ORDER Order, const int M, const int N, double *A,
                   const int lda, int *ipiv);
int clapack_sgetrf(const enum CBLAS_ORDER Order, const int M, const int N, float *A,
                   const int lda, int *ipiv);
/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:218 (clapack_getrs, d and s) */
int clapack_dgetrs(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE Trans, const int N,
                   const int NRHS, const double *A, const int lda, const int *ipiv, double *B,
                   const int ldb);
int clapack_sgetrs(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE Trans, const int N,
                   const int NRHS, const float *A, const int lda, const int *ipiv, float *B,
                   const int ldb);
/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:62 (clapack_gesv, d and s) */
int clapack_dgesv(const enum CBLAS_ORDER Order, const int N, const int NRHS, double *A,
                  const int lda, int *ipiv, double *B, const int ldb);
int clapack_sgesv(const enum CBLAS_ORDER Order, const int N, const int NRHS, float *A,
                  const int lda, int *ipiv, float *B, const int ldb);

/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:320-362 (clapack_potrf, d and s) */
int clapack_dpotrf(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N,
                   double *A, const int lda);
int clapack_spotrf(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N,
                   float *A, const int lda);
/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:363-410 (clapack_potrs, d and s) */
int clapack_dpotrs(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const int N,
                   const int NRHS, const double *A, const int lda, double *B, const int ldb);
int clapack_spotrs(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const int N,
                   const int NRHS, const float *A, const int lda, float *B, const int ldb);
/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:266-315 (clapack_posv, d and s) */
int clapack_dposv(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N,
                  const int NRHS, double *A, const int lda, double *B, const int ldb);
int clapack_sposv(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo, const int N,
                  const int NRHS, float *A, const int lda, float *B, const int ldb);

/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:411-452 (clapack_trtri, d and s) */
int clapack_dtrtri(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo,
                   const enum ATLAS_DIAG Diag, const int N, double *A, const int lda);
int clapack_strtri(const enum ATLAS_ORDER Order, const enum ATLAS_UPLO Uplo,
                   const enum ATLAS_DIAG Diag, const int N, float *A, const int lda);
/* ---- LAPACK: AtlasBase/Clint/atlas-clp.base:115-139 (clapack_getri, d and s) */
int clapack_dgetri(const enum CBLAS_ORDER Order, const int N, double *A, const int lda,
                   const int *ipiv);
int clapack_sgetri(const enum CBLAS_ORDER Order, const int N, float *A, const int lda,
                   const int *ipiv);

/* ---- new methods (no reference counterpart: ATLAS has neither a
 *      mixed-precision solver nor an adjoint).  Column-major. */
/* Split-precision DGEMM: cblas_dgemm's interface and checks, computed from
 * `nslices` (1..8) 7-bit integer slices of each operand (per-row / per-column
 * power-of-two scaling) multiplied exactly on tcgen05 tensor cores and
 * recombined in FP64 (the Ozaki scheme in integer form: Ozaki, Ogita, Oishi
 * and Rump 2012; Ootomo, Ozaki and Yokota 2024).  With 8 slices the error is
 * about 3e-16 of sum |a||b| per entry. */
void dgemm_split(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TA,
                 const enum CBLAS_TRANSPOSE TB, const int M, const int N, const int K,
                 const double alpha, const double *A, const int lda, const double *B,
                 const int ldb, const double beta, double *C, const int ldc, const int nslices);
/* FP32 LU + FP64 iterative refinement (LAPACK dsgesv stopping test), with an
 * FP64-LU fallback.  A is unchanged unless the fallback ran (status 1; A then
 * holds the FP64 factors); B is unchanged; X receives the solution; berr and
 * ferr have NRHS entries (normwise backward error, last-correction forward
 * error estimate); iters = refinement steps.  Returns 0 or i > 0 (zero pivot
 * in the FP64 factor). */
int dgesv_mixed(const int N, const int NRHS, double *A, const int lda, int *ipiv,
                const double *B, const int ldb, double *X, const int ldx, double *berr,
                double *ferr, int *iters, int *status);
/* Split-DGEMM form of dgesv: clapack_dgesv's ColMajor interface; the LU's
 * trailing updates (outer blocks of 1024 columns) run on the split-precision
 * DGEMM with 8 slices, FP64-accurate at any condition number; the solve is the
 * FP64 getrs.  Returns 0 or the first zero pivot (1-based). */
int dgesv_split(const int N, const int NRHS, double *A, const int lda, int *ipiv,
                double *B, const int ldb);
/* Adjoint of X = A^-1 B on the factors of clapack_dgetrf (ColMajor):
 * gB = A^-T gX (transposed solve, as ATL_getrs Trans: AtlasBase/Clint/
 * atlas-lp.base:1675-1682) and gA = -gB X^T (DGEMM). */
int dgesv_adjoint(const int n, const int nrhs, const double *LU, const int lda,
                  const int *ipiv, const double *X, const int ldx, const double *gX,
                  const int ldgx, double *gA, const int ldga, double *gB, const int ldgb);

/* ---- device-pointer variants (no reference counterpart: the reference has
 *      no device memory; these are the same operations on GPU-resident data,
 *      column-major, used by callers that keep matrices in HBM).
 *      Ordering: work runs on `stream` (NULL: the library's own stream,
 *      atlg_stream(), created non-blocking).  A non-blocking stream does not
 *      wait for the legacy default stream or any other stream, so data written
 *      on another stream must be ordered before the call by the caller (an
 *      event wait or a device synchronize). */
int      atlg_num_sms(void);
void    *atlg_stream(void);
unsigned atlg_status(void);   /* device wait-timeout flags since the last call, cleared */
/* benchmark support: kernels launched by the library so far; GEMM launch
 * timing with CUDA events (enable, then collect ms / flops / launches);
 * FP64 and FP32 FMA-pipe throughput probes in TFLOP/s */
unsigned long long atlg_launch_count(void);
void atlg_prof_enable(int on);
int  atlg_prof_collect(double *ms, double *flops, int *count);
void atlg_probe_peaks(double *fp64_tflops, double *fp32_tflops);
/* benchmark support (no reference counterpart): FP64 tensor-core throughput
 * in TFLOP/s of mma.sync with f64 operands, shapes m8n8k4, m16n8k4 and
 * m16n8k16 (any pointer may be NULL) */
void atlg_probe_fp64_mma(double *m8n8k4, double *m16n8k4, double *m16n8k16);
/* benchmark support (no reference counterpart): CUDA events around every LU
 * panel launch; collect returns the summed panel time, the summed gaps
 * between consecutive panels on the factorization's stream, and the count
 * (synchronizes) */
void atlg_prof_panels(int on);
int atlg_prof_panels_collect(double *panel_ms, double *gap_ms, int *count);
int atlg_dgemm_dev(int TA, int TB, int M, int N, int K, double alpha, const double *A, int lda,
                   const double *B, int ldb, double beta, double *C, int ldc, void *stream);
int atlg_dgemm_dev_opts(int TA, int TB, int M, int N, int K, double alpha, const double *A,
                        int lda, const double *B, int ldb, double beta, double *C, int ldc,
                        int allow_tma, void *stream);
int atlg_dgemm_split_dev(int TA, int TB, int M, int N, int K, double alpha, const double *A,
                         int lda, const double *B, int ldb, double beta, double *C, int ldc,
                         int nslices, void *stream);
/* C += alpha * A * B (FP32, column-major, no transposes) on tcgen05 tensor
 * cores with the 3xTF32 split (the mixed solver's factor update). */
int atlg_sgemm_tf32x3_dev(int M, int N, int K, float alpha, const float *A, int lda,
                          const float *B, int ldb, float *C, int ldc, void *stream);
int atlg_sgemm_dev(int TA, int TB, int M, int N, int K, float alpha, const float *A, int lda,
                   const float *B, int ldb, float beta, float *C, int ldc, void *stream);
int atlg_dtrsm_dev(int Side, int Uplo, int TA, int Diag, int M, int N, double alpha,
                   const double *A, int lda, double *B, int ldb, void *stream);
/* cblas_i?amax on device data (AtlasBase/Clint/cblas-lvl1.base:408): the
 * 0-based index is written to the device int *result.  Returns 0, -1 for
 * N < 0.  Calls whose work overlaps on the GPU (different streams) race on
 * the search's completion counter: serialise them. */
int atlg_idamax_dev(int N, const double *X, int incX, int *result, void *stream);
int atlg_isamax_dev(int N, const float *X, int incX, int *result, void *stream);
/* ATL_laswp semantics (AtlasBase/Clint/atlas-lp.base:1053); rows [0,nrows) may move */
int atlg_dlaswp_dev(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci,
                    int nrows, void *stream);
/* The same row interchanges as atlg_dlaswp_dev without any device allocation
 * (no reference counterpart): its scratch is a fixed 16 MiB array that every
 * GPU loading the library holds until exit.  For callers that cannot let a
 * library call cudaMalloc/cudaFree (their own pool owns device memory, or
 * they cannot take the device-wide synchronisation those calls imply).
 * Returns 0; -1 bad size (also K1 < 0 or K2 > nrows); -2 when 4*nrows
 * (rounded up to 256) + 8*nrows*N bytes exceed the 16 MiB scratch; -3 when
 * one of its own launches fails.  stream NULL is the library's own stream, as
 * for the other atlg_*_dev calls.  The first call on a device looks up the
 * scratch address (cudaGetSymbolAddress): make it before any stream capture.
 * Calls that overlap on the GPU share the scratch and race: serialise them. */
int atlg_dlaswp_noalloc(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci,
                        int nrows, void *stream);
/* LU panel implementation: 1 (default) factors panels that fit one thread-
 * block cluster's shared memory with the cluster kernel, 0 always uses the
 * cooperative-grid kernel; both give bit-identical factors and pivots */
void atlg_panel_cluster(int on);
/* LU panels too tall for one cluster at their full width (no reference
 * counterpart): 1 (default) factors them as two halves on the cluster (left
 * half, its interchanges, triangular solve and update on the right half,
 * right half), 0 on the cooperative-grid kernel; factors agree to rounding,
 * pivots are the same partial-pivoting choices */
void atlg_panel_split(int on);
/* the mixed solver's FP32 factor (no reference counterpart): while at least
 * `rows` rows lie at and below a step's panel, every other step's trailing
 * update of the columns beyond the next panel is deferred into the next
 * step's, which then updates them with rank 2 x 64 (one pass over the
 * trailing matrix for two panels); default 12288, 0 never defers, negative
 * restores the default.  Factors agree to rounding */
void atlg_lu_defer_rows(int rows);
/* the mixed solver's FP32 factor (no reference counterpart): 1 (default) a
 * full-width cluster panel applies the previous step's interchanges,
 * block-row solve and FP32 update of its own columns as it loads them, 0
 * leaves them to separate launches (3xTF32 update); factors agree to
 * rounding */
void atlg_panel_fuse(int on);
/* refinement solves of dgesv_mixed with one right-hand side (no reference
 * counterpart): 1 (default) the chained TRSV over 128-row blocks with block
 * inverses formed once per factorization, 0 the 64-row look-back TRSV; both
 * converge to the same FP64-accurate solution */
void atlg_refine_trsv(int chained);
/* CTAs of the cooperative-grid LU panel (0: the default, a quarter of the SMs
 * when the factorization overlaps its updates); results do not depend on it */
void atlg_panel_grid(int ctas);
/* panel width of the FP64 LU (8..64, rounded down to a multiple of 8; other
 * values: the default); pivots and factors agree with the default to
 * rounding */
void atlg_panel_width(int w);
/* column-major LU; info written to device memory */
int atlg_dgetrf_dev(int M, int N, double *A, int lda, int *ipiv, int *info, void *stream);
int atlg_sgetrf_dev(int M, int N, float *A, int lda, int *ipiv, int *info, void *stream);
/* the mixed solver's FP32 factorization (no reference counterpart): the same
 * LU with partial pivoting, trailing updates on the tensor cores in 3xTF32
 * (FP32-level accuracy); pivots follow the FP32 values it computes */
int atlg_sgetrf_tc_dev(int M, int N, float *A, int lda, int *ipiv, int *info, void *stream);
/* SA = A rounded to FP32 (to nearest even), the conversion the mixed solver
 * factors (LAPACK dlag2s; no ATLAS counterpart); device arrays; returns 1
 * when some |a| exceeds FLT_MAX (that entry becomes an infinity), 0
 * otherwise, -1 for a bad argument; synchronizes the stream */
int atlg_dlag2s_dev(int M, int N, const double *A, int lda, float *SA, int ldsa, void *stream);
/* the split-DGEMM LU on device data (0-based device pivots), nslices 1..8,
 * outer block nb (rounded down to a multiple of 256; 1024 in dgesv_split);
 * returns info; synchronizes once per outer block */
int atlg_dgetrf_split_dev(int N, double *A, int lda, int *ipiv, int nslices, int nb,
                          void *stream);
/* widest block column the split LU hands to the FP64 LU (rounded down to a
 * multiple of 256; 0: the default 512); narrower leaves move more of the
 * block column's own updates onto split products */
void atlg_split_lu_leaf(int nb);
int atlg_dgetrs_dev(int Order, int Trans, int N, int NRHS, const double *A, int lda,
                    const int *ipiv, double *B, int ldb, void *stream);
/* column-major SYRK / Cholesky on device data (Uplo, Trans, Order take the
 * CBLAS values); potrf returns info and synchronizes once per 64 columns */
int atlg_dsyrk_dev(int Uplo, int Trans, int N, int K, double alpha, const double *A, int lda,
                   double beta, double *C, int ldc, void *stream);
int atlg_dpotrf_dev(int Uplo, int N, double *A, int lda, void *stream);
int atlg_dpotrs_dev(int Order, int Uplo, int N, int NRHS, const double *A, int lda, double *B,
                    int ldb, void *stream);
/* column-major TRMM; GEMV with M, N the dimensions of A (a negative incX
 * counts from the far end; y contiguous); TRSV with incX = 1 */
int atlg_dtrmm_dev(int Side, int Uplo, int TA, int Diag, int M, int N, double alpha,
                   const double *A, int lda, double *B, int ldb, void *stream);
int atlg_dgemv_dev(int TA, int M, int N, double alpha, const double *A, int lda,
                   const double *X, int incX, double beta, double *Y, void *stream);
int atlg_dtrsv_dev(int Uplo, int TA, int Diag, int N, const double *A, int lda, double *X,
                   void *stream);
/* FP32 triangular solve A x = x (no transpose, incX = 1) for a triangle solved
 * many times, as in iterative refinement (no reference counterpart; the
 * single-solve form is cblas_strsv, AtlasBase/Clint/cblas-lvl2.base:273).
 * _prepare forms the 128 x 128 diagonal-block inverses and the couplings to
 * the block solved before each into ws (atlg_strsv_chain_ws(N) bytes,
 * 16-byte aligned); _dev then solves with one launch.  ws must be prepared
 * again after A changes.  Rounding differs from substitution.  Returns 0, -1
 * on a bad argument. */
size_t atlg_strsv_chain_ws(int N);
int atlg_strsv_chain_prepare_dev(int Uplo, int Diag, int N, const float *A, int lda, float *ws,
                                 void *stream);
int atlg_strsv_chain_dev(int Uplo, int N, const float *A, int lda, const float *ws, float *X,
                         void *stream);
/* trtri returns its info (synchronizes once); getri reads the 0-based
 * device pivots back to the host first */
int atlg_dtrtri_dev(int Order, int Uplo, int Diag, int N, double *A, int lda, void *stream);
int atlg_dgetri_dev(int N, double *A, int lda, const int *ipiv, void *stream);
/* berr, ferr (NRHS entries), iters and status are host pointers; synchronizes */
int atlg_dgesv_mixed_dev(int N, int NRHS, double *A, int lda, int *ipiv, const double *B,
                         int ldb, double *X, int ldx, double *berr, double *ferr, int *iters,
                         int *status, void *stream);
int atlg_dgesv_adjoint_dev(int n, int nrhs, const double *LU, int lda, const int *ipiv,
                           const double *X, int ldx, const double *gX, int ldgx, double *gA,
                           int ldga, double *gB, int ldgb, void *stream);

#ifdef __cplusplus
}
#endif
#endif
