// lu.cuh -- device-pointer LU factorization, interchanges and solve.
#pragma once
#include <cuda_runtime.h>

namespace atlg {

// false forces the cooperative-grid panel (the cluster panel is the default
// where the panel fits one cluster's shared memory); results are identical.
void set_panel_cluster(bool on);
void set_panel_split(bool on);
// Rows at and below a panel above which the FP32 tensor-core factorization
// pairs side steps into rank-2*NB far updates (0: never, negative: default).
void set_defer_rows(int rows);
// true (default): in the FP32 tensor-core factorization a full-width cluster
// panel applies the previous step's update of its columns itself
void set_panel_fuse(bool on);
// CTAs of the cooperative-grid panel (0: a quarter of the SMs with look-ahead,
// more when the row slices would not fit shared memory).
void set_panel_grid(int ctas);
void set_panel_width_f64(int w);

// Column-major LU with partial pivoting of the M x N matrix A (device).
// ipiv (device, min(M,N) ints, 0-based, global row indices) and info
// (device int: 0, or the 1-based index of the first exactly-zero pivot).
void dev_dgetrf(int M, int N, double *A, int lda, int *ipiv, int *info, cudaStream_t st);
// dev_dgetrf with an explicit panel width (8..64, a multiple of 8)
void dev_dgetrf_pw(int M, int N, double *A, int lda, int *ipiv, int *info, int pw, cudaStream_t st);
void dev_sgetrf(int M, int N, float *A, int lda, int *ipiv, int *info, cudaStream_t st);
// FP32 LU whose trailing updates run on tcgen05 tensor cores in 3xTF32 (the
// mixed-precision solver's factor; pivots may differ from the FFMA sgetrf
// at near-ties).
void dev_sgetrf_tc(int M, int N, float *A, int lda, int *ipiv, int *info, cudaStream_t st);
// ATL_laswp semantics on device data; rows [0, nrows) may move (nrows > every pivot).
void dev_dlaswp(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows, cudaStream_t st);
void dev_slaswp(int N, float *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows, cudaStream_t st);
// ATL_getrs semantics (Order, Trans) on device data.
void dev_dgetrs(int order, int trans, int N, int NRHS, const double *A, int lda, const int *ipiv, double *B, int ldb,
                cudaStream_t st);
void dev_sgetrs(int order, int trans, int N, int NRHS, const float *A, int lda, const int *ipiv, float *B, int ldb,
                cudaStream_t st);
void dev_perm_from_ipiv(const int *ipiv, int n, int *perm, cudaStream_t st);
void dev_sgetrs_perm(int n, const float *LU, int lda, const int *perm, float *x, float *tmp, cudaStream_t st);
// the same solve through the chained TRSV (wsL, wsU from dev_strsv_chain_prepare)
void dev_sgetrs_perm_chain(int n, const float *LU, int lda, const int *perm, float *x, float *tmp, const float *wsL,
                           const float *wsU, cudaStream_t st);
unsigned lu_status_read_and_clear();

}  // namespace atlg
