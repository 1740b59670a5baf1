// lu.cu -- LU factorization with partial pivoting (getrf), row interchanges
// (laswp) and the solve with the factors (getrs), FP64 and FP32, on GB300.
//
// Reference path replaced: ATL_getrfC / ATL_getrfR, the recursive LU
// (AtlasBase/Clint/atlas-lp.base:1210-1617) with its base cases LU2 / getf2
// (:1301-1391, :5204-5360), ATL_laswp (:1053-1166) and ATL_getrs (:1631-1717);
// the pivot search is cblas_iamax (AtlasBase/Clint/atlas-lvl1.base:1148).
//
// GB300 design: right-looking blocked LU, panel width NB=64.  Per panel:
//  1. panel_kernel: one cooperative grid (one CTA per SM, bounded grid
//     barrier) factors the (M-k) x NB panel column by column.  Each CTA owns
//     a contiguous slice of rows.  For column j every CTA finds its local
//     first-max |a|, stages that candidate row and (owner of row j) row j in
//     global scratch, one grid barrier, then every CTA picks the same global
//     winner (largest |a|, lowest row on ties -- the iamax rule), swaps the
//     two rows and eliminates in its own rows.  One barrier per column.  The
//     pivot is applied as a reciprocal when |pivot| > SAFMIN and by division
//     otherwise, as the reference does.  CTA 0 also reduces the panel's NB
//     interchanges to a row permutation (at most 2*NB rows move).
//  2. apply_perm: the permutation is applied to every column outside the
//     panel as a gather (all source rows read, then all destination rows
//     written) instead of NB dependent swaps -- the laswp of the reference.
//  3. U12 = L11^-1 A12 (warp-per-column unit-lower solve, trsm.cu).
//  4. A22 -= L21 * U12 on the DFMA GEMM (gemm.cu).
// Pivots are bit-identical to the reference whenever no two candidates of a
// pivot search are within rounding of each other; the factors agree to
// rounding (different but equally stable summation order).
#include <float.h>
#include <limits.h>

#include <cooperative_groups.h>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "context.cuh"
#include "gemm.cuh"
#include "lu.cuh"
#include "tf32.cuh"
#include "trsm.cuh"

namespace cg = cooperative_groups;

namespace atlg {

__device__ unsigned g_lu_status;

constexpr int NB = 64;          // panel width
constexpr int PT = 256;         // threads per panel CTA
constexpr size_t kPanelSmemMax = 192 * 1024;   // shared-memory panel slice limit

template <typename T> struct Lim;
template <> struct Lim<double> { __device__ static double safmin() { return DBL_MIN; } };
template <> struct Lim<float>  { __device__ static float safmin() { return FLT_MIN; } };

// Pivot search on integer keys.  For x not NaN, the bit pattern of |x| read
// as a signed integer orders exactly as |x| does; NaN maps to -1, below every
// candidate, so it never wins (as `|x| > best` never holds for NaN).  GB300
// runs FP64 compares on its narrow FP64 pipe, so the reductions of the
// search compare keys on the integer pipe instead; the winner is the same.
template <typename T> struct PivKey;
template <> struct PivKey<double> {
  using K = long long;
  __device__ static K key(double x) {
    const K b = __double_as_longlong(x) & 0x7fffffffffffffffLL;
    return b > 0x7ff0000000000000LL ? K(-1) : b;
  }
  __device__ static double as_t(K k) { return __longlong_as_double(k); }
  __device__ static K from_t(double v) { return __double_as_longlong(v); }
};
template <> struct PivKey<float> {
  using K = int;
  __device__ static K key(float x) {
    const K b = __float_as_int(x) & 0x7fffffff;
    return b > 0x7f800000 ? K(-1) : b;
  }
  __device__ static float as_t(K k) { return __int_as_float(k); }
  __device__ static K from_t(float v) { return __float_as_int(v); }
};

template <typename K>
struct BlockArgmax {
  K v[PT / 32];
  int i[PT / 32];
};

// Warp-wide first-max on (key, idx): the larger key wins, the lower idx
// among equal keys; every lane ends with the result.  Hardware warp
// reductions (redux.sync) instead of a five-level shuffle tree; a 64-bit key
// is compared as (signed high word, unsigned low word).
__device__ __forceinline__ void warp_argmax(int &key, int &idx) {
  const int mk = __reduce_max_sync(0xffffffffu, key);
  idx = __reduce_min_sync(0xffffffffu, key == mk ? idx : 0x7fffffff);
  key = mk;
}
__device__ __forceinline__ void warp_argmax(long long &key, int &idx) {
  const int hi = (int)(key >> 32);
  const unsigned lo = (unsigned)(key & 0xffffffffLL);
  const int mh = __reduce_max_sync(0xffffffffu, hi);
  const unsigned ml = __reduce_max_sync(0xffffffffu, hi == mh ? lo : 0u);
  idx = __reduce_min_sync(0xffffffffu, (hi == mh && lo == ml) ? idx : 0x7fffffff);
  key = (long long)(((unsigned long long)(unsigned)mh << 32) | ml);
}

// first-max reduction over the block: (key, idx) with the larger key
// winning, lower idx winning ties; key < 0 marks "no candidate".  Warp 0
// ends with the result.
template <typename K>
__device__ void block_argmax(K &val, int &idx, BlockArgmax<K> &sh) {
  warp_argmax(val, idx);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sh.v[w] = val; sh.i[w] = idx; }
  __syncthreads();
  if (w == 0) {
    val = lane < PT / 32 ? sh.v[lane] : K(-1);
    idx = lane < PT / 32 ? sh.i[lane] : 0x7fffffff;
    warp_argmax(val, idx);
  }
  __syncthreads();
}

// The rows a panel CTA owns, either in global memory (rows of the panel,
// leading dimension lda) or copied to a column-major shared-memory tile of
// R rows for the whole factorization of the panel.
template <typename T, bool SM>
struct PanelRows {
  T *g;
  int lda;
  T *s;
  int R, r0;
  __device__ __forceinline__ T &at(int i, int c) const {
    if (SM) return s[(i - r0) + c * R];
    return g[i + (size_t)c * lda];
  }
};

// Candidate records in global scratch, double buffered by column parity.
// Other CTAs write them between grid barriers, so every read after a barrier
// goes to L2 (__ldcg): an L1 line from the same buffer two columns earlier
// would otherwise be stale.
// rec[(par*G + b)*RS + c] holds CTA b's candidate row (c < NB), then the
// pivot key of its |a| (c = NB, its bits stored in a T; negative: no
// candidate) and its row index (c = NB+1, exact in T for any matrix this
// library can hold).  One record per CTA, so a
// reader gets value, index and row of every candidate from one place.
template <typename T> __host__ __device__ constexpr int rec_stride() { return sizeof(T) == 8 ? NB + 2 : NB + 4; }

// Local candidate for column j among own rows [max(r0,j), r1); stage it.
template <typename T, bool SM>
__device__ void stage_candidate(const PanelRows<T, SM> &A, int j, int jb, int r0, int r1, int par, int G, T *rec,
                                T *jrow, BlockArgmax<typename PivKey<T>::K> &sh, int *s_idx) {
  using K = typename PivKey<T>::K;
  constexpr int RS = rec_stride<T>();
  K best = K(-1);
  int bi = 0x7fffffff;
  const int lo = r0 > j ? r0 : j;
  for (int i = lo + threadIdx.x; i < r1; i += PT) {      // ascending rows per thread
    const K a = PivKey<T>::key(A.at(i, j));
    if (a > best) { best = a; bi = i; }
  }
  block_argmax(best, bi, sh);
  T *r = rec + ((size_t)par * G + blockIdx.x) * RS;
  if (threadIdx.x == 0) {
    r[NB] = PivKey<T>::as_t(best);
    r[NB + 1] = best >= K(0) ? (T)bi : T(-1);
    *s_idx = best >= K(0) ? bi : -1;
  }
  __syncthreads();
  const int ci = *s_idx;
  if (ci >= 0)
    for (int c = threadIdx.x; c < jb; c += PT) r[c] = A.at(ci, c);
  if (j >= r0 && j < r1)
    for (int c = threadIdx.x; c < jb; c += PT) jrow[par * NB + c] = A.at(j, c);
}

// One warp: the panel's jb interchanges (row j <-> row piv_local[j], panel-
// relative, in order) as one permutation of at most 2*NB rows, written as
// perm = {count, dst[2NB], src[2NB]} for apply_perm_kernel.
__device__ void reduce_interchanges(const int *piv_local, int jb, int *perm) {
  __shared__ int rows[2 * NB], content[2 * NB];
  __shared__ int cnt;
  const int lane = threadIdx.x & 31;
  for (int t = lane; t < jb; t += 32) { rows[t] = t; content[t] = t; }
  if (lane == 0) cnt = jb;
  __syncwarp();
  for (int j = 0; j < jb; ++j) {
    const int p = piv_local[j];
    int slot;
    if (p < jb) {
      slot = p;
    } else {
      const int n = cnt;
      int found = -1;
      for (int base = jb; base < n; base += 32) {
        const int t = base + lane;
        const unsigned m = __ballot_sync(0xffffffffu, t < n && rows[t] == p);
        if (m) { found = base + __ffs(m) - 1; break; }
      }
      if (found < 0) {
        found = n;
        if (lane == 0) { rows[n] = p; content[n] = p; cnt = n + 1; }
      }
      slot = found;
    }
    __syncwarp();
    if (lane == 0 && slot != j) {
      const int t = content[j];
      content[j] = content[slot];
      content[slot] = t;
    }
    __syncwarp();
  }
  const int n = cnt;
  for (int t = lane; t < n; t += 32) {
    perm[1 + t] = rows[t];
    perm[1 + 2 * NB + t] = content[t];
  }
  if (lane == 0) perm[0] = n;
}

template <typename T, bool SM>
__global__ void __launch_bounds__(PT)
    panel_kernel(T *Ag, int lda, int M, int jb, int koff, int *ipiv, int *info, T *rec, T *jrow, unsigned *bar,
                 int *perm) {
  using K = typename PivKey<T>::K;
  extern __shared__ __align__(16) unsigned char panel_dyn[];
  __shared__ BlockArgmax<K> sh;
  __shared__ T P[NB], J[NB];
  __shared__ int s_idx, s_p, s_zero, s_use_rcp;
  __shared__ T s_rcp;
  __shared__ int piv_local[NB];
  constexpr int LB = SM ? 1 : 2048;
  __shared__ T lbuf[LB];

  const int G = gridDim.x;
  const int chunk = (M + G - 1) / G;
  const int r0 = blockIdx.x * chunk;
  const int r1 = (r0 + chunk < M) ? r0 + chunk : M;
  const bool big = !SM && (r1 - r0) > 2048;
  PanelRows<T, SM> A;
  A.g = Ag;
  A.lda = lda;
  A.s = reinterpret_cast<T *>(panel_dyn);
  A.R = chunk;
  A.r0 = r0;
  if (SM) {
    const int nr = r1 - r0;
    if (nr > 0)
      for (int e = threadIdx.x; e < nr * jb; e += PT) {
        const int i = e % nr, c = e / nr;
        A.s[i + c * chunk] = Ag[(r0 + i) + (size_t)c * lda];
      }
    __syncthreads();
  }

  constexpr int RS = rec_stride<T>();
  // every CTA copies all G candidate records when they fit this buffer
  constexpr int GATHER = (24 * 1024) / (RS * (int)sizeof(T));
  __shared__ __align__(16) T gath[GATHER * RS];
  const bool gather_all = G <= GATHER;

  stage_candidate(A, 0, jb, r0, r1, 0, G, rec, jrow, sh, &s_idx);
  for (int j = 0; j < jb; ++j) {
    const int par = j & 1;
    if (!grid_barrier_count(&bar[0], (unsigned)(koff + j + 1) * (unsigned)G, &g_lu_status)) return;
    const T *rp = rec + (size_t)par * G * RS;
    // ---- global winner (identical in every CTA) ----
    if (gather_all) {
      // one round trip: every record (value, index, row) and row j
      for (int e = threadIdx.x; e < G * RS; e += PT) gath[e] = __ldcg(rp + e);
      for (int c = threadIdx.x; c < jb; c += PT) J[c] = __ldcg(jrow + par * NB + c);
      __syncthreads();
    }
    if (threadIdx.x < 32) {
      K best = K(-1);
      int bb = 0x7fffffff;
      for (int b = threadIdx.x; b < G; b += 32) {
        const K v = PivKey<T>::from_t(gather_all ? gath[b * RS + NB] : __ldcg(rp + (size_t)b * RS + NB));
        if (v > best) { best = v; bb = b; }
      }
      warp_argmax(best, bb);
      if (threadIdx.x == 0) {
        int p = -1;
        if (bb < G && best > K(0)) p = (int)(gather_all ? gath[bb * RS + NB + 1] : __ldcg(rp + (size_t)bb * RS + NB + 1));
        s_zero = (p < 0);
        s_p = (p < 0) ? j : p;
        s_idx = bb;
      }
    }
    __syncthreads();
    const int p = s_p;
    const bool zero = s_zero != 0;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      ipiv[j] = koff + p;
      piv_local[j] = p;
      if (zero && *info == 0) *info = koff + j + 1;
    }
    if (!zero) {
      const int wb = s_idx;
      for (int c = threadIdx.x; c < jb; c += PT) {
        if (gather_all) {
          P[c] = gath[wb * RS + c];
        } else {
          P[c] = __ldcg(rp + (size_t)wb * RS + c);
          J[c] = __ldcg(jrow + par * NB + c);
        }
        if (c == j) {   // once per CTA: FP64 division (and compare) is costly
          const T pj = P[c];
          s_rcp = T(1) / pj;
          s_use_rcp = (pj < T(0) ? -pj : pj) > Lim<T>::safmin();
        }
      }
      __syncthreads();
      const T pv = P[j];
      const bool use_rcp = s_use_rcp != 0;
      const T rcp = s_rcp;
      // pass 1: multipliers (column j) and the two swapped rows' L parts
      const int lo = r0 > j ? r0 : j;
      for (int i = lo + threadIdx.x; i < r1; i += PT) {
        if (i == j) {
          if (!SM && !big) lbuf[i - r0] = T(0);
          continue;
        }
        const T src = (i == p) ? J[j] : A.at(i, j);
        const T l = use_rcp ? src * rcp : src / pv;
        A.at(i, j) = l;
        if (!SM && !big) lbuf[i - r0] = l;
      }
      // row j <- pivot row (all columns); row p <- old row j in the L part
      if (j >= r0 && j < r1)
        for (int c = threadIdx.x; c < jb; c += PT) A.at(j, c) = P[c];
      if (p != j && p >= r0 && p < r1)
        for (int c = threadIdx.x; c < j; c += PT) A.at(p, c) = J[c];
      __syncthreads();
      // pass 2: rank-1 update of columns j+1..jb-1 in own rows i > j; a
      // thread per row walks the columns (consecutive threads touch
      // consecutive rows of a column, no index division)
      for (int i = lo + threadIdx.x; i < r1; i += PT) {
        if (i == j) continue;
        const T l = (SM || big) ? A.at(i, j) : lbuf[i - r0];
        if (i == p) {
          for (int c = j + 1; c < jb; ++c) A.at(i, c) = J[c] - l * P[c];
        } else {
#pragma unroll 4
          for (int c = j + 1; c < jb; ++c) A.at(i, c) -= l * P[c];
        }
      }
      __syncthreads();
    }
    if (j + 1 < jb) stage_candidate(A, j + 1, jb, r0, r1, (j + 1) & 1, G, rec, jrow, sh, &s_idx);
  }
  if (SM) {
    __syncthreads();
    const int nr = r1 - r0;
    if (nr > 0)
      for (int e = threadIdx.x; e < nr * jb; e += PT) {
        const int i = e % nr, c = e / nr;
        Ag[(r0 + i) + (size_t)c * lda] = A.s[i + c * chunk];
      }
  }
  // ---- CTA 0: reduce the NB interchanges to a permutation of rows ----
  if (blockIdx.x == 0 && threadIdx.x < 32) reduce_interchanges(piv_local, jb, perm);
}

// ---------------------------------------------------------------------------
// Cluster panel: the same factorization as panel_kernel (identical arithmetic
// per element, so identical pivots and factors) for panels whose rows fit the
// shared memory of one thread-block cluster (up to 16 CTAs on one GPC).
// Per column j every CTA sends to every CTA of the cluster (itself
// included) its first-max candidate -- key of |a|, row index and the whole
// row -- and the owner of row j sends row j, all as 16-byte st.async stores
// that count down the receiver's mbarrier for that column.  A CTA waits only
// on its own mbarrier (no cluster barrier, no remote load on the critical
// path), picks the winner from its local copies (every warp the same), takes
// the winner's row and row j from its own shared memory, eliminates in its
// rows and reduces its first-max of column j+1, which it sends on before the
// rest of its rank-1 update.  The receive areas and mbarriers are double
// buffered by column parity: a CTA sends column j+2 only after it has
// received column j+1 from every CTA, which each sent only after copying
// what it needed of column j.  Every message of the fixed protocol is sent,
// so every wait ends; the waits are bounded all the same.
constexpr int kClusterMax = 16;

// One column's receive area: every CTA's candidate record (the row's
// 16-byte vectors, then {key low, key high, row index, 0}) and row j.
template <typename T>
struct ClusterRecv {
  uint4 row[kClusterMax][NB * sizeof(T) / 16 + 1];
  uint4 jrow[NB * sizeof(T) / 16];
};

template <typename T> struct Vec16;
template <> struct Vec16<float> { using type = float4; };
template <> struct Vec16<double> { using type = double2; };

// (larger key, then lower source) wins; every lane ends with the winner.
// Lane s holds source s (b = s), so the winner's row comes from lane b.
template <typename K>
__device__ __forceinline__ void warp_winner(K &v, int &b, int &idx) {
  warp_argmax(v, b);
  idx = __shfl_sync(0xffffffffu, idx, b & 31);
}

constexpr int CT = 512;         // threads per cluster-panel CTA (16 warps)

// Row stride of the cluster panel's shared-memory tile for a panel of jb
// columns: jb rounded up to an even number of 16-byte vectors plus one
// vector -- an odd number of vectors, so 16-byte accesses to consecutive rows
// hit distinct banks (NB + 16/sizeof(T) for a full panel).  A narrower
// panel's rows take proportionally less shared memory, so taller panels fit
// one cluster.
template <typename T> __host__ __device__ constexpr int cl_rs(int jb) {
  return (jb + 32 / (int)sizeof(T) - 1) / (32 / (int)sizeof(T)) * (32 / (int)sizeof(T)) + 16 / (int)sizeof(T);
}

// Vector update of one row's columns [cb, jb) (cb >= 1): a -= l * P.
template <typename T>
__device__ __forceinline__ void row_axpy(T *row, const T *P, T l, int cb, int jb) {
  using V = typename Vec16<T>::type;
  constexpr int VE = 16 / (int)sizeof(T);
  const int nvj = (jb + VE - 1) / VE;
  int q = cb / VE;
  V *rv = reinterpret_cast<V *>(row);
  const V *pvec = reinterpret_cast<const V *>(P);
  if (q < nvj && (cb % VE != 0 || (q + 1) * VE > jb)) {   // first vector, masked
    V a0 = rv[q];
    const V p0 = pvec[q];
    T *x0 = reinterpret_cast<T *>(&a0);
    const T *y0 = reinterpret_cast<const T *>(&p0);
#pragma unroll
    for (int e = 0; e < VE; ++e)
      if (q * VE + e >= cb && q * VE + e < jb) x0[e] -= l * y0[e];
    rv[q] = a0;
    ++q;
  }
  const int qend = jb / VE;
  for (; q + 1 < qend; q += 2) {
    V a0 = rv[q], a1 = rv[q + 1];
    const V p0 = pvec[q], p1 = pvec[q + 1];
    T *x0 = reinterpret_cast<T *>(&a0);
    T *x1 = reinterpret_cast<T *>(&a1);
    const T *y0 = reinterpret_cast<const T *>(&p0);
    const T *y1 = reinterpret_cast<const T *>(&p1);
#pragma unroll
    for (int e = 0; e < VE; ++e) {
      x0[e] -= l * y0[e];
      x1[e] -= l * y1[e];
    }
    rv[q] = a0;
    rv[q + 1] = a1;
  }
  if (q < qend) {
    V a0 = rv[q];
    const V p0 = pvec[q];
    T *x0 = reinterpret_cast<T *>(&a0);
    const T *y0 = reinterpret_cast<const T *>(&p0);
#pragma unroll
    for (int e = 0; e < VE; ++e) x0[e] -= l * y0[e];
    rv[q] = a0;
    ++q;
  }
  if (q < nvj) {   // partial last vector
    V a0 = rv[q];
    const V p0 = pvec[q];
    T *x0 = reinterpret_cast<T *>(&a0);
    const T *y0 = reinterpret_cast<const T *>(&p0);
#pragma unroll
    for (int e = 0; e < VE; ++e)
      if (q * VE + e < jb) x0[e] -= l * y0[e];
    rv[q] = a0;
  }
}

// The previous step's update of this panel's columns, applied by the panel
// kernel itself as it loads them (FP32 factorization, full-width panels):
// L = the previous panel (A(kp.., kp..), kp = koff - NB), perm its
// interchange record (rows relative to kp); pw = NB, or 0 for none.  Each CTA
// applies the interchanges to its rows, solves the previous block row
// U12 = inv(L11) P A12 itself (a warp per four columns, from the unmodified
// values in global memory) and takes rows -= L21 U12 in FP32; CTA 0 writes
// U12 back after the cluster's last barrier, when every CTA has read what it
// needed.  The interchanges, the block-row solve and the update of the next
// panel's columns leave the path between two panels.
struct PanelPend {
  const float *L;
  const int *perm;
  int pw;
};
// U12 staged behind the panel's rows: 64 rows of four 16-column quarters at a
// stride of 20 floats (16-byte loads of the four quarters hit distinct banks)
constexpr int kPendUS = 80;
constexpr size_t kPendSmem = sizeof(float) * (size_t)NB * kPendUS;   // also holds L11 during the solve

// One CTA per SM (the panel's rows fill its shared memory): the whole
// register file is the CTA's.
template <typename T>
__global__ void __launch_bounds__(CT, 1)
    panel_cluster_kernel(T *Ag, int lda, int M, int jb, int koff, int *ipiv, int *info, int *perm, PanelPend pd) {
  using V = typename Vec16<T>::type;
  using K = typename PivKey<T>::K;
  constexpr int VE = 16 / (int)sizeof(T);        // elements per 16-byte vector
  constexpr int NV = NB / VE;                    // vectors per row
  const int RS = cl_rs<T>(jb);
  constexpr int NW = CT / 32;
  extern __shared__ __align__(16) unsigned char panel_dyn[];
  __shared__ __align__(16) ClusterRecv<T> recv[2];
  __shared__ __align__(8) uint64_t rbar[2];
  // pivot row and row j, double buffered by column parity: a thread still in
  // the previous column's phase 2 may read one while the next is copied
  __shared__ __align__(16) T Pb[2][NB];
  __shared__ __align__(16) T Jb[2][NB];
  __shared__ T s_rcp[2];
  __shared__ int s_use_rcp[2];
  __shared__ K wv[NW];
  __shared__ int wi[NW];
  __shared__ int piv_local[NB];
  cg::cluster_group cluster = cg::this_cluster();
  const int CN = (int)cluster.num_blocks();
  const int me = (int)cluster.block_rank();
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int chunk = (M + CN - 1) / CN;
  const int r0 = me * chunk;
  const int r1 = (r0 + chunk < M) ? r0 + chunk : M;
  const int nr = r1 - r0;
  const int nvj = (jb + VE - 1) / VE;            // vectors holding the jb columns
  T *sa = reinterpret_cast<T *>(panel_dyn);      // own rows, row-major, stride RS
#define AT(i_, c_) sa[(size_t)((i_) - r0) * RS + (c_)]
  // own rows into shared memory: a thread per row, each element an
  // asynchronous copy (coalesced over the warp's consecutive rows), all of
  // them in flight at once
  for (int i = tid; i < nr; i += CT) {
    const T *src = Ag + r0 + i;
    T *dst = sa + (size_t)i * RS;
    for (int c = 0; c < jb; ++c) {
      if (sizeof(T) == 8) cp_async8(dst + c, src + (size_t)c * lda, true);
      else cp_async4(dst + c, src + (size_t)c * lda, true);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  float *us = nullptr;   // U12 of the pending update (CTA 0 writes it back at the end)
  if constexpr (sizeof(T) == 4) {
    if (pd.pw == NB && jb == NB) {
      __shared__ int p_dst[2 * NB], p_src[2 * NB];
      us = reinterpret_cast<float *>(panel_dyn + (size_t)chunk * RS * sizeof(T));
      float *tri = us;                                   // L11 of the previous panel, then U12
      const int pn = pd.perm[0];
      for (int e = tid; e < pn; e += CT) {
        p_dst[e] = pd.perm[1 + e];
        p_src[e] = pd.perm[1 + 2 * NB + e];
      }
      for (int e = tid; e < NB * NB; e += CT) {   // asynchronous copies, all in flight
        const int i = e & (NB - 1), jj = e / NB;
        cp_async4(&tri[e], jj < i ? pd.L + i + (size_t)jj * lda : pd.L, jj < i);
      }
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      // own rows that the previous interchanges fill with block-row contents
      // (record entries NB.., whose sources are block rows: rows Ag - NB ..)
      for (int e = tid; e < (pn - NB) * NB; e += CT) {
        const int q = NB + e / NB, c = e % NB;
        const int r = p_dst[q] - NB;                     // this panel's row
        if (r >= r0 && r < r1 && p_dst[q] != p_src[q]) AT(r, c) = Ag[(p_src[q] - NB) + (size_t)c * lda];
      }
      // the previous block row's new rows (record entries 0..NB-1), solved:
      // warp w owns columns w, w+16, w+32, w+48; lane l rows l and l+32
      float x[4][2];
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const float *col = Ag + (size_t)(w + 16 * cc) * lda - NB;
        x[cc][0] = col[p_src[lane]];
        x[cc][1] = col[p_src[lane + 32]];
      }
      for (int jj = 0; jj < NB - 1; ++jj) {
        const int hi = jj >> 5;
        float xj[4];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) xj[cc] = __shfl_sync(0xffffffffu, hi ? x[cc][1] : x[cc][0], jj & 31);
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i > jj) {
            const float l = tri[jj * NB + i];
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) x[cc][s2] = fmaf(-l, xj[cc], x[cc][s2]);
          }
        }
      }
      __syncthreads();                                   // every warp is done with L11
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) {
        const int c = w + 16 * cc;
        us[lane * kPendUS + (c >> 4) * 20 + (c & 15)] = x[cc][0];
        us[(lane + 32) * kPendUS + (c >> 4) * 20 + (c & 15)] = x[cc][1];
      }
      __syncthreads();
      // rows -= L21 U12: thread (row pair p, quarter q) takes rows p and p+128
      // of each 256-row pass, 16 columns, FMAs onto the row values
      const int q4 = tid & 3, pr = tid >> 2;
      const float *L21 = pd.L + NB;                      // row koff + i of the previous panel: L21[i]
      for (int base = r0; base < r1; base += 256) {
        const int ia = base + pr, ib = ia + 128;
        const bool va = ia < r1, vb = ib < r1;
        float ca[16], cb[16];
        float4 *ra = reinterpret_cast<float4 *>(&AT(va ? ia : r0, q4 * 16));
        float4 *rb = reinterpret_cast<float4 *>(&AT(vb ? ib : r0, q4 * 16));
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const float4 a4 = ra[v], b4 = rb[v];
          ca[4 * v] = a4.x; ca[4 * v + 1] = a4.y; ca[4 * v + 2] = a4.z; ca[4 * v + 3] = a4.w;
          cb[4 * v] = b4.x; cb[4 * v + 1] = b4.y; cb[4 * v + 2] = b4.z; cb[4 * v + 3] = b4.w;
        }
        for (int j0 = 0; j0 < NB; j0 += 16) {
          // the 32 L values of this chunk in flight together (L2 latency, not
          // the FMAs, bounds this loop otherwise)
          float la[16], lb[16];
#pragma unroll
          for (int t = 0; t < 16; ++t) {
            la[t] = va ? L21[ia + (size_t)(j0 + t) * lda] : 0.f;
            lb[t] = vb ? L21[ib + (size_t)(j0 + t) * lda] : 0.f;
          }
#pragma unroll
          for (int t = 0; t < 16; ++t) {
            const float4 *u4 = reinterpret_cast<const float4 *>(us + (j0 + t) * kPendUS + q4 * 20);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              const float4 u = u4[v];
              ca[4 * v] = fmaf(-la[t], u.x, ca[4 * v]);
              ca[4 * v + 1] = fmaf(-la[t], u.y, ca[4 * v + 1]);
              ca[4 * v + 2] = fmaf(-la[t], u.z, ca[4 * v + 2]);
              ca[4 * v + 3] = fmaf(-la[t], u.w, ca[4 * v + 3]);
              cb[4 * v] = fmaf(-lb[t], u.x, cb[4 * v]);
              cb[4 * v + 1] = fmaf(-lb[t], u.y, cb[4 * v + 1]);
              cb[4 * v + 2] = fmaf(-lb[t], u.z, cb[4 * v + 2]);
              cb[4 * v + 3] = fmaf(-lb[t], u.w, cb[4 * v + 3]);
            }
          }
        }
        if (va)
#pragma unroll
          for (int v = 0; v < 4; ++v) ra[v] = make_float4(ca[4 * v], ca[4 * v + 1], ca[4 * v + 2], ca[4 * v + 3]);
        if (vb)
#pragma unroll
          for (int v = 0; v < 4; ++v) rb[v] = make_float4(cb[4 * v], cb[4 * v + 1], cb[4 * v + 2], cb[4 * v + 3]);
      }
      __syncthreads();
    }
  }
  // bytes a CTA receives per column: CN candidate records and row j
  const unsigned TX = (unsigned)(16 * (CN * (nvj + 1) + nvj));
  if (tid == 0) {
    mbar_init(&rbar[0], 1);
    mbar_init(&rbar[1], 1);
    fence_mbar_init();
    mbar_arrive_expect_tx(&rbar[0], TX);               // columns 0 and 1
    if (jb > 1) mbar_arrive_expect_tx(&rbar[1], TX);
  }
  __syncthreads();
  cluster.sync();   // every CTA's mbarriers are armed before the first message
  bool broken = false;   // a wait gave up: no further waits (the result is flagged)

  // Reduce the per-thread candidates (rows ci already complete) to the CTA's
  // first-max; keep its row and row jn locally, push |a| and row to all.
  auto publish = [&](K best, int bi, int jn) -> int {
    warp_argmax(best, bi);
    if (lane == 0) { wv[w] = best; wi[w] = bi; }
    __syncthreads();
    best = lane < NW ? wv[lane] : K(-1);
    bi = lane < NW ? wi[lane] : 0x7fffffff;
    warp_argmax(best, bi);
    return best >= K(0) ? bi : -1;
  };
  // Send column jn's candidate record (row ci, then {key, ci}) to every CTA,
  // and row jn if this CTA owns it: 16-byte st.async stores, a few per
  // thread.  Called after a CTA barrier that follows every write to those
  // rows.
  auto push = [&](K best, int ci, int jn) {
    const int par = jn & 1;
    const unsigned lbar = smem_u32(&rbar[par]);
    const bool own_j = (jn >= r0 && jn < r1);
    const int per = nvj + 1;
    for (int e = tid; e < CN * per; e += CT) {
      const int d = e / per, q = e - d * per;
      const unsigned db = cluster_map(lbar, d);
      uint4 v;
      if (q == nvj) {
        const unsigned long long kb = (unsigned long long)(long long)best;
        v = make_uint4((unsigned)kb, (unsigned)(kb >> 32), (unsigned)ci, 0u);
      } else {
        v = ci >= 0 ? reinterpret_cast<const uint4 *>(&AT(ci, 0))[q] : make_uint4(0u, 0u, 0u, 0u);
        if (own_j)
          st_async16(cluster_map(smem_u32(&recv[par].jrow[q]), d), reinterpret_cast<const uint4 *>(&AT(jn, 0))[q], db);
      }
      st_async16(cluster_map(smem_u32(&recv[par].row[me][q]), d), v, db);
    }
  };

  {
    K best = K(-1);
    int bi = 0x7fffffff;
    for (int i = r0 + tid; i < r1; i += CT) {
      const K a = PivKey<T>::key(AT(i, 0));
      if (a > best) { best = a; bi = i; }
    }
    const int ci = publish(best, bi, 0);
    push(ci >= 0 ? PivKey<T>::key(AT(ci, 0)) : K(-1), ci, 0);
  }

  for (int j = 0; j < jb; ++j) {
    const int par = j & 1;
    if (!broken) {                     // column j has arrived from every CTA
      // a column's exchange takes microseconds: give up after 2 s
      const bool ok = mbar_wait_for(&rbar[par], (unsigned)(j >> 1) & 1u, 2000000000ull);
      if (!ok) {
        broken = true;
        atomicOr(&g_lu_status, kErrMbarTimeout);
      } else if (tid == 0 && j + 2 < jb) {
        mbar_arrive_expect_tx(&rbar[par], TX);           // armed for column j+2
      }
    }
    // ---- global winner, computed by every warp from its own CTA's copies ----
    K v = K(-1);
    int b = 0x7fffffff, idx = -1;
    if (lane < CN) {
      const uint4 r = recv[par].row[lane][nvj];
      v = (K)(long long)(((unsigned long long)r.y << 32) | r.x);
      idx = (int)r.z;
      b = lane;
    }
    warp_winner(v, b, idx);
    const bool zero = !(b < CN && v > K(0));
    const int p = zero ? j : idx;
    if (tid == 0) {                // the pivots reach global memory after the loop
      piv_local[j] = p;
      if (zero && me == 0 && *info == 0) *info = koff + j + 1;
    }
    const bool last = (j + 1 >= jb);
    K best = K(-1);
    int bi = 0x7fffffff;
    if (!zero) {
      // the winner's row and row j, copied from the receive area (which the
      // senders reuse for column j+2 once this CTA has sent column j+1)
      T *Ps = Pb[par];
      T *Js = Jb[par];
      if (tid < 2 * NV) {
        if (tid < NV) {
          const uint4 pu = recv[par].row[b][tid < nvj ? tid : 0];
          const V pvec = *reinterpret_cast<const V *>(&pu);
          reinterpret_cast<V *>(Ps)[tid] = pvec;
          if (tid == j / VE) {   // once per CTA: FP64 division is costly
            const T *pe = reinterpret_cast<const T *>(&pvec);
            T pj = pe[0];
#pragma unroll
            for (int e = 1; e < VE; ++e)
              if (tid * VE + e == j) pj = pe[e];
            s_rcp[par] = T(1) / pj;
            s_use_rcp[par] = (pj < T(0) ? -pj : pj) > Lim<T>::safmin();
          }
        } else {
          const uint4 ju = recv[par].jrow[tid - NV < nvj ? tid - NV : 0];
          reinterpret_cast<V *>(Js)[tid - NV] = *reinterpret_cast<const V *>(&ju);
        }
      }
      __syncthreads();   // also: every thread is done with the previous column's phase 2
      const T pv = Ps[j];
      const bool use_rcp = s_use_rcp[par] != 0;
      const T rcp = s_rcp[par];
      const int lo = r0 > j ? r0 : j;
      // phase 1: rows j and p completely, one 16-byte vector per lane of a
      // warp each (nvj <= 32); every other own row its multiplier and
      // column j+1, with the first-max of column j+1
      if (w == NW - 1 && j >= r0 && j < r1 && lane < nvj)        // row j <- pivot row
        reinterpret_cast<V *>(&AT(j, 0))[lane] = reinterpret_cast<const V *>(Ps)[lane];
      if (w == NW - 2 && p != j && p >= r0 && p < r1 && lane < nvj) {   // row p <- old row j, eliminated
        const T l = use_rcp ? Js[j] * rcp : Js[j] / pv;
        V jv = reinterpret_cast<const V *>(Js)[lane];
        const V pvec = reinterpret_cast<const V *>(Ps)[lane];
        T *x = reinterpret_cast<T *>(&jv);
        const T *y = reinterpret_cast<const T *>(&pvec);
#pragma unroll
        for (int e = 0; e < VE; ++e) {
          const int c = lane * VE + e;
          if (c == j) x[e] = l;
          else if (c > j && c < jb) x[e] = x[e] - l * y[e];
        }
        reinterpret_cast<V *>(&AT(p, 0))[lane] = jv;
        if (!last && lane == (j + 1) / VE) {   // the lane's own store: visible to it
          const K a = PivKey<T>::key(AT(p, j + 1));
          if (a > best || (a == best && p < bi)) { best = a; bi = p; }
        }
      }
      for (int i = lo + tid; i < r1; i += CT) {
        if (i == j || i == p) continue;
        T *row = &AT(i, 0);
        const T src = row[j];
        const T l = use_rcp ? src * rcp : src / pv;
        row[j] = l;
        if (!last) {
          row[j + 1] -= l * Ps[j + 1];
          const K a = PivKey<T>::key(row[j + 1]);
          if (a > best || (a == best && i < bi)) { best = a; bi = i; }
        }
      }
      if (!last) {
        const int ci = publish(best, bi, j + 1);
        // complete the rows other CTAs may read: the candidate and row j+1
        const bool own_next = (j + 1 >= r0 && j + 1 < r1);
        if (tid < 32) {
          const int r = tid < 16 ? ci : (own_next ? j + 1 : -1);
          if (r >= 0 && r != p && r != j && (tid < 16 || r != ci)) {
            // 16 lanes per row, one vector each, over the columns j+2 .. jb-1
            for (int q = (tid & 15) + (j + 2) / VE; q < nvj; q += 16) {
              T *row = &AT(r, 0);
              const T l = row[j];
              V a0 = reinterpret_cast<V *>(row)[q];
              const V p0 = reinterpret_cast<const V *>(Ps)[q];
              T *x0 = reinterpret_cast<T *>(&a0);
              const T *y0 = reinterpret_cast<const T *>(&p0);
#pragma unroll
              for (int e = 0; e < VE; ++e)
                if (q * VE + e >= j + 2 && q * VE + e < jb) x0[e] -= l * y0[e];
              reinterpret_cast<V *>(row)[q] = a0;
            }
          }
        }
        __syncthreads();
        push(ci >= 0 ? PivKey<T>::key(AT(ci, j + 1)) : K(-1), ci, j + 1);
        // phase 2 (overlaps the exchange): columns j+2.. of the other rows
        if (j + 2 < jb) {
          for (int i = lo + tid; i < r1; i += CT) {
            if (i == j || i == p || i == ci || i == j + 1) continue;
            T *row = &AT(i, 0);
            row_axpy<T>(row, Ps, row[j], j + 2, jb);
          }
        }
      }
    } else if (!last) {
      const int lo = r0 > j + 1 ? r0 : j + 1;
      for (int i = lo + tid; i < r1; i += CT) {
        const K a = PivKey<T>::key(AT(i, j + 1));
        if (a > best) { best = a; bi = i; }
      }
      const int ci = publish(best, bi, j + 1);
      __syncthreads();
      push(ci >= 0 ? PivKey<T>::key(AT(ci, j + 1)) : K(-1), ci, j + 1);
    }
    if (last) break;
  }
  // every message to this CTA has arrived (the last column's wait); the
  // cluster barrier keeps all CTAs resident until that holds for each
  cluster.sync();
  if (me == 0)
    for (int t = tid; t < jb; t += CT) ipiv[t] = koff + piv_local[t];
  if (sizeof(T) == 4 && us != nullptr && me == 0)   // the pending update's U12, rows Ag - NB ..
    for (int e = tid; e < NB * NB; e += CT) {
      const int i = e & (NB - 1), c = e / NB;
      reinterpret_cast<float *>(Ag)[(i - NB) + (size_t)c * lda] = us[i * kPendUS + (c >> 4) * 20 + (c & 15)];
    }
  // warp 0 of the last CTA reduces the interchanges while its other warps
  // (and every other CTA) write the rows back: a thread per row, 16-byte
  // shared-memory reads, stores coalesced over the warp's consecutive rows
  const bool red = (me == CN - 1);
  if (red && w == 0) {
    reduce_interchanges(piv_local, jb, perm);
  } else {
    const int t0 = red ? tid - 32 : tid, nt = red ? CT - 32 : CT;
    for (int i = t0; i < nr; i += nt) {
      const V *srow = reinterpret_cast<const V *>(sa + (size_t)i * RS);
      T *dst = Ag + r0 + i;
      for (int q = 0; q < nvj; ++q) {
        const V v = srow[q];
        const T *x = reinterpret_cast<const T *>(&v);
#pragma unroll
        for (int e = 0; e < VE; ++e)
          if (q * VE + e < jb) dst[(size_t)(q * VE + e) * lda] = x[e];
      }
    }
  }
#undef AT
}

// The permutation record of a panel factored in two halves: its jb pivots
// (global rows, ipiv[t] for column koff + t) reduced as the panel kernels
// reduce theirs.  One warp.
__global__ void panel_perm_kernel(const int *ipiv, int jb, int koff, int *perm) {
  __shared__ int pl[NB];
  for (int t = threadIdx.x; t < jb; t += 32) pl[t] = ipiv[t] - koff;
  __syncwarp();
  reduce_interchanges(pl, jb, perm);
}

// Apply a row permutation (perm: count, dst[], src[] relative to row k) to
// the columns [0, c_split) and [c_from, N) of A: row k+dst[t] <- row k+src[t].
template <typename T>
__global__ void __launch_bounds__(256)
    apply_perm_kernel(T *A, int lda, int k, const int *perm, int c_split, int c_from, int N) {
  constexpr int CB = 32;
  __shared__ T v[2 * NB][CB];
  __shared__ int dst[2 * NB], src[2 * NB];
  const int n = perm[0];
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    dst[t] = perm[1 + t];
    src[t] = perm[1 + 2 * NB + t];
  }
  __syncthreads();
  const int nleft_blocks = (c_split + CB - 1) / CB;
  int c0;
  if ((int)blockIdx.x < nleft_blocks) c0 = blockIdx.x * CB;
  else c0 = c_from + (blockIdx.x - nleft_blocks) * CB;
  const int cend = ((int)blockIdx.x < nleft_blocks) ? c_split : N;
  const int ncols = (cend - c0 < CB) ? cend - c0 : CB;
  if (ncols <= 0) return;
  for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
    const int t = e % n, c = e / n;
    v[t][c] = A[k + src[t] + (size_t)(c0 + c) * lda];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
    const int t = e % n, c = e / n;
    if (dst[t] != src[t]) A[k + dst[t] + (size_t)(c0 + c) * lda] = v[t][c];
  }
}

// The interchanges of several steps on the columns left of their panels, in
// step order, in one launch: record r (perm0 + off[r], rows relative to k[r])
// applies to columns [0, kq[r]).  Only the finished factorization reads
// those columns, so a step's interchanges can wait for the batch.
constexpr int kPermBatch = 8;
struct PermBatch {
  int n;
  int k[kPermBatch], kq[kPermBatch], off[kPermBatch];
};

template <typename T>
__global__ void __launch_bounds__(256) apply_perm_batch_kernel(T *A, int lda, const int *perm0, PermBatch b) {
  constexpr int CB = 32;
  __shared__ T v[2 * NB][CB];
  __shared__ int dst[2 * NB], src[2 * NB];
  const int c0 = blockIdx.x * CB;
  for (int r = 0; r < b.n; ++r) {
    if (c0 >= b.kq[r]) continue;                     // the same for the whole CTA
    const int *perm = perm0 + b.off[r];
    const int k = b.k[r];
    const int n = perm[0];
    __syncthreads();                                 // the previous record's stores are done
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      dst[t] = perm[1 + t];
      src[t] = perm[1 + 2 * NB + t];
    }
    __syncthreads();
    const int ncols = (b.kq[r] - c0 < CB) ? b.kq[r] - c0 : CB;
    for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
      const int t = e % n, c = e / n;
      v[t][c] = A[k + src[t] + (size_t)(c0 + c) * lda];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * ncols; e += blockDim.x) {
      const int t = e % n, c = e / n;
      if (dst[t] != src[t]) A[k + dst[t] + (size_t)(c0 + c) * lda] = v[t][c];
    }
  }
}

// The block row of step k of the FP32 factorization for the columns
// [c0, c0 + ncols), in one launch: the panel's interchanges (record perm,
// rows relative to k), the solve with the panel's unit-lower jb x jb block
// (A(k.., k..)), and, when Bp is given, the solved rows packed as the 3xTF32
// B operand (row c of Bp is column c0 + c: TF32 high part, low part, high
// part, each kp floats, zero beyond the rows).  It replaces an interchange
// launch, a solve launch and a packing launch on the path between two panels.
// With jp = NB the previous panel's trailing update of these columns is
// still pending (the factorization pairs two steps into one update of rank
// 2 NB): the block rows first take x_i -= sum_j Lp(i, j) * u_j, u = the
// previous block row's solution (rows k-jp.. of the column), Lp = that
// panel's L at the block rows (A(k.., k-jp..), already interchanged), and
// the packing holds u then the solution (rank jp + jb).
// The record lists the jb block rows first (dst[t] = t for t < jb, as
// reduce_interchanges writes it), then the rows below that receive other
// contents.  Each CTA owns whole columns and reads every source of a column
// before it writes any destination.  A warp owns four columns; in the solve
// lane l holds rows l and l + 32 of each, and row i takes
// x_i -= L(i, j) * x_j for j = 0, 1, ... in turn (the order of the
// one-thread-per-column solve, so the results are the same).
constexpr int kBrCols = 32, kBrWarps = 8, kBrCpw = kBrCols / kBrWarps;

__global__ void __launch_bounds__(kBrWarps * 32)
    blockrow_kernel(float *__restrict__ A, int lda, int k, int jb, const int *__restrict__ perm, int c0, int ncols,
                    float *__restrict__ Bp, int kp, int jp) {
  extern __shared__ float br_dyn[];
  float *tri = br_dyn;                            // tri[j * NB + i] = L(i, j) for j < i < jb
  float *lp = br_dyn + NB * NB;                   // lp[j * NB + i] = Lp(i, j) (jp > 0 only)
  __shared__ float xs[kBrCols][NB + 1];           // new rows k..k+jb-1, one column per row of xs
  __shared__ float bl[NB][kBrCols + 1];           // record entries jb.. (rows below the block)
  __shared__ int dst[2 * NB], src[2 * NB];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int n = perm[0];
  const int cb = c0 + blockIdx.x * kBrCols;
  const int nc = (c0 + ncols - cb < kBrCols) ? c0 + ncols - cb : kBrCols;
  for (int e = t; e < n; e += kBrWarps * 32) {
    dst[e] = perm[1 + e];
    src[e] = perm[1 + 2 * NB + e];
  }
  // L11 (and Lp) as asynchronous copies, zero fill outside the triangle: all
  // of a thread's loads in flight at once (a load-then-store loop waited for
  // each in turn and dominated the kernel's latency)
  for (int e = t; e < NB * NB; e += kBrWarps * 32) {
    const int i = e & (NB - 1), j = e / NB;
    const bool ok = j < i && i < jb;
    cp_async4(&tri[e], ok ? A + k + i + (size_t)(k + j) * lda : A, ok);
    if (jp) {
      const bool okp = i < jb;
      cp_async4(&lp[e], okp ? A + k + i + (size_t)(k - jp + j) * lda : A, okp);
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  // gather: every load of the warp's columns issued before the first store
  float v[kBrCpw][4];
#pragma unroll
  for (int cc = 0; cc < kBrCpw; ++cc) {
    const int c = warp + kBrWarps * cc;
    const float *col = A + k + (size_t)(cb + c) * lda;
#pragma unroll
    for (int qq = 0; qq < 4; ++qq) {
      const int q = lane + 32 * qq;
      v[cc][qq] = (c < nc && q < n) ? col[src[q]] : 0.f;
    }
  }
#pragma unroll
  for (int cc = 0; cc < kBrCpw; ++cc) {
    const int c = warp + kBrWarps * cc;
#pragma unroll
    for (int qq = 0; qq < 4; ++qq) {
      const int q = lane + 32 * qq;
      if (q < jb) xs[c][dst[q]] = v[cc][qq];
      else if (q < n) bl[q - jb][c] = v[cc][qq];
    }
  }
  __syncthreads();
  // rows below the block, then the solve of the warp's own columns
#pragma unroll
  for (int cc = 0; cc < kBrCpw; ++cc) {
    const int c = warp + kBrWarps * cc;
    if (c < nc) {
      float *col = A + k + (size_t)(cb + c) * lda;
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        const int q = jb + lane + 32 * qq;
        if (q < n && dst[q] != src[q]) col[dst[q]] = bl[q - jb][c];
      }
    }
  }
  float x[kBrCpw][2], u[kBrCpw][2];
#pragma unroll
  for (int cc = 0; cc < kBrCpw; ++cc) {
    const int c = warp + kBrWarps * cc;
    x[cc][0] = (lane < jb) ? xs[c][lane] : 0.f;
    x[cc][1] = (lane + 32 < jb) ? xs[c][lane + 32] : 0.f;
    const float *col = A + k + (size_t)(cb + (c < nc ? c : 0)) * lda;
    u[cc][0] = (jp && lane < jp) ? col[lane - jp] : 0.f;
    u[cc][1] = (jp && lane + 32 < jp) ? col[lane + 32 - jp] : 0.f;
  }
  for (int j = 0; j < jp; ++j) {
    const int hi = j >> 5;
    float uj[kBrCpw];
#pragma unroll
    for (int cc = 0; cc < kBrCpw; ++cc) uj[cc] = __shfl_sync(0xffffffffu, hi ? u[cc][1] : u[cc][0], j & 31);
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const float l = lp[j * NB + lane + 32 * s2];
#pragma unroll
      for (int cc = 0; cc < kBrCpw; ++cc) x[cc][s2] = fmaf(-l, uj[cc], x[cc][s2]);
    }
  }
  for (int j = 0; j < jb - 1; ++j) {
    const int hi = j >> 5;
    float xj[kBrCpw];
#pragma unroll
    for (int cc = 0; cc < kBrCpw; ++cc) xj[cc] = __shfl_sync(0xffffffffu, hi ? x[cc][1] : x[cc][0], j & 31);
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int i = lane + 32 * s2;
      if (i > j) {
        const float l = tri[j * NB + i];
#pragma unroll
        for (int cc = 0; cc < kBrCpw; ++cc) x[cc][s2] = fmaf(-l, xj[cc], x[cc][s2]);
      }
    }
  }
#pragma unroll
  for (int cc = 0; cc < kBrCpw; ++cc) {
    const int c = warp + kBrWarps * cc;
    if (c >= nc) continue;
    float *col = A + k + (size_t)(cb + c) * lda;
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int i = lane + 32 * s2;
      if (i < jb) col[i] = x[cc][s2];
    }
    if (Bp) {
      // packed row: u (jp values, 0 or NB), then the solution (jb values)
      float *out = Bp + (size_t)(blockIdx.x * kBrCols + c) * 3 * kp;
      float val[4] = {jp ? u[cc][0] : x[cc][0], jp ? u[cc][1] : x[cc][1], jp ? x[cc][0] : 0.f,
                      jp ? x[cc][1] : 0.f};
#pragma unroll
      for (int sl = 0; sl < 4; ++sl) {
        const int i = lane + 32 * sl;
        if (i < kp) {
          const float xv = i < jp + jb ? val[sl] : 0.f;
          const float h = tf32_rna(xv);
          out[i] = h;
          out[kp + i] = xv - h;
          out[2 * kp + i] = h;
        }
      }
    }
  }
}

static void blockrow_f32(float *A, int lda, int k, int jb, const int *perm, int c0, int ncols, float *Bp, int jp,
                         cudaStream_t st) {
  if (ncols <= 0) return;
  static std::once_flag once;
  std::call_once(once, [] {
    ATLG_CHECK(cudaFuncSetAttribute(blockrow_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(sizeof(float) * 2 * NB * NB)));
  });
  const int kp = (jp + jb + 31) / 32 * 32;
  const size_t smem = sizeof(float) * (jp ? 2 : 1) * NB * NB;
  blockrow_kernel<<<(ncols + kBrCols - 1) / kBrCols, kBrWarps * 32, smem, st>>>(A, lda, k, jb, perm, c0, ncols, Bp,
                                                                               kp, jp);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

// laswp as one permutation: laswp_perm_kernel runs the interchange sequence
// K1..K2-1 (reversed when inci < 0) on a row-content table held in shared
// memory (global memory above kPermSmemRows rows), then the rows are moved
// by laswp_cols_kernel (or, for tables too large for shared memory, by one
// gather into scratch and one copy back).  use_smem = 2 also stages the
// K2-K1 pivots in shared memory first, so the one-thread interchange chain
// runs on shared-memory operands only (no L2 round trip per interchange).
constexpr int kPermSmemRows = 48 * 1024;

__global__ void laswp_perm_kernel(const int *ipiv, int K1, int K2, int inci, int *content_g, int nrows,
                                  int use_smem) {
  extern __shared__ int content_s[];
  int *content = use_smem ? content_s : content_g;
  int *piv_s = content_s + nrows;
  const int n = K2 - K1;
  const int step = inci > 0 ? inci : -inci;
  for (int i = threadIdx.x; i < nrows; i += blockDim.x) content[i] = i;
  if (use_smem == 2)
    for (int s = threadIdx.x; s < n; s += blockDim.x) piv_s[s] = ipiv[(size_t)(K1 + s) * step];
  __syncthreads();
  if (threadIdx.x == 0 && use_smem == 2) {
    // pivots read a batch ahead into registers: each interchange is then two
    // shared loads with known addresses and two stores, no load-to-address wait
    constexpr int B = 16;
    for (int s0 = 0; s0 < n; s0 += B) {
      int ipb[B];
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int s = s0 + u;
        ipb[u] = s < n ? piv_s[(inci > 0 ? K1 + s : K2 - 1 - s) - K1] : -1;
      }
#pragma unroll
      for (int u = 0; u < B; ++u) {
        const int s = s0 + u;
        const int i = inci > 0 ? K1 + s : K2 - 1 - s;
        const int ip = ipb[u];
        if (s >= n || ip == i || ip < 0 || ip >= nrows) continue;
        const int a = content[i], b = content[ip];
        content[i] = b;
        content[ip] = a;
      }
    }
  } else if (threadIdx.x == 0) {
    for (int s = 0; s < n; ++s) {
      const int i = inci > 0 ? K1 + s : K2 - 1 - s;
      const int ip = ipiv[(size_t)i * step];
      if (ip == i || ip < 0 || ip >= nrows) continue;
      const int t = content[i];
      content[i] = content[ip];
      content[ip] = t;
    }
  }
  __syncthreads();
  if (use_smem)
    for (int i = threadIdx.x; i < nrows; i += blockDim.x) content_g[i] = content_s[i];
}
// The interchange chain without the chain, for pivots that only look down
// (ipiv[i] >= i, as getrf produces).  Position i is final after step i, and
// what it receives is what the last earlier step with the same target left
// there, so with
//   last(x)  = the largest source j whose target ipiv[j] is x,
//   prev(j)  = the largest source j' < j with the same target as j,
//   V(i)     = the row at position i just before step i
//            = V(last(i)) when some j < i targets i, else i,
// the forward result is content[i] = V(prev(i)), or ipiv[i] when i is the
// first source of its target, or V(i) for a self-interchange (i in [K1,K2));
// content[x] = V(last(x)), or x when nothing targets x (elsewhere).  The
// backward order (inci < 0) gives the inverse permutation.  One CTA.
// prev/last come from a counting sort of the sources by target: counts per
// target (shared-memory atomics), an exclusive scan over the targets, each
// source dropped into its target's bucket, then one thread per target sorts
// its (few) sources and links them -- every step parallel over the CTA.
// When some target has more than kBucketMax sources, or the buckets do not
// fit, warp 0 finds prev/last 32 sources at a time instead
// (__match_any_sync groups equal targets).  Pointer jumping resolves V in
// log2(n) rounds.  Pivot vectors that do not look down run the one-thread
// chain on the same shared arrays.
// Shared memory: ints r[n] (pivots, then the encoded prev), ptr[n], val[n],
// ls[nrows] (last(x)); with buckets also cnt[nrows + 1] and bkt[n].
constexpr int kChainThreads = 1024;
constexpr int kChainPer = 16;                       // sources per thread in the jumping rounds
constexpr size_t kChainSmemMax = 200 * 1024;
constexpr int kBucketMax = 64;                      // sources per target sorted by one thread

static size_t chain_smem_bytes(int nrows, int n, bool buckets) {
  return sizeof(int) * (3 * (size_t)n + (size_t)nrows + (buckets ? (size_t)nrows + 1 + n : 0));
}
static bool chain_fits(int nrows, int n) {
  return n <= kChainThreads * kChainPer && chain_smem_bytes(nrows, n, false) <= kChainSmemMax;
}
static bool chain_bucket_fits(int nrows, int n) {
  return n <= kChainThreads * kChainPer && chain_smem_bytes(nrows, n, true) <= kChainSmemMax;
}

// Exclusive scan of v[0..m) in place by the whole CTA (kChainThreads
// threads); returns the total.
__device__ int cta_exclusive_scan(int *v, int m, int *wsum) {
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int per = (m + kChainThreads - 1) / kChainThreads;
  const int b = tid * per, e = min(b + per, m);
  int sum = 0;
  for (int i = b; i < e; ++i) sum += v[i];
  int incl = sum;                                    // warp inclusive scan of the segment sums
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    int x = wsum[lane], xi = x;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    wsum[lane] = xi - x;                             // exclusive over warps
    if (lane == 31) wsum[32] = xi;
  }
  __syncthreads();
  int run = wsum[w] + incl - sum;
  for (int i = b; i < e; ++i) {
    const int t = v[i];
    v[i] = run;
    run += t;
  }
  const int total = wsum[32];
  __syncthreads();
  return total;
}

// PER: sources per thread in the jumping rounds (8 when n <= 8192: half the
// predicated-off work of 16 for the common sizes)
template <int PER>
__global__ void __launch_bounds__(kChainThreads)
    laswp_chain_kernel(const int *ipiv, int K1, int K2, int inci, int *content_g, int nrows, int buckets) {
  extern __shared__ int ch_smem[];
  __shared__ int wsum[33];
  const int n = K2 - K1;
  const int step = inci > 0 ? inci : -inci;
  int *r = ch_smem, *ptr = ch_smem + n, *val = ch_smem + 2 * n, *ls = ch_smem + 3 * n;
  int *cnt = ls + nrows, *bkt = cnt + nrows + 1;
  const int tid = threadIdx.x;
  int viol = 0;
  for (int x = tid; x < nrows; x += kChainThreads) ls[x] = -1;
  // the pivots, 8 loads in flight per thread (one dependent round trip per
  // batch instead of per pivot)
  for (int s0 = tid; s0 < n; s0 += 8 * kChainThreads) {
    int ipb[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int s = s0 + u * kChainThreads;
      ipb[u] = s < n ? ipiv[(size_t)(K1 + s) * step] : 0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int s = s0 + u * kChainThreads, j = K1 + s, ip = ipb[u];
      if (s < n) {
        r[s] = ip;
        if (ip != j && ip >= 0 && ip < nrows && ip < j) viol = 1;
      }
    }
  }
  if (__syncthreads_or(viol)) {        // general pivots: the chain, one thread
    for (int x = tid; x < nrows; x += kChainThreads) ls[x] = x;
    __syncthreads();
    if (tid == 0)
      for (int t = 0; t < n; ++t) {
        const int s = inci > 0 ? t : n - 1 - t;
        const int i = K1 + s, ip = r[s];
        if (ip == i || ip < 0 || ip >= nrows) continue;
        const int a = ls[i], b = ls[ip];
        ls[i] = b;
        ls[ip] = a;
      }
    __syncthreads();
    for (int x = tid; x < nrows; x += kChainThreads) content_g[x] = ls[x];
    return;
  }
  bool linked = false;
  if (buckets) {                       // counting sort of the sources by target
    for (int x = tid; x <= nrows; x += kChainThreads) cnt[x] = 0;
    __syncthreads();
    for (int s = tid; s < n; s += kChainThreads) {
      const int j = K1 + s, ip = r[s];
      if (ip != j && ip >= 0 && ip < nrows) atomicAdd(&cnt[ip], 1);
    }
    __syncthreads();
    cta_exclusive_scan(cnt, nrows, wsum);
    for (int s = tid; s < n; s += kChainThreads) {
      const int j = K1 + s, ip = r[s];
      if (ip != j && ip >= 0 && ip < nrows) bkt[atomicAdd(&cnt[ip], 1)] = j;
    }
    __syncthreads();
    // cnt[x] is now the end of bucket x, cnt[x-1] its start
    int big = 0;
    for (int x = tid; x < nrows; x += kChainThreads) {
      const int b0 = x ? cnt[x - 1] : 0, b1 = cnt[x];
      if (b1 - b0 > kBucketMax) big = 1;
    }
    if (!__syncthreads_or(big)) {
      for (int s = tid; s < n; s += kChainThreads) {   // sources that move nothing: V(j)
        const int j = K1 + s, ip = r[s];
        if (!(ip != j && ip >= 0 && ip < nrows)) r[s] = j;
      }
      __syncthreads();
      for (int x = tid; x < nrows; x += kChainThreads) {
        const int b0 = x ? cnt[x - 1] : 0, b1 = cnt[x];
        if (b1 == b0) continue;
        for (int a = b0 + 1; a < b1; ++a) {          // insertion sort by source
          const int v = bkt[a];
          int c = a - 1;
          while (c >= b0 && bkt[c] > v) { bkt[c + 1] = bkt[c]; --c; }
          bkt[c + 1] = v;
        }
        int prev = -2 - x;                             // the first source receives original row x
        for (int a = b0; a < b1; ++a) {
          const int j = bkt[a];
          r[j - K1] = prev;
          prev = j;
        }
        ls[x] = prev;
      }
      linked = true;
    }
  }
  if (!linked && tid < 32) {           // prev(j) into r, last(x) into ls, 32 sources at a time
    const int lane = tid;
    for (int s0 = 0; s0 < n; s0 += 32) {
      const int s = s0 + lane, j = K1 + s;
      int x = -1;
      if (s < n) {
        const int ip = r[s];
        if (ip != j && ip >= 0 && ip < nrows) x = ip;
      }
      const unsigned grp = __match_any_sync(0xffffffffu, x >= 0 ? x : -1 - lane);
      const unsigned lower = grp & ((1u << lane) - 1u);
      int q = j;                                       // self: V(j)
      if (x >= 0) {
        if (lower) q = K1 + s0 + (31 - __clz(lower));  // an earlier source in this group of 32
        else {
          const int l = ls[x];
          q = l >= 0 ? l : -2 - x;                     // -2 - x: the original row x
        }
      }
      const bool top = x >= 0 && (grp >> lane) == 1u;  // the group's last source
      __syncwarp();
      if (s < n) r[s] = q;
      if (top) ls[x] = j;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int s = tid; s < n; s += kChainThreads) {
    const int l = ls[K1 + s];
    ptr[s] = l >= 0 ? l - K1 : -1;
    val[s] = K1 + s;
  }
  __syncthreads();
  for (;;) {                           // pointer jumping: V(i) = V(last(i))
    int np[PER], nv[PER];
    int any = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int s = tid + k * kChainThreads;
      np[k] = -1;
      nv[k] = 0;
      if (s < n) {
        const int p = ptr[s];
        if (p >= 0) {
          nv[k] = val[p];
          np[k] = ptr[p];
          any = 1;
        } else {
          nv[k] = val[s];
        }
      }
    }
    if (!__syncthreads_or(any)) break;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int s = tid + k * kChainThreads;
      if (s < n) {
        ptr[s] = np[k];
        val[s] = nv[k];
      }
    }
    __syncthreads();
  }
  for (int x = tid; x < nrows; x += kChainThreads) {
    int c;
    if (x >= K1 && x < K2) {
      const int q = r[x - K1];
      c = q >= 0 ? val[q - K1] : -2 - q;
    } else {
      const int l = ls[x];
      c = l >= 0 ? val[l - K1] : x;
    }
    if (inci > 0) content_g[x] = c;
    else content_g[c] = x;
  }
}

// The row-content table of the interchanges K1..K2-1 into content (nrows ints).
static void launch_interchange_table(const int *ipiv, int K1, int K2, int inci, int *content, int nrows,
                                     cudaStream_t st) {
  const int n = K2 - K1;
  if (chain_fits(nrows, n)) {
    // the warp scan takes n/32 dependent rounds: cheap for a block column's
    // interchanges, the counting sort wins for a whole pivot vector
    const bool bk = n > 2048 && chain_bucket_fits(nrows, n);
    const size_t smem = chain_smem_bytes(nrows, n, bk);
    if (n <= 8 * kChainThreads) {
      ATLG_CHECK(cudaFuncSetAttribute(laswp_chain_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kChainSmemMax));
      laswp_chain_kernel<8><<<1, kChainThreads, smem, st>>>(ipiv, K1, K2, inci, content, nrows, bk ? 1 : 0);
    } else {
      ATLG_CHECK(cudaFuncSetAttribute(laswp_chain_kernel<kChainPer>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kChainSmemMax));
      laswp_chain_kernel<kChainPer><<<1, kChainThreads, smem, st>>>(ipiv, K1, K2, inci, content, nrows,
                                                                    bk ? 1 : 0);
    }
  } else {
    const int mode = ((long)nrows + n <= kPermSmemRows) ? 2 : (nrows <= kPermSmemRows ? 1 : 0);
    const size_t smem = mode == 2 ? sizeof(int) * ((size_t)nrows + n) : mode == 1 ? sizeof(int) * (size_t)nrows : 0;
    ATLG_CHECK(cudaFuncSetAttribute(laswp_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    laswp_perm_kernel<<<1, 1024, smem, st>>>(ipiv, K1, K2, inci, content, nrows, mode);
  }
}

template <typename T>
__global__ void gather_rows_kernel(const T *A, int lda, T *W, int ldw, const int *content, int nrows, int N) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)nrows * N; e += (long)gridDim.x * blockDim.x) {
    const int r = (int)(e % nrows), c = (int)(e / nrows);
    W[r + (size_t)c * ldw] = A[content[r] + (size_t)c * lda];
  }
}
template <typename T>
__global__ void copy_rows_kernel(T *A, int lda, const T *W, int ldw, int nrows, int N) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)nrows * N; e += (long)gridDim.x * blockDim.x) {
    const int r = (int)(e % nrows), c = (int)(e / nrows);
    A[r + (size_t)c * lda] = W[r + (size_t)c * ldw];
  }
}

static int grid_for(long work) {
  long b = (work + 255) / 256;
  if (b > 8L * 152) b = 8L * 152;
  if (b < 1) b = 1;
  return (int)b;
}

// laswp_cols_kernel applies the row permutation `content` (row r <- row
// content[r], rows [0, nrows)) to N columns of A with the rows of a column
// held in shared memory: one read of what moves and one write, no scratch
// copy of A.  Every CTA loads the table, counts the rows that move (mv) and
// the span [lo, hi) they cover, then per column
//   dense  (4*mv >= span): rows [lo, hi) read with coalesced loads into
//          shared memory, only the moved rows written back;
//   sparse (a few rows moving in a tall column, as for the interchanges of
//          one block column): a compact (destination, source) list, only the
//          source rows read, for G columns at a time.
// Algorithmic bytes per column: 2 * sizeof(T) * mv (each moved element read
// and written once); the dense form also reads the unmoved rows of the span.
constexpr int kLcThreads = 1024;
constexpr size_t kLaswpColsSmemMax = 200 * 1024;

__host__ __device__ inline size_t laswp_cols_table_bytes(int nrows) {
  return ((size_t)nrows * sizeof(int) + 15) & ~size_t(15);
}
template <typename T>
inline size_t laswp_cols_smem(int nrows) {
  return laswp_cols_table_bytes(nrows) + (size_t)nrows * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(kLcThreads)
    laswp_cols_kernel(T *A, int lda, const int *__restrict__ content_g, int nrows, int N) {
  extern __shared__ __align__(16) unsigned char lc_smem[];
  int *content = reinterpret_cast<int *>(lc_smem);
  unsigned char *buf = lc_smem + laswp_cols_table_bytes(nrows);
  const size_t buf_bytes = (size_t)nrows * sizeof(T);
  __shared__ int s_lo, s_hi, s_mv, s_cnt;
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) { s_lo = nrows; s_hi = 0; s_mv = 0; s_cnt = 0; }
  __syncthreads();
  int lo = nrows, hi = 0, mv = 0;
  for (int r0 = tid; r0 < nrows; r0 += 8 * kLcThreads) {   // 8 table loads in flight per thread
    int sb[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int r = r0 + u * kLcThreads;
      sb[u] = r < nrows ? __ldg(content_g + r) : r;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int r = r0 + u * kLcThreads, s = sb[u];
      if (r < nrows) {
        content[r] = s;
        if (s != r) { lo = min(lo, r); hi = max(hi, r + 1); ++mv; }
      }
    }
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  mv = __reduce_add_sync(0xffffffffu, mv);
  if (lane == 0) { atomicMin(&s_lo, lo); atomicMax(&s_hi, hi); atomicAdd(&s_mv, mv); }
  __syncthreads();
  lo = s_lo; hi = s_hi; mv = s_mv;
  if (mv == 0) return;
  if (4 * (long)mv >= (long)(hi - lo)) {
    T *col = reinterpret_cast<T *>(buf);
    constexpr int U = 8;
    for (int c = blockIdx.x; c < N; c += gridDim.x) {
      T *colp = A + (size_t)c * lda;
      for (int b = lo + tid; b < hi; b += U * kLcThreads) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int r = b + u * kLcThreads;
          v[u] = r < hi ? colp[r] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int r = b + u * kLcThreads;
          if (r < hi) col[r] = v[u];
        }
      }
      __syncthreads();
      for (int r = lo + tid; r < hi; r += kLcThreads) {
        const int s = content[r];
        if (s != r) colp[r] = col[s];
      }
      __syncthreads();
    }
    return;
  }
  // sparse: compact (destination, source) pairs, warp-aggregated
  int2 *pr = reinterpret_cast<int2 *>(buf);
  for (int r0 = lo + (tid & ~31); r0 < hi; r0 += kLcThreads) {
    const int r = r0 + lane;
    const int s = r < hi ? content[r] : r;
    const bool moves = r < hi && s != r;
    const unsigned m = __ballot_sync(0xffffffffu, moves);
    int base = 0;
    if (lane == 0 && m) base = atomicAdd(&s_cnt, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (moves) pr[base + __popc(m & ((1u << lane) - 1u))] = make_int2(r, s);
  }
  __syncthreads();
  const size_t pair_bytes = ((size_t)mv * sizeof(int2) + 15) & ~size_t(15);
  T *vals = reinterpret_cast<T *>(buf + pair_bytes);
  int G = (int)((buf_bytes - pair_bytes) / ((size_t)mv * sizeof(T)));
  G = G < 1 ? 1 : (G > 8 ? 8 : G);
  for (int c0 = blockIdx.x * G; c0 < N; c0 += gridDim.x * G) {
    const int gc = (N - c0 < G) ? N - c0 : G;
    for (int e = tid; e < gc * mv; e += kLcThreads) {
      const int g = e / mv, k = e - g * mv;
      vals[e] = A[pr[k].y + (size_t)(c0 + g) * lda];
    }
    __syncthreads();
    for (int e = tid; e < gc * mv; e += kLcThreads) {
      const int g = e / mv, k = e - g * mv;
      A[pr[k].x + (size_t)(c0 + g) * lda] = vals[e];
    }
    __syncthreads();
  }
}

// The rows that can move are [0, nrows); nrows must exceed every pivot.
template <typename T>
static void laswp_impl(int N, T *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows,
                       cudaStream_t st) {
  if (K2 <= K1 || N <= 0 || nrows <= 0) return;
  Context &c = ctx();
  int *content = static_cast<int *>(c.buffer(kBufW3, sizeof(int) * (size_t)nrows));
  launch_interchange_table(ipiv, K1, K2, inci, content, nrows, st);
  const size_t csmem = laswp_cols_smem<T>(nrows);
  if (csmem <= kLaswpColsSmemMax) {
    ATLG_CHECK(cudaFuncSetAttribute(laswp_cols_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kLaswpColsSmemMax));
    int per_sm = 0;
    ATLG_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, laswp_cols_kernel<T>, kLcThreads, csmem));
    if (per_sm < 1) per_sm = 1;
    const long cap = (long)per_sm * c.num_sms;
    const int grid = (int)(N < cap ? N : cap);
    laswp_cols_kernel<T><<<grid, kLcThreads, csmem, st>>>(A, lda, content, nrows, N);
    note_launch(2);
  } else {
    T *W = static_cast<T *>(c.buffer(kBufW4, sizeof(T) * (size_t)nrows * N));
    gather_rows_kernel<T><<<grid_for((long)nrows * N), 256, 0, st>>>(A, lda, W, nrows, content, nrows, N);
    copy_rows_kernel<T><<<grid_for((long)nrows * N), 256, 0, st>>>(A, lda, W, nrows, nrows, N);
    note_launch(3);
  }
  ATLG_CHECK(cudaGetLastError());
}

// Row permutation of a factorization: perm[i] = source row of row i after
// the interchanges ipiv[0..n) are applied in order (ATL_laswp forward), so
// that the forward interchange of one vector is y[i] = b[perm[i]].
void dev_perm_from_ipiv(const int *ipiv, int n, int *perm, cudaStream_t st) {
  launch_interchange_table(ipiv, 0, n, 1, perm, n, st);
  note_launch();
  ATLG_CHECK(cudaGetLastError());
}

template <typename T>
__global__ void permute_vec_kernel(int n, const int *perm, const T *in, T *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = in[perm[i]];
}

// x <- (LU)^-1 P x for one FP32 right-hand side with a precomputed permutation
// (the refinement loop solves with the same factor many times).
void dev_sgetrs_perm(int n, const float *LU, int lda, const int *perm, float *x, float *tmp, cudaStream_t st) {
  permute_vec_kernel<float><<<(n + 255) / 256, 256, 0, st>>>(n, perm, x, tmp);
  ATLG_CHECK(cudaMemcpyAsync(x, tmp, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, st));
  note_launch();
  dev_strsv_inv(kLower, kNoTrans, kUnit, n, LU, lda, x, st);
  dev_strsv_inv(kUpper, kNoTrans, kNonUnit, n, LU, lda, x, st);
}

void dev_sgetrs_perm_chain(int n, const float *LU, int lda, const int *perm, float *x, float *tmp, const float *wsL,
                           const float *wsU, cudaStream_t st) {
  permute_vec_kernel<float><<<(n + 255) / 256, 256, 0, st>>>(n, perm, x, tmp);
  note_launch();
  dev_strsv_chain(kLower, n, LU, lda, wsL, tmp, st);
  dev_strsv_chain(kUpper, n, LU, lda, wsU, tmp, st);
  ATLG_CHECK(cudaMemcpyAsync(x, tmp, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, st));
}

void dev_dlaswp(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows, cudaStream_t st) {
  laswp_impl<double>(N, A, lda, K1, K2, ipiv, inci, nrows, st);
}
void dev_slaswp(int N, float *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows, cudaStream_t st) {
  laswp_impl<float>(N, A, lda, K1, K2, ipiv, inci, nrows, st);
}

// ------------------------------------------------------------------ getrf
template <typename T>
static void gemm_any(int M, int N, int K, const T *A, int lda, const T *B, int ldb, T *C, int ldc, cudaStream_t st);
template <>
void gemm_any<double>(int M, int N, int K, const double *A, int lda, const double *B, int ldb, double *C, int ldc,
                      cudaStream_t st) {
  dev_dgemm(kNoTrans, kNoTrans, M, N, K, -1.0, A, lda, B, ldb, 1.0, C, ldc, st);
}
template <>
void gemm_any<float>(int M, int N, int K, const float *A, int lda, const float *B, int ldb, float *C, int ldc,
                     cudaStream_t st) {
  dev_sgemm(kNoTrans, kNoTrans, M, N, K, -1.0f, A, lda, B, ldb, 1.0f, C, ldc, st);
}

// Trailing update A22 -= L21 * U12 for columns [c0, c0+n) of the U12 block
// (first column c_from): the FFMA/DFMA GEMM, or for the mixed solver's FP32
// factor the 3xTF32 tensor-core update on panels packed once per step.
template <typename T>
static void trailing_update(bool tc, int m, int n, int jb, const T *L21, const T *U12, T *C, int lda, int boff,
                            int ntot, const float *Ap, const float *Bp, cudaStream_t st) {
  if (m <= 0 || n <= 0) return;
  if (tc) {
    dev_sgemm_tf32x3_packed(m, n, jb, -1.0f, Ap, Bp, ntot, boff, (float *)C + (size_t)boff * lda, lda, st);
    return;
  }
  gemm_any<T>(m, n, jb, L21, lda, U12 + (size_t)boff * lda, lda, C + (size_t)boff * lda, lda, st);
}

// The block row of step k (rows k..k+jb-1) for columns [c0, c0+n): the
// panel's interchanges and the unit-lower solve; FP32 in one launch that
// also packs the 3xTF32 B operand when Bp is given.
// jp = NB: the previous panel's update of these columns is pending (FP32
// tensor-core factorization only; blockrow_kernel).
template <typename T>
static void block_row(T *A, int lda, int k, int jb, const int *perm, int c0, int n, float *Bp, int jp,
                      cudaStream_t st) {
  if (n <= 0) return;
  if constexpr (sizeof(T) == 4) {
    blockrow_f32(A, lda, k, jb, perm, c0, n, Bp, jp, st);
  } else {
    apply_perm_kernel<T><<<(n + 31) / 32, 256, 0, st>>>(A, lda, k, perm, 0, c0, c0 + n);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    dev_trsm_llnu_block(A, lda, k, jb, A + k + (size_t)c0 * lda, lda, n, st);
  }
}

// Largest cluster (16, else 8 CTAs) the panel kernel can be launched with at
// its full shared-memory size (the device's opt-in maximum per block less the
// kernel's static shared memory -- the receive areas of the exchange); size 0
// when clusters are unavailable.
struct ClusterCfg {
  int size = 0;
  size_t smem = 0;   // dynamic shared memory per CTA: the rows of the panel
};
static bool g_panel_cluster = true;

template <typename T>
static const ClusterCfg &cluster_cfg() {
  static std::once_flag once;
  static ClusterCfg cfg;
  std::call_once(once, [] {
    auto k = panel_cluster_kernel<T>;
    cudaFuncAttributes fa;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, (const void *)k) != cudaSuccess || (size_t)optin <= fa.sharedSizeBytes + 1024) {
      (void)cudaGetLastError();
      return;
    }
    const size_t smax = ((size_t)optin - fa.sharedSizeBytes) & ~size_t(1023);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax) != cudaSuccess) {
      (void)cudaGetLastError();
      return;
    }
    const int sizes[2] = {16, 8};
    for (int q = 0; q < 2; ++q) {
      cudaLaunchConfig_t lc = {};
      cudaLaunchAttribute at[1];
      lc.gridDim = dim3(sizes[q]);
      lc.blockDim = dim3(CT);
      lc.dynamicSmemBytes = smax;
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = sizes[q];
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      lc.attrs = at;
      lc.numAttrs = 1;
      int n = 0;
      if (cudaOccupancyMaxActiveClusters(&n, (const void *)k, &lc) == cudaSuccess && n > 0) {
        cfg.size = sizes[q];
        cfg.smem = smax;
        break;
      }
      (void)cudaGetLastError();
    }
  });
  return cfg;
}

void set_panel_cluster(bool on) { g_panel_cluster = on; }
// A panel too tall for one cluster at its full width, but not at half of it,
// is factored as two halves on the cluster (left half; its interchanges,
// triangular solve and update on the right half; right half) instead of on
// the cooperative grid: the cluster's per-column exchange is the faster one.
static bool g_panel_split = true;
void set_panel_split(bool on) { g_panel_split = on; }
// Below ~12k rows the panel chain, not the update, is the critical path, and
// a paired step only lengthens it (n = 16384: 12288 measured best of 4096 to
// 12288 in steps of 2048).
constexpr int kDeferRowsDefault = 12288;
static int g_defer_rows = kDeferRowsDefault;
// FP32 tensor-core factorization: the next panel applies a step's update of
// its columns itself (PanelPend) where it can
static bool g_panel_fuse = true;
void set_panel_fuse(bool on) { g_panel_fuse = on; }
void set_defer_rows(int rows) { g_defer_rows = rows < 0 ? kDeferRowsDefault : rows > 0 ? rows : INT_MAX; }
static int g_panel_grid = 0;   // CTAs of the grid panel; 0: the default below
void set_panel_grid(int ctas) { g_panel_grid = ctas > 0 ? ctas : 0; }
// Panel width of the FP64 LU (8..NB, a multiple of 8).  A panel's own
// rank-1 updates run on the FP64 pipe of the few SMs the panel occupies
// (M x w^2 / 2 FMAs per panel); a narrower panel moves that work into the
// trailing DGEMMs, which use every SM.
static int g_panel_nb_f64 = NB;
void set_panel_width_f64(int w) { g_panel_nb_f64 = (w >= 8 && w <= NB) ? w / 8 * 8 : NB; }

template <typename T>
static void getrf_impl(int M, int N, T *A, int lda, int *ipiv, int *info, cudaStream_t st, bool tc = false,
                       int pw_f64 = 0) {
  ATLG_CHECK(cudaMemsetAsync(info, 0, sizeof(int), st));
  if (M <= 0 || N <= 0) return;
  Context &c = ctx();
  const int MN = M < N ? M : N;
  const int PW = (sizeof(T) == 8) ? (pw_f64 > 0 ? pw_f64 : g_panel_nb_f64) : NB;   // panel width
  // Look-ahead: the trailing update of step k is split into the next panel's
  // columns (on the caller's stream, so panel k+1 can start at once) and the
  // rest (on a low-priority side stream, overlapping panel k+1).  The panel
  // grid then takes a quarter of the SMs, as few as its shared-memory slices
  // allow, leaving the rest to the concurrent update.
  const bool lookahead = MN > 2 * PW && N > 2 * PW;
  int G = c.num_sms;
  if (lookahead) {
    G = c.num_sms / 4;
    while (G < c.num_sms && ((size_t)((M + G - 1) / G) * PW * sizeof(T)) > kPanelSmemMax) G += 1;
  }
  if (g_panel_grid > 0) G = g_panel_grid < c.num_sms ? g_panel_grid : c.num_sms;
  // at least a few rows per CTA for the tallest panel
  if (G > (M + 7) / 8) G = (M + 7) / 8;
  if (G < 1) G = 1;
  // one scratch block: rec[2G][RS] T, jrow[2NB] T, bar[2], perm[npan][1+4NB]
  // (a permutation record per panel: the interchanges of the columns left of
  // a panel run later, on the side stream)
  const int npan = (MN + PW - 1) / PW;
  constexpr int kPermInts = 1 + 4 * NB;
  const size_t tbytes = sizeof(T) * ((size_t)2 * G * rec_stride<T>() + 2 * NB);
  const size_t ibytes = sizeof(int) * ((size_t)2 + (size_t)kPermInts * npan);
  unsigned char *scr = static_cast<unsigned char *>(c.buffer(kBufW0, tbytes + ibytes + 64));
  T *rec = reinterpret_cast<T *>(scr);
  T *jrow = rec + (size_t)2 * G * rec_stride<T>();
  unsigned *bar = reinterpret_cast<unsigned *>(scr + ((tbytes + 15) & ~size_t(15)));
  int *perm0 = reinterpret_cast<int *>(bar + 2);
  ATLG_CHECK(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), st));
  ATLG_CHECK(cudaFuncSetAttribute(panel_kernel<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kPanelSmemMax));
  cudaStream_t side = c.side_stream();
  cudaEvent_t ev_ready = c.sync_event(0), ev_side = c.sync_event(1), ev_first = c.sync_event(4);
  bool side_pending = false;    // side-stream work of the last side step not yet waited for
  bool first_pending = false;   // its first part (the columns of the panel after next)
  const int cn = g_panel_cluster ? cluster_cfg<T>().size : 0;
  const size_t cmax = cluster_cfg<T>().smem;
  bool used_cluster = false;
  // A side step of the tensor-core factorization whose trailing matrix is
  // tall defers its far update into the next step's: one update of rank 2 PW
  // reads and writes C once for two panels (the C read-modify-write bounds
  // that update).  The next panel's columns still get this step's update at
  // once.  pend = the rank (0 or PW) owed by the previous step.
  auto side_step_at = [&](int kk) {
    const int jbk = (MN - kk < PW) ? MN - kk : PW;
    const int cf = kk + jbk;
    const int nx = (cf < MN) ? ((MN - cf < PW) ? MN - cf : PW) : 0;
    return lookahead && cf < N && kk + jbk < M && nx > 0 && cf + nx < N;
  };
  auto tc_at = [&](int kk) {
    const int jbk = (MN - kk < PW) ? MN - kk : PW;
    return tc && M - kk - jbk >= 256 && N - kk - jbk >= 128;
  };
  int pend = 0;
  // the next-panel update a step hands to the next panel's kernel (FP32
  // tensor-core factorization; PanelPend)
  PanelPend next_pend = {nullptr, nullptr, 0};
  // interchanges of the columns left of the panels, batched on the side stream
  PermBatch lbatch;
  lbatch.n = 0;
  auto flush_left = [&](cudaStream_t s) {
    if (lbatch.n == 0) return;
    int maxq = 0;
    for (int r = 0; r < lbatch.n; ++r) maxq = lbatch.kq[r] > maxq ? lbatch.kq[r] : maxq;
    apply_perm_batch_kernel<T><<<(maxq + 31) / 32, 256, 0, s>>>(A, lda, perm0, lbatch);
    note_launch();
    ATLG_CHECK(cudaGetLastError());
    lbatch.n = 0;
  };
  if (tc && lookahead) {   // the packings at their largest (rank 2 PW) once, before any side-stream use
    c.buffer(kBufT0, sizeof(float) * tf32x3_packed_floats(M, 2 * PW, false));
    c.buffer(kBufT2, sizeof(float) * tf32x3_packed_floats(M, 2 * PW, false));
    c.buffer(kBufT1, sizeof(float) * tf32x3_packed_floats(N, 2 * PW, true));
  }

  for (int k = 0; k < MN; k += PW) {
    const int jb = (MN - k < PW) ? MN - k : PW;
    T *Ap = A + k + (size_t)k * lda;
    int Mp = M - k;
    int *ipk = ipiv + k;
    int koff = k;
    int *perm = perm0 + (size_t)(k / PW) * kPermInts;
    void *args[] = {&Ap, (void *)&lda, &Mp, (void *)&jb, &koff, &ipk, &info, &rec, &jrow, &bar, &perm};
    cudaEvent_t prof_b = nullptr;
    if (c.prof_panels) {
      prof_b = c.event();
      ATLG_CHECK(cudaEventRecord(prof_b, st));
    }
    // one cluster when the panel fits its shared memory (panels only shrink,
    // so the grid path below is never needed after it)
    auto cluster_tile = [&](int rows, int width) -> size_t {
      return cn ? sizeof(T) * (size_t)((rows + cn - 1) / cn) * cl_rs<T>(width) : 0;
    };
    auto launch_cluster = [&](T *Apan, int rows, int width, int kof, int *ip, size_t tile, PanelPend pd) {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      cfg.gridDim = dim3(cn);
      cfg.blockDim = dim3(CT);
      cfg.dynamicSmemBytes = tile;
      cfg.stream = st;
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = cn;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      ATLG_CHECK(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T>, Apan, lda, rows, width, kof, ip, info, perm, pd));
    };
    const PanelPend none = {nullptr, nullptr, 0};
    const size_t ctile = cluster_tile(Mp, jb);
    const int h = jb / 2;
    const size_t htile = cluster_tile(Mp, jb - h);   // the taller half is the left one
    if (next_pend.pw && !(cn && jb == NB && ctile + kPendSmem <= cmax)) {
      fprintf(stderr, "atlas_gb300: getrf: a pending panel update without room for it\n");
      abort();
    }
    if (cn && ctile <= cmax) {
      launch_cluster(Ap, Mp, jb, koff, ipk, ctile + (next_pend.pw ? kPendSmem : 0), next_pend);
      next_pend = none;
      used_cluster = true;
    } else if (cn && g_panel_split && h >= 8 && htile <= cmax) {
      T *Ar = A + k + (size_t)(k + h) * lda;          // rows k.. of the right half
      launch_cluster(Ap, Mp, h, koff, ipk, htile, none);
      block_row<T>(A, lda, k, h, perm, k + h, jb - h, nullptr, 0, st);
      gemm_any<T>(Mp - h, jb - h, h, Ap + h, lda, Ar, lda, Ar + h, lda, st);
      launch_cluster(Ar + h, Mp - h, jb - h, koff + h, ipk + h, cluster_tile(Mp - h, jb - h), none);
      apply_perm_kernel<T><<<(h + 31) / 32, 256, 0, st>>>(A, lda, k + h, perm, 0, k, k + h);
      panel_perm_kernel<<<1, 32, 0, st>>>(ipk, jb, koff, perm);
      note_launch(3);   // with the one below: two panels, the left half's interchanges, the record
      ATLG_CHECK(cudaGetLastError());
      used_cluster = true;
    } else {
      if (used_cluster) {   // the grid barrier counts every earlier column
        const unsigned base = (unsigned)koff * (unsigned)G;
        ATLG_CHECK(cudaMemcpyAsync(bar, &base, sizeof(unsigned), cudaMemcpyHostToDevice, st));
        ATLG_CHECK(cudaStreamSynchronize(st));
        used_cluster = false;
      }
      // the CTA's rows of the panel live in shared memory when they fit
      const size_t tile = sizeof(T) * (size_t)((Mp + G - 1) / G) * jb;
      if (tile <= kPanelSmemMax)
        ATLG_CHECK(cudaLaunchCooperativeKernel((const void *)panel_kernel<T, true>, dim3(G), dim3(PT), args, tile, st));
      else
        ATLG_CHECK(cudaLaunchCooperativeKernel((const void *)panel_kernel<T, false>, dim3(G), dim3(PT), args, 0, st));
    }
    note_launch();
    if (prof_b) {
      cudaEvent_t prof_e = c.event();
      ATLG_CHECK(cudaEventRecord(prof_e, st));
      c.panel_recs.push_back({prof_b, prof_e, (double)jb});
    }
    const int c_from = k + jb;
    const int nxt = (c_from < MN) ? ((MN - c_from < PW) ? MN - c_from : PW) : 0;
    const int far0 = c_from + nxt;                     // first column beyond the next panel
    const int nl = (k + 31) / 32;
    // A side step splits the work right of the panel: the next panel's
    // columns (interchanges, block-row solve, update) on the caller's stream,
    // so panel k+1 starts at once; everything beyond them on the side stream,
    // which (tensor-core updates) does the panel after next's columns first
    // and records that, so step k+1 waits only for those.  The left columns' interchanges (needed
    // only by the finished factorization) run last on the side stream.
    const bool side_step = lookahead && c_from < N && k + jb < M && nxt > 0 && far0 < N;
    if (side_step) {
      if (first_pending) {                             // the next panel's columns got step k-1's update
        ATLG_CHECK(cudaStreamWaitEvent(st, ev_first, 0));
        first_pending = false;
      }
      const int m = M - k - jb, ntot = N - c_from;
      const bool use_tc = tc && m >= 256 && ntot >= 128;
      const bool defer = pend == 0 && use_tc && jb == PW && M - k >= g_defer_rows && side_step_at(k + PW) &&
                         tc_at(k + PW);
      // the next panel applies this step's update of its columns itself when
      // it is one full-width cluster panel with room for the staged block row
      const bool fuse = sizeof(T) == 4 && g_panel_fuse && use_tc && !defer && pend == 0 && jb == NB &&
                        nxt == NB && cn && cluster_tile(M - c_from, NB) + kPendSmem <= cmax;
      const int kq = k - pend;                          // this step's update: L columns kq..k+jb-1
      const int rk = pend + jb;                         // its rank
      const T *L21 = A + (k + jb) + (size_t)kq * lda;
      const T *U12 = A + kq + (size_t)c_from * lda;
      T *C = A + (k + jb) + (size_t)c_from * lda;
      if (pend) {   // the deferred panel's L rows take this step's interchanges before they are used
        apply_perm_kernel<T><<<(pend + 31) / 32, 256, 0, st>>>(A, lda, k, perm, 0, kq, k);
        note_launch();
        ATLG_CHECK(cudaGetLastError());
      }
      float *Ap = nullptr, *Bp = nullptr;
      if (use_tc) {   // two A packings in turn: the side stream may still read the last one
        Ap = static_cast<float *>(c.buffer(((k / PW) & 1) ? kBufT2 : kBufT0,
                                           sizeof(float) * tf32x3_packed_floats(m, rk, false)));
        Bp = static_cast<float *>(c.buffer(kBufT1, sizeof(float) * tf32x3_packed_floats(ntot, rk, true)));
      }
      if (fuse) {
        next_pend = {reinterpret_cast<const float *>(A + k + (size_t)k * lda), perm, NB};
      } else {
        block_row<T>(A, lda, k, jb, perm, c_from, nxt, Bp, pend, st);
        if (use_tc) dev_sgemm_tf32x3_pack_a(m, rk, (const float *)L21, lda, Ap, st);
        trailing_update<T>(use_tc, m, nxt, rk, L21, U12, C, lda, 0, ntot, Ap, Bp, st);
      }
      ATLG_CHECK(cudaEventRecord(ev_ready, st));
      ATLG_CHECK(cudaStreamWaitEvent(side, ev_ready, 0));
      if (fuse) dev_sgemm_tf32x3_pack_a(m, rk, (const float *)L21, lda, Ap, side);
      const int nfar = N - far0;
      const size_t rstride = (size_t)3 * ((rk + 31) / 32 * 32);   // floats per packed row of B
      block_row<T>(A, lda, k, jb, perm, far0, nfar, (use_tc && !defer) ? Bp + (size_t)nxt * rstride : nullptr, pend,
                   side);
      if (defer) {
        ATLG_CHECK(cudaEventRecord(ev_first, side));
      } else {
        // the panel after next's columns as their own launch only where the
        // update is fast enough for the panel chain to be the critical path
        // (tensor-core updates); the FFMA/DFMA update is the critical path
        // itself, and a split would only add a small, inefficient launch
        const int nxt2 = (far0 < MN) ? ((MN - far0 < PW) ? MN - far0 : PW) : 0;
        const int first = (use_tc && nxt2 > 0 && nxt2 < nfar) ? nxt2 : nfar;
        trailing_update<T>(use_tc, m, first, rk, L21, U12, C, lda, nxt, ntot, Ap, Bp, side);
        ATLG_CHECK(cudaEventRecord(ev_first, side));
        if (first < nfar)
          trailing_update<T>(use_tc, m, nfar - first, rk, L21, U12, C, lda, nxt + first, ntot, Ap, Bp, side);
      }
      first_pending = true;
      if (kq > 0) {                                     // left columns (the deferred panel's are done)
        lbatch.k[lbatch.n] = k;
        lbatch.kq[lbatch.n] = kq;
        lbatch.off[lbatch.n] = (k / PW) * kPermInts;
        if (++lbatch.n == kPermBatch) flush_left(side);
      }
      ATLG_CHECK(cudaEventRecord(ev_side, side));
      side_pending = true;
      pend = defer ? jb : 0;
      continue;
    }
    // otherwise everything on the caller's stream, after all side work
    if (lbatch.n) {
      flush_left(side);
      ATLG_CHECK(cudaEventRecord(ev_side, side));
      side_pending = true;
    }
    if (side_pending) {
      ATLG_CHECK(cudaStreamWaitEvent(st, ev_side, 0));
      side_pending = false;
      first_pending = false;
    }
    const int nr = (N - c_from + 31) / 32;
    if (nl + nr > 0) {
      apply_perm_kernel<T><<<nl + nr, 256, 0, st>>>(A, lda, k, perm, k, c_from, N);
      note_launch();
      ATLG_CHECK(cudaGetLastError());
    }
    if (c_from < N) {
      dev_trsm_llnu_block(A, lda, k, jb, A + k + (size_t)c_from * lda, lda, N - c_from, st);
      if (k + jb < M) {
        const int m = M - k - jb, ntot = N - c_from;
        const T *L21 = A + (k + jb) + (size_t)k * lda;
        const T *U12 = A + k + (size_t)c_from * lda;
        T *C = A + (k + jb) + (size_t)c_from * lda;
        const bool use_tc = tc && m >= 256 && ntot >= 128;
        float *Ap = nullptr, *Bp = nullptr;
        if (use_tc) {
          Ap = static_cast<float *>(c.buffer(kBufT0, sizeof(float) * tf32x3_packed_floats(m, jb, false)));
          Bp = static_cast<float *>(c.buffer(kBufT1, sizeof(float) * tf32x3_packed_floats(ntot, jb, true)));
          dev_sgemm_tf32x3_pack_a(m, jb, (const float *)L21, lda, Ap, st);
          dev_sgemm_tf32x3_pack_b(jb, ntot, (const float *)U12, lda, Bp, st);
        }
        trailing_update<T>(use_tc, m, ntot, jb, L21, U12, C, lda, 0, ntot, Ap, Bp, st);
      }
    }
  }
  if (lbatch.n) {
    flush_left(side);
    ATLG_CHECK(cudaEventRecord(ev_side, side));
    side_pending = true;
  }
  if (side_pending) ATLG_CHECK(cudaStreamWaitEvent(st, ev_side, 0));
}

void dev_dgetrf(int M, int N, double *A, int lda, int *ipiv, int *info, cudaStream_t st) {
  getrf_impl<double>(M, N, A, lda, ipiv, info, st);
}
void dev_dgetrf_pw(int M, int N, double *A, int lda, int *ipiv, int *info, int pw, cudaStream_t st) {
  getrf_impl<double>(M, N, A, lda, ipiv, info, st, false, (pw >= 8 && pw <= NB) ? pw / 8 * 8 : NB);
}
void dev_sgetrf(int M, int N, float *A, int lda, int *ipiv, int *info, cudaStream_t st) {
  getrf_impl<float>(M, N, A, lda, ipiv, info, st);
}
void dev_sgetrf_tc(int M, int N, float *A, int lda, int *ipiv, int *info, cudaStream_t st) {
  getrf_impl<float>(M, N, A, lda, ipiv, info, st, true);
}

// ------------------------------------------------------------------ getrs
template <typename T>
static void trsm_any(int order, int side, int uplo, int ta, int diag, int M, int N, const T *A, int lda, T *B,
                     int ldb, cudaStream_t st) {
  // cblas order handling: RowMajor flips Side and Uplo and swaps M, N
  if (order == kRowMajor) {
    side = side == kLeft ? kRight : kLeft;
    uplo = uplo == kUpper ? kLower : kUpper;
    const int t = M; M = N; N = t;
  }
  if (sizeof(T) == 8)
    dev_dtrsm(side, uplo, ta, diag, M, N, 1.0, (const double *)A, lda, (double *)B, ldb, st);
  else
    dev_strsm(side, uplo, ta, diag, M, N, 1.0f, (const float *)A, lda, (float *)B, ldb, st);
}

template <typename T>
static void getrs_impl(int order, int trans, int N, int NRHS, const T *A, int lda, const int *ipiv, T *B, int ldb,
                       cudaStream_t st) {
  if (!N || !NRHS) return;
  // laswp over the N "rows" of B in the column-major sense, as the reference calls it
  if (order == kColMajor && NRHS == 1) {
    // one right-hand side: single-launch look-back TRSV for each factor
    auto trsv = [&](int uplo, int ta, int diag) {
      if (sizeof(T) == 8) dev_dtrsv(uplo, ta, diag, N, (const double *)A, lda, (double *)B, st);
      else dev_strsv(uplo, ta, diag, N, (const float *)A, lda, (float *)B, st);
    };
    if (trans == kNoTrans) {
      laswp_impl<T>(1, B, ldb, 0, N, ipiv, 1, N, st);
      trsv(kLower, kNoTrans, kUnit);
      trsv(kUpper, kNoTrans, kNonUnit);
    } else {
      trsv(kUpper, trans, kNonUnit);
      trsv(kLower, trans, kUnit);
      laswp_impl<T>(1, B, ldb, 0, N, ipiv, -1, N, st);
    }
    return;
  }
  if (order == kColMajor && NRHS >= 8 && N >= 256) {
    // many right-hand sides: the solves apply 64 x 64 diagonal-block inverses
    auto solve = [&](int uplo, int ta, int diag) {
      if (sizeof(T) == 8)
        dev_dtrsm_left_inv(uplo, ta, diag, N, NRHS, (const double *)A, lda, (double *)B, ldb, st);
      else
        dev_strsm_left_inv(uplo, ta, diag, N, NRHS, (const float *)A, lda, (float *)B, ldb, st);
    };
    if (trans == kNoTrans) {
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, 1, N, st);
      solve(kLower, kNoTrans, kUnit);
      solve(kUpper, kNoTrans, kNonUnit);
    } else {
      solve(kUpper, kTrans, kNonUnit);
      solve(kLower, kTrans, kUnit);
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, -1, N, st);
    }
  } else if (order == kColMajor) {
    if (trans == kNoTrans) {
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, 1, N, st);
      trsm_any<T>(order, kLeft, kLower, kNoTrans, kUnit, N, NRHS, A, lda, B, ldb, st);
      trsm_any<T>(order, kLeft, kUpper, kNoTrans, kNonUnit, N, NRHS, A, lda, B, ldb, st);
    } else {
      trsm_any<T>(order, kLeft, kUpper, trans, kNonUnit, N, NRHS, A, lda, B, ldb, st);
      trsm_any<T>(order, kLeft, kLower, trans, kUnit, N, NRHS, A, lda, B, ldb, st);
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, -1, N, st);
    }
  } else {
    if (trans == kNoTrans) {
      trsm_any<T>(order, kRight, kLower, kTrans, kNonUnit, NRHS, N, A, lda, B, ldb, st);
      trsm_any<T>(order, kRight, kUpper, kTrans, kUnit, NRHS, N, A, lda, B, ldb, st);
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, -1, N, st);
    } else {
      laswp_impl<T>(NRHS, B, ldb, 0, N, ipiv, 1, N, st);
      trsm_any<T>(order, kRight, kUpper, kNoTrans, kUnit, NRHS, N, A, lda, B, ldb, st);
      trsm_any<T>(order, kRight, kLower, kNoTrans, kNonUnit, NRHS, N, A, lda, B, ldb, st);
    }
  }
}

void dev_dgetrs(int order, int trans, int N, int NRHS, const double *A, int lda, const int *ipiv, double *B, int ldb,
                cudaStream_t st) {
  getrs_impl<double>(order, trans, N, NRHS, A, lda, ipiv, B, ldb, st);
}
void dev_sgetrs(int order, int trans, int N, int NRHS, const float *A, int lda, const int *ipiv, float *B, int ldb,
                cudaStream_t st) {
  getrs_impl<float>(order, trans, N, NRHS, A, lda, ipiv, B, ldb, st);
}

unsigned lu_status_read_and_clear() {
  unsigned v = 0, z = 0;
  ATLG_CHECK(cudaMemcpyFromSymbol(&v, g_lu_status, sizeof(v)));
  if (v) ATLG_CHECK(cudaMemcpyToSymbol(g_lu_status, &z, sizeof(z)));
  return v;
}


// ------------------------------------------------- laswp without allocation
// Some callers cannot let a library allocate device memory in the middle of
// their work: programs that hand all device memory to their own pool
// allocator up front, and programs that cannot accept the device-wide
// synchronisation that cudaMalloc / cudaFree imply.  atlg_dlaswp_noalloc is
// the row-interchange operation of atlg_dlaswp_dev for them: its scratch (the
// row-content table and the gathered rows) lives in the fixed array below,
// which the CUDA runtime reserves on every GPU that loads this library and
// keeps until the process exits.
//
//  - Limit: 4*nrows bytes (rounded up to 256) + 8*nrows*N bytes must fit in
//    kNoAllocScratchBytes (16 MiB); larger calls are rejected with a message
//    on stderr and return -2, before any work is queued.
//  - Set-up: the first call on each device looks up the array's device
//    address with cudaGetSymbolAddress while that device is current.  Make
//    that first call before beginning any stream capture.
//  - Every call shares the one array, so calls whose work overlaps on the GPU
//    (different streams, or concurrent host threads) race on it; serialise
//    them.  Nothing in the array has to start at zero: the permutation kernel
//    fills its whole table and the gather writes every element the copy back
//    reads, so the contents left by the previous call are never read.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static unsigned char *noalloc_scratch_for_current_device() {
  static std::mutex mu;
  static unsigned char *addr[256] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      fprintf(stderr, "atlg_dlaswp_noalloc: cudaGetSymbolAddress failed on device %d: %s\n", dev,
              cudaGetErrorString(e));
      return nullptr;
    }
    addr[dev] = static_cast<unsigned char *>(p);
  }
  return addr[dev];
}

}  // namespace atlg

extern "C" int atlg_dlaswp_noalloc(int N, double *A, int lda, int K1, int K2, const int *ipiv, int inci, int nrows,
                                   void *stream) {
  using namespace atlg;
  if (N < 0 || nrows < 0 || lda < (nrows > 1 ? nrows : 1)) return -1;
  if (K2 <= K1 || N == 0 || nrows == 0) return 0;
  // the interchanges K1..K2-1 name rows of the table, which has nrows entries
  if (K1 < 0 || K2 > nrows) return -1;
  const size_t table = ((size_t)nrows * sizeof(int) + 255) & ~size_t(255);
  const size_t need = table + (size_t)nrows * (size_t)N * sizeof(double);
  if (need > kNoAllocScratchBytes) {
    fprintf(stderr,
            "atlg_dlaswp_noalloc: %d rows x %d columns need %zu bytes of scratch; the fixed scratch holds %zu "
            "(4*nrows rounded to 256 + 8*nrows*N must not exceed it)\n",
            nrows, N, need, kNoAllocScratchBytes);
    return -2;
  }
  unsigned char *base = noalloc_scratch_for_current_device();
  if (!base) return -3;
  int *content = reinterpret_cast<int *>(base);
  double *W = reinterpret_cast<double *>(base + table);
  // NULL means the library's own stream, as for every other atlg_*_dev entry
  // point (creating it allocates no device memory)
  cudaStream_t st = stream_of(stream);
  int use_smem = nrows <= kPermSmemRows;
  const size_t smem = use_smem ? sizeof(int) * (size_t)nrows : 0;
  if (cudaFuncSetAttribute(laswp_perm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
      cudaSuccess)
    return -3;
  // each launch reports its own status, so an error left by an unrelated
  // earlier call is neither blamed on this one nor cleared
  const dim3 grid(grid_for((long)nrows * N));
  int ld_w = nrows;
  void *perm_args[] = {(void *)&ipiv, &K1, &K2, &inci, &content, &nrows, &use_smem};
  void *gather_args[] = {&A, &lda, &W, &ld_w, &content, &nrows, &N};
  void *copy_args[] = {&A, &lda, &W, &ld_w, &nrows, &N};
  if (cudaLaunchKernel((const void *)laswp_perm_kernel, dim3(1), dim3(1024), perm_args, smem, st) != cudaSuccess)
    return -3;
  if (cudaLaunchKernel((const void *)gather_rows_kernel<double>, grid, dim3(256), gather_args, 0, st) !=
      cudaSuccess)
    return -3;
  if (cudaLaunchKernel((const void *)copy_rows_kernel<double>, grid, dim3(256), copy_args, 0, st) != cudaSuccess)
    return -3;
  note_launch(3);
  return 0;
}
