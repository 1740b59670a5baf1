"""Generates tests/golden/atlas_ref_fixtures.npz from the reference's own
routines (oracle/_ref/libatlref.so, built by oracle/ref_build.sh from the
reference basefiles).  Run once where the reference source tree is present:

    sh oracle/ref_build.sh <reference tree> && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --large      # headline sizes (minutes)

The fixtures pin the oracle and the GPU library to the reference:
  * ATL_rand streams and ATL_gegen matrices (bit-exact),
  * ATL_getrfC / ATL_getrfR pivots and info (bit-exact) and LU factors,
  * ATL_laswp permutations (bit-exact),
  * ATL_getrs solutions, reference-BLAS gemm and trsm results (tolerance).
"""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REFLIB = os.path.join(ROOT, "oracle", "_ref", "libatlref.so")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "atlas_ref_fixtures.npz")

dp = np.ctypeslib.ndpointer(np.float64, flags="F_CONTIGUOUS")
sp = np.ctypeslib.ndpointer(np.float32, flags="F_CONTIGUOUS")
ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
v1 = np.ctypeslib.ndpointer(np.float64, ndim=1, flags="C_CONTIGUOUS")
I, D, F = C.c_int, C.c_double, C.c_float


def load():
    R = C.CDLL(REFLIB)
    R.atlref_srand.argtypes = [I]
    R.atlref_rand.restype = I
    R.atlref_dgegen.argtypes = [I, I, dp, I, I]
    R.atlref_sgegen.argtypes = [I, I, sp, I, I]
    R.atlref_dgetrf.argtypes = [I, I, I, dp, I, ip]
    R.atlref_dgetrf.restype = I
    R.atlref_sgetrf.argtypes = [I, I, I, sp, I, ip]
    R.atlref_sgetrf.restype = I
    R.atlref_dgetrs.argtypes = [I, I, I, I, dp, I, ip, dp, I]
    R.atlref_dlaswp.argtypes = [I, dp, I, I, I, ip, I]
    R.atlref_dgemm.argtypes = [I, I, I, I, I, I, D, dp, I, dp, I, D, dp, I]
    R.atlref_dtrsm.argtypes = [I, I, I, I, I, I, I, D, dp, I, dp, I]
    R.atlref_dsyrk.argtypes = [I, I, I, I, I, D, dp, I, D, dp, I]
    R.atlref_dpotrf.argtypes = [I, I, I, dp, I]
    R.atlref_dpotrf.restype = I
    R.atlref_spotrf.argtypes = [I, I, I, sp, I]
    R.atlref_spotrf.restype = I
    R.atlref_dpotrs.argtypes = [I, I, I, I, dp, I, dp, I]
    R.atlref_dtrmm.argtypes = [I, I, I, I, I, I, I, D, dp, I, dp, I]
    R.atlref_dgemv.argtypes = [I, I, I, I, D, dp, I, v1, I, D, v1, I]
    R.atlref_dtrsv.argtypes = [I, I, I, I, I, dp, I, v1, I]
    R.atlref_dtrtri.argtypes = [I, I, I, I, dp, I]
    R.atlref_dtrtri.restype = I
    R.atlref_dgetri.argtypes = [I, I, dp, I, ip]
    R.atlref_dgetri.restype = I
    return R


def iamax_cases(rng):
    """(buffer, N, incX) cases for cblas_i?amax: random, ties, zeros, signed
    zeros, infinities, and NaNs followed by ordered and inverted runs."""
    nan, inf = np.nan, np.inf
    vecs = [rng.standard_normal(n) for n in (0, 1, 2, 3, 4, 5, 7, 8, 9, 31, 100, 1000)]
    vecs += [np.array(v, dtype=np.float64) for v in (
        [1.0, -3.0, 3.0, 2.0, -3.0], [0.0, 0.0, 0.0, 0.0, 0.0], [0.0, -0.0, 0.0, -0.0, 0.0, 0.0],
        [-0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 5e-324], [2.0, inf, 1.0, -inf, 7.0], [1.0, -inf, inf, 3.0],
        [nan, 1.0, 2.0, 3.0], [1.0, 2.0, nan], [5.0, nan, 0.0, 0.0, 0.0, 0.0], [5.0, nan, -0.0, 1.0],
        [5.0, nan, 3.0, -2.0, -1.0, -0.5, 0.25, 4.0, 1.0], [5.0, nan, 3.0, -2.0, -1.0, -4.0, 2.0, 6.0, 6.0],
        [9.0, nan, 2.0, -1.0, -0.5, -0.25], [nan, nan, 8.0, nan, 4.0, -3.0, 10.0, -10.0],
        [nan, -2.0, 1.0, 1.5, -3.0, 0.5], [1.0, nan, 0.0, -0.0, 0.0, 2.0], [3.0, 1.0, nan, 7.0],
        [0.0, 0.0, nan, 0.0, 0.0, 0.0, 0.0])]
    big = rng.standard_normal(3000)
    big[1234] = 40.0
    big[2500] = -40.0
    vecs.append(big)
    big2 = rng.standard_normal(3000)
    big2[700] = nan
    big2[701] = 0.5
    big2[702:705] = [-0.4, -0.3, 0.2]
    vecs.append(big2)
    cases = []
    for v in vecs:
        cases.append((v.copy(), v.size, 1))
        if v.size >= 2:             # the same values at stride 3, other slots filled with larger noise
            buf = np.full(3 * (v.size - 1) + 1, 1e6)
            buf[::3] = v
            cases.append((buf, v.size, 3))
    cases.append((np.array([1.0, -7.0, 2.0]), 3, -1))     # negative increment: 0
    return cases


def gegen(R, M, N, lda, seed, dtype=np.float64):
    A = np.zeros((lda, N), dtype=dtype, order="F")
    (R.atlref_dgegen if dtype == np.float64 else R.atlref_sgegen)(M, N, A, lda, seed)
    return A


# (M, N, lda) cases of the LU fixtures; seeds follow xdlutst (M*N+lda)
LU_CASES = [(1, 1, 1), (2, 2, 2), (3, 5, 4), (5, 3, 7), (17, 17, 17), (64, 64, 64),
            (100, 100, 103), (37, 80, 40), (80, 37, 80), (129, 129, 130), (200, 200, 200),
            (257, 513, 260)]
# (N, lda) of the Cholesky fixtures; the SPD input is G G^T + N I from a
# gegen matrix G, built here once and stored
CHOL_CASES = [(1, 1), (2, 3), (3, 3), (4, 6), (5, 5), (7, 9), (17, 17), (64, 64), (100, 103),
              (129, 130), (200, 200)]
# (N, lda, bad): the CHOL_CASES input with A[bad, bad] = -1
CHOL_BAD = [(17, 17, 3), (100, 103, 57), (129, 130, 128), (64, 64, 0), (200, 200, 199)]
SYRK_CASES = [(121, 111, 37, 29), (122, 111, 37, 29), (121, 112, 20, 45), (122, 112, 20, 45),
              (122, 111, 64, 1)]
GEMM_CASES = [(111, 111, 37, 29, 41, 1.0, 0.0), (111, 112, 64, 64, 64, 1.0, 0.0),
              (112, 111, 33, 65, 17, -1.5, 0.5), (112, 112, 50, 20, 70, 0.75, -2.0),
              (111, 111, 128, 96, 1, 1.0, 1.0)]


def main():
    if not os.path.exists(REFLIB):
        sys.exit("build the reference routines first: sh oracle/ref_build.sh")
    R = load()
    out = {}
    seeds = np.array([0, 1, 7, 513 * 7 + 90, 12345, 65536 + 3, 8192 * 8192 + 8192, -5, 2**31 - 1],
                     dtype=np.int64)
    streams = []
    for s in seeds:
        R.atlref_srand(int(s))
        streams.append([R.atlref_rand() for _ in range(256)])
    out["rand_seeds"] = seeds
    out["rand_streams"] = np.array(streams, dtype=np.int64)
    out["gegen_7x3_lda9"] = gegen(R, 7, 3, 9, 7 * 3 + 9)
    out["sgegen_7x3_lda9"] = gegen(R, 7, 3, 9, 7 * 3 + 9, np.float32)

    out["lu_cases"] = np.array(LU_CASES, dtype=np.int64)
    for (M, N, lda) in LU_CASES:
        for order, tag in ((102, "C"), (101, "R")):
            rows = M if order == 102 else N
            cols = N if order == 102 else M
            ld = max(lda, rows)
            A = gegen(R, rows, cols, ld, M * N + lda)
            piv = np.zeros(max(min(M, N), 1), dtype=np.int32)
            info = R.atlref_dgetrf(order, M, N, A, ld, piv)
            key = f"lu{tag}_{M}x{N}_{lda}"
            out[key + "_ipiv"] = piv[: min(M, N)].copy()
            out[key + "_info"] = np.array(info)
            if rows * cols <= 130 * 130:
                out[key + "_lu"] = A[:rows, :cols].copy()
        As = gegen(R, M, N, max(lda, M), M * N + lda, np.float32)
        piv = np.zeros(max(min(M, N), 1), dtype=np.int32)
        info = R.atlref_sgetrf(102, M, N, As, max(lda, M), piv)
        out[f"sluC_{M}x{N}_{lda}_ipiv"] = piv[: min(M, N)].copy()
        out[f"sluC_{M}x{N}_{lda}_info"] = np.array(info)

    # singular matrices: a zero column (info = first zero pivot, 1-based)
    for (n, zc) in ((8, 3), (50, 0), (64, 63), (100, 70)):
        A = gegen(R, n, n, n, n * n + n)
        A[:, zc] = 0.0
        A0 = A.copy(order="F")
        piv = np.zeros(n, dtype=np.int32)
        info = R.atlref_dgetrf(102, n, n, A, n, piv)
        out[f"sing_{n}_{zc}_a"] = A0
        out[f"sing_{n}_{zc}_ipiv"] = piv
        out[f"sing_{n}_{zc}_info"] = np.array(info)
        out[f"sing_{n}_{zc}_lu"] = A.copy()

    # laswp forward and backward with a random pivot vector (ipiv[i] >= i)
    rng = np.random.default_rng(20260)
    for (m, n, k1, k2) in ((40, 70, 0, 40), (100, 33, 5, 77), (64, 64, 0, 64)):
        piv = np.array([rng.integers(i, m) for i in range(m)], dtype=np.int32)
        A = gegen(R, m, n, m, m * n)
        for inci in (1, -1):
            B = A.copy(order="F")
            R.atlref_dlaswp(n, B, m, k1, k2, piv, inci)
            out[f"laswp_{m}_{n}_{k1}_{k2}_{inci}"] = B
        out[f"laswp_{m}_{n}_{k1}_{k2}_piv"] = piv

    # getrs NoTrans / Trans on the factor of a 60x60 and a 129x129 matrix
    for n, nrhs in ((60, 3), (129, 5)):
        A = gegen(R, n, n, n, n * n + n)
        piv = np.zeros(n, dtype=np.int32)
        R.atlref_dgetrf(102, n, n, A, n, piv)
        for trans in (111, 112):
            B = gegen(R, n, nrhs, n, 77 + n)
            R.atlref_dgetrs(102, trans, n, nrhs, A, n, piv, B, n)
            out[f"getrs_{n}_{nrhs}_{trans}"] = B

    # reference-BLAS gemm (gemmtst seeds)
    out["gemm_cases"] = np.array(GEMM_CASES, dtype=np.float64)
    for (ta, tb, M, N, K, al, be) in GEMM_CASES:
        mA, nA = (M, K) if ta == 111 else (K, M)
        mB, nB = (K, N) if tb == 111 else (N, K)
        A = gegen(R, mA, nA, mA, mA * nA + 513 * 7 + 90)
        B = gegen(R, mB, nB, mB, mB * nB + 127 * 50 + 77)
        Cm = gegen(R, M, N, M, M * N + 101 * 2 + 53)
        R.atlref_dgemm(102, ta, tb, M, N, K, al, A, mA, B, mB, be, Cm, M)
        out[f"gemm_{ta}_{tb}_{M}_{N}_{K}"] = Cm

    # reference trsm, all 16 Side/Uplo/Trans/Diag cases, diagonally dominant A
    for side in (141, 142):
        for uplo in (121, 122):
            for ta in (111, 112):
                for diag in (131, 132):
                    M, N = 45, 38
                    na = M if side == 141 else N
                    A = gegen(R, na, na, na, na * na + 11)
                    A += np.eye(na) * na
                    B = gegen(R, M, N, M, M * N + 3)
                    R.atlref_dtrsm(102, side, uplo, ta, diag, M, N, 1.5, A, na, B, M)
                    out[f"trsm_{side}_{uplo}_{ta}_{diag}"] = B
    # reference-BLAS syrk through cblas_syrk's order mapping
    out["syrk_cases"] = np.array(SYRK_CASES, dtype=np.int64)
    for (uplo, tr, N, K) in SYRK_CASES:
        for order in (101, 102):
            nt = (tr == 111) == (order == 102)      # A stored with N rows
            lda, cols = (N, K) if nt else (K, N)
            A = gegen(R, lda, cols, lda, 99 + N + K)
            Cm = gegen(R, N, N, N, 5 + N)
            R.atlref_dsyrk(order, uplo, tr, N, K, 1.5, A, lda, 0.5, Cm, N)
            out[f"syrk_{order}_{uplo}_{tr}_{N}_{K}"] = Cm

    # Cholesky: ATL_potrf for both triangles and orders, then ATL_potrs
    out["chol_cases"] = np.array(CHOL_CASES, dtype=np.int64)
    for (n, lda) in CHOL_CASES:
        G = gegen(R, n, n, n, n * n + lda)
        A = np.full((lda, n), -2.56e9, order="F")
        A[:n, :n] = G @ G.T + n * np.eye(n)
        A[:n, :n] = 0.5 * (A[:n, :n] + A[:n, :n].T)
        out[f"chol_{n}_{lda}_a"] = A
        for uplo in (121, 122):
            for order in (101, 102):
                F = A.copy(order="F")
                info = R.atlref_dpotrf(order, uplo, n, F, lda)
                out[f"chol_{n}_{lda}_{uplo}_{order}_info"] = np.array(info)
                if n <= 130:
                    out[f"chol_{n}_{lda}_{uplo}_{order}_f"] = F
                    B = gegen(R, n, 3, n, 77 + n)
                    R.atlref_dpotrs(order, uplo, n, 3, F, lda, B, n)
                    out[f"chol_{n}_{lda}_{uplo}_{order}_x"] = B
        Fs = A.astype(np.float32, order="F")
        out[f"chol_{n}_{lda}_s_info"] = np.array(R.atlref_spotrf(102, 122, n, Fs, lda))
    # not positive definite: a negative diagonal entry (info = its 1-based index)
    out["chol_bad"] = np.array(CHOL_BAD, dtype=np.int64)
    for (n, lda, bad) in CHOL_BAD:
        A = out[f"chol_{n}_{lda}_a"].copy(order="F")
        A[bad, bad] = -1.0
        for uplo in (121, 122):
            F = A.copy(order="F")
            out[f"cholbad_{n}_{bad}_{uplo}_info"] = np.array(R.atlref_dpotrf(102, uplo, n, F, lda))
    # reference trmm, all 16 cases and both orders (M x N = 37 x 29)
    for order in (101, 102):
        for side in (141, 142):
            for uplo in (121, 122):
                for ta in (111, 112):
                    for diag in (131, 132):
                        M, N = 37, 29
                        na = M if side == 141 else N
                        rows, cols = (M, N) if order == 102 else (N, M)
                        A = gegen(R, na, na, na, na * na + 11)
                        A += np.eye(na) * na
                        B = gegen(R, rows, cols, rows, M * N + 3)
                        R.atlref_dtrmm(order, side, uplo, ta, diag, M, N, 1.5, A, na, B, rows)
                        out[f"trmm_{order}_{side}_{uplo}_{ta}_{diag}"] = B
    # reference gemv (M x N = 33 x 21) with positive and negative increments
    for order in (101, 102):
        for ta in (111, 112):
            for incx, incy in ((1, 1), (-2, 3), (2, -3)):
                M, N = 33, 21
                A = gegen(R, M, N, M, 7) if order == 102 else gegen(R, N, M, N, 7)
                lx, ly = (N, M) if ta == 111 else (M, N)
                x = gegen(R, lx * abs(incx), 1, lx * abs(incx), 8)[:, 0].copy()
                y = gegen(R, ly * abs(incy), 1, ly * abs(incy), 9)[:, 0].copy()
                R.atlref_dgemv(order, ta, M, N, 0.7, A, A.shape[0], x, incx, 0.3, y, incy)
                out[f"gemv_{order}_{ta}_{incx}_{incy}"] = y
    # reference trsv (N = 40) with unit and negative increments
    for order in (101, 102):
        for uplo in (121, 122):
            for ta in (111, 112):
                for diag in (131, 132):
                    for incx in (1, -2):
                        n = 40
                        A = gegen(R, n, n, n, 5)
                        A += np.eye(n) * n
                        x = gegen(R, n * abs(incx), 1, n * abs(incx), 6)[:, 0].copy()
                        R.atlref_dtrsv(order, uplo, ta, diag, n, A, n, x, incx)
                        out[f"trsv_{order}_{uplo}_{ta}_{diag}_{incx}"] = x
    # triangular inverse, both triangles, orders and diagonals
    for uplo in (121, 122):
        for order in (101, 102):
            for diag in (131, 132):
                for n in (1, 2, 3, 4, 5, 50):
                    T = gegen(R, n, n, n, 3 + n)
                    T += np.eye(n) * n
                    info = R.atlref_dtrtri(order, uplo, diag, n, T, n)
                    out[f"trtri_{uplo}_{order}_{diag}_{n}"] = T
                    out[f"trtri_{uplo}_{order}_{diag}_{n}_info"] = np.array(info)
    for (n, z) in ((10, 0), (50, 37), (130, 129)):
        T = gegen(R, n, n, n, 3 + n)
        T += np.eye(n) * n
        T[z, z] = 0.0
        out[f"trtri_sing_{n}_{z}_info"] = np.array(R.atlref_dtrtri(102, 121, 131, n, T, n))
    # inverse from the LU factors
    for n in (1, 2, 3, 5, 17, 64, 65, 100):
        for order in (101, 102):
            A = gegen(R, n, n, n, n * n + n)
            piv = np.zeros(n, dtype=np.int32)
            R.atlref_dgetrf(order, n, n, A, n, piv)
            out[f"getri_{n}_{order}_lu"] = A.copy()
            out[f"getri_{n}_{order}_piv"] = piv.copy()
            out[f"getri_{n}_{order}_info"] = np.array(R.atlref_dgetri(order, n, A, n, piv))
            out[f"getri_{n}_{order}_inv"] = A
    # cblas_i?amax (ATL_i?amax): ties, zeros, infinities and NaN runs, unit and strided
    R.atlref_cblas_idamax.argtypes = [I, dp, I]
    R.atlref_cblas_idamax.restype = I
    R.atlref_cblas_isamax.argtypes = [I, sp, I]
    R.atlref_cblas_isamax.restype = I
    for k, (x, n, inc) in enumerate(iamax_cases(np.random.default_rng(4242))):
        for pre, dt, f in (("d", np.float64, R.atlref_cblas_idamax), ("s", np.float32, R.atlref_cblas_isamax)):
            xx = np.asfortranarray(x.astype(dt))
            out[f"iamax_{pre}_{k}_x"] = xx
            out[f"iamax_{pre}_{k}_meta"] = np.array([n, inc, f(n, xx, inc)], dtype=np.int64)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


LARGE_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "atlas_ref_large.npz")
# headline sizes: column-major LU with the xdlutst seed n*n+lda (lda = n) and
# the plain dgesv's right-hand side gegen(n, 1, n+1); FP32 pivots at 4096
LARGE_LU = (2048, 4096, 8192)
LARGE_SLU = (4096,)
# DGEMM 1024^3 NoTrans/NoTrans, alpha 1, beta 0, gemmtst seeds
LARGE_GEMM = 1024
LARGE_GEMM_SAMPLES = 16384


def main_large():
    """Reference results at the headline sizes, too large for the main
    fixture file: the reference's own ATL_getrfC pivots (and the diagonal of U
    and the getrs solution) at n = 2048, 4096, 8192, FP32 pivots at 4096, and
    sampled entries and column 1-norms of the reference BLAS product at
    1024^3.  The n = 8192 factorization runs on the reference's triple-loop
    BLAS on one core: minutes."""
    if not os.path.exists(REFLIB):
        sys.exit("build the reference routines first: sh oracle/ref_build.sh <reference tree>")
    R = load()
    out = {}
    for n in LARGE_LU:
        A = gegen(R, n, n, n, n * n + n)
        piv = np.zeros(n, dtype=np.int32)
        info = R.atlref_dgetrf(102, n, n, A, n, piv)
        out[f"lu_{n}_ipiv"] = piv
        out[f"lu_{n}_info"] = np.array(info)
        out[f"lu_{n}_udiag"] = np.diag(A).copy()
        b = gegen(R, n, 1, n, n + 1)
        R.atlref_dgetrs(102, 111, n, 1, A, n, piv, b, n)
        out[f"lu_{n}_x"] = b[:, 0].copy()
        print("lu", n, "info", info, flush=True)
    for n in LARGE_SLU:
        A = gegen(R, n, n, n, n * n + n, np.float32)
        piv = np.zeros(n, dtype=np.int32)
        info = R.atlref_sgetrf(102, n, n, A, n, piv)
        out[f"slu_{n}_ipiv"] = piv
        out[f"slu_{n}_info"] = np.array(info)
        print("slu", n, "info", info, flush=True)
    n = LARGE_GEMM
    A = gegen(R, n, n, n, n * n + 513 * 7 + 90)
    B = gegen(R, n, n, n, n * n + 127 * 50 + 77)
    Cm = gegen(R, n, n, n, n * n + 101 * 2 + 53)
    R.atlref_dgemm(102, 111, 111, n, n, n, 1.0, A, n, B, n, 0.0, Cm, n)
    rng = np.random.default_rng(1024)
    idx = rng.integers(0, n * n, LARGE_GEMM_SAMPLES)
    out["gemm_1024_idx"] = idx.astype(np.int64)                    # column-major flat index
    out["gemm_1024_val"] = Cm.reshape(-1, order="F")[idx].copy()
    out["gemm_1024_colnrm1"] = np.abs(Cm).sum(axis=0)
    np.savez_compressed(LARGE_OUT, **out)
    print("wrote", LARGE_OUT, os.path.getsize(LARGE_OUT), "bytes")


if __name__ == "__main__":
    if "--large" in sys.argv[1:]:
        main_large()
    else:
        main()
