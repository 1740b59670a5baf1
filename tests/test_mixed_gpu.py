"""Mixed-precision dgesv (FP32 LU + FP64 iterative refinement, FP64
fallback) through the C ABI.  A = U diag(s) V^T with U, V from Householder QR
of seeded Gaussian matrices and s geometric from 1 to 1/kappa; b Gaussian.
Accuracy is measured against the FP64 oracle solve: normwise backward error
<= n*eps (double-double residual), forward error comparable to the FP64
LU's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_system(n, kappa, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.geomspace(1.0, 1.0 / kappa, n)
    A = np.asfortranarray((U * s) @ V.T)
    b = np.asfortranarray(rng.standard_normal((n, 1)))
    return A, b


@pytest.mark.parametrize("kappa,expect_fallback", [(1e2, False), (1e6, False), (1e10, True)])
def test_dgesv_mixed_accuracy(gb, ora, kappa, expect_fallback):
    n = 1024
    A, b = make_system(n, kappa, 20260 + int(np.log10(kappa)))
    A0 = A.copy(order="F")
    X = np.zeros((n, 1), order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    info, berr, ferr, iters, status = gb.dgesv_mixed(A, ipiv, b.copy(order="F"), X)
    assert info == 0
    assert status == (1 if expect_fallback else 0), (status, iters, berr)
    eps = np.finfo(float).eps
    be = ora.backward_error(A0, X[:, 0], b[:, 0])
    assert be <= n * eps, be
    assert abs(be - berr[0]) <= 1e-2 * be + 1e-18 or berr[0] <= n * eps
    # FP64 oracle solve for the forward-error comparison
    Ao = A0.copy(order="F")
    xo = b.copy(order="F")
    ora.lib().ora_dgesv(102, n, 1, Ao, n, np.zeros(n, dtype=np.int32), xo, n)
    fe_mixed = np.abs(X - xo).max() / np.abs(xo).max()
    assert fe_mixed <= max(1e3 * kappa * eps, 1e-12)
    if not expect_fallback:
        assert np.array_equal(A, A0)          # A untouched when refinement converged
        assert 1 <= iters <= 30


def test_dgesv_mixed_multiple_rhs(gb, ora):
    n, nrhs = 700, 4
    A, _ = make_system(n, 1e3, 5)
    rng = np.random.default_rng(9)
    B = np.asfortranarray(rng.standard_normal((n, nrhs)))
    X = np.zeros((n, nrhs), order="F")
    info, berr, ferr, iters, status = gb.dgesv_mixed(A.copy(order="F"), np.zeros(n, dtype=np.int32), B, X)
    assert info == 0 and status == 0 and berr.shape == (nrhs,)
    for j in range(nrhs):
        assert ora.backward_error(A, X[:, j], B[:, j]) <= n * np.finfo(float).eps


def test_dgesv_mixed_singular_reports_info(gb):
    n = 64
    A = np.asfortranarray(np.random.default_rng(1).standard_normal((n, n)))
    A[:, 5] = 0.0
    X = np.zeros((n, 1), order="F")
    b = np.ones((n, 1), order="F")
    info, berr, ferr, iters, status = gb.dgesv_mixed(A, np.zeros(n, dtype=np.int32), b, X)
    assert info == 6 and status == 2


def test_tf32x3_update_is_fp32_accurate(gb):
    """The mixed solver's factor update (3xTF32 on tcgen05) against an FP64
    product: error at FP32 level, far below single-pass TF32 (~1e-3)."""
    torch = pytest.importorskip("torch")
    # (384, 512, 96): every tile inside C (the epilogue without bounds tests)
    for (M, N, K) in ((1000, 700, 64), (513, 300, 200), (256, 128, 64), (384, 512, 96)):
        g = torch.Generator(device="cuda").manual_seed(M + N)
        A = torch.randn(K, M, device="cuda", generator=g)     # column-major M x K storage
        B = torch.randn(N, K, device="cuda", generator=g)     # column-major K x N storage
        C = torch.randn(N, M, device="cuda", generator=g)
        ref = C.double().T - (A.double().T @ B.double().T)
        gb.lib().atlg_sgemm_tf32x3_dev(M, N, K, -1.0, A.data_ptr(), M, B.data_ptr(), K, C.data_ptr(), M, None)
        torch.cuda.synchronize()
        # relative to the result's magnitude: FP32 rounding is 6e-8, the
        # 3xTF32 split adds ~2^-22; single-pass TF32 would be ~1e-3
        err = (C.double().T - ref).abs().max().item() / ref.abs().max().item()
        assert err < 1e-5, (M, N, K, err)
        assert gb.lib().atlg_status() == 0


@pytest.mark.parametrize("n", [1, 127, 129, 1000, 2049])
def test_dgesv_mixed_ragged_sizes(gb, ora, n):
    """Sizes that leave a partial 128-row block in the chained refinement
    solves (and the degenerate n = 1)."""
    A, b = make_system(n, 1e4, 300 + n)
    A0 = A.copy(order="F")
    X = np.zeros((n, 1), order="F")
    info, berr, ferr, iters, status = gb.dgesv_mixed(A, np.zeros(n, dtype=np.int32), b.copy(order="F"), X)
    assert info == 0 and status == 0, (status, iters)
    assert ora.backward_error(A0, X[:, 0], b[:, 0]) <= max(n, 16) * np.finfo(float).eps


def test_dgesv_mixed_n16384_kappa1e6(gb):
    """The mixed-precision configuration at its own size: n = 16384,
    kappa = 1e6, A = U diag(s) V^T (U, V from Householder QR of seeded
    Gaussian matrices on the GPU), b Gaussian.  The backward error is computed
    here from b - A x in FP64 on the untouched matrix (not the solver's
    estimate) and must be <= n eps; the forward error is compared with the
    plain FP64 LU solve of the same system."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    n, kappa = 16384, 1e6
    L = gb.lib()
    g = torch.Generator(device="cuda").manual_seed(16384)
    U, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g))
    V, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g))
    s = torch.logspace(0, -np.log10(kappa), n, device="cuda", dtype=torch.float64)
    Acm = ((U * s) @ V.T).t().contiguous()      # column-major storage of A
    del U, V
    Am = Acm.T                                   # the matrix
    b = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    A = Acm.clone()
    X = torch.zeros(n, device="cuda", dtype=torch.float64)
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    berr, ferr, it, stt = C.c_double(), C.c_double(), C.c_int(), C.c_int()
    torch.cuda.synchronize()
    info = L.atlg_dgesv_mixed_dev(n, 1, A.data_ptr(), n, piv.data_ptr(), b.data_ptr(), n, X.data_ptr(), n,
                                  C.byref(berr), C.byref(ferr), C.byref(it), C.byref(stt), None)
    torch.cuda.synchronize()
    assert info == 0 and stt.value == 0, (info, stt.value, it.value)
    assert 1 <= it.value <= 30
    assert torch.equal(A, Acm)                   # refinement converged: A untouched
    r = b - Am @ X
    be = float(r.abs().max() / (Am.abs().sum(dim=1).max() * X.abs().max() + b.abs().max()))
    assert be <= n * np.finfo(float).eps, be
    # plain FP64 LU solve of the same system
    inf = torch.zeros(4, dtype=torch.int32, device="cuda")
    A.copy_(Acm)
    xp = b.clone()
    torch.cuda.synchronize()
    L.atlg_dgetrf_dev(n, n, A.data_ptr(), n, piv.data_ptr(), inf.data_ptr(), None)
    L.atlg_dgetrs_dev(102, 111, n, 1, A.data_ptr(), n, piv.data_ptr(), xp.data_ptr(), n, None)
    torch.cuda.synchronize()
    fe = float((X - xp).abs().max() / xp.abs().max())
    assert fe <= 1e3 * kappa * np.finfo(float).eps, fe
    assert L.atlg_status() == 0


def _sgetrf_tc(gb, A0, defer_rows, fuse=1):
    """FP32 tensor-core factorization of A0 (float32, column-major) on the
    GPU with the given deferral threshold and panel fusion (both restored to
    their defaults after)."""
    torch = pytest.importorskip("torch")
    m, n = A0.shape
    L = gb.lib()
    A = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()      # column-major storage
    piv = torch.zeros(min(m, n), dtype=torch.int32, device="cuda")
    info = torch.zeros(4, dtype=torch.int32, device="cuda")
    L.atlg_lu_defer_rows(defer_rows)
    L.atlg_panel_fuse(fuse)
    try:
        torch.cuda.synchronize()
        assert L.atlg_sgetrf_tc_dev(m, n, A.data_ptr(), m, piv.data_ptr(), info.data_ptr(), None) == 0
        torch.cuda.synchronize()
    finally:
        L.atlg_lu_defer_rows(-1)
        L.atlg_panel_fuse(1)
    assert L.atlg_status() == 0
    return A.cpu().numpy().T, piv.cpu().numpy(), int(info[0])


@pytest.mark.parametrize("m,n,defer_rows,fuse", [(2048, 2048, 256, 1), (1500, 1700, 320, 1), (1700, 1500, 256, 1),
                                                 (2048, 2048, 0, 1), (2048, 2048, 0, 0), (1700, 1500, 0, 1),
                                                 (1500, 1700, 0, 0), (3000, 3000, 1024, 1)])
def test_sgetrf_tc_paired_updates(gb, ora, m, n, defer_rows, fuse):
    """The mixed solver's FP32 factorization with every other far update
    deferred into the next step's rank-128 update (threshold lowered so that
    small matrices pair steps; 0 = never), and with the next panel applying a
    step's update of its columns itself (fuse 1) or not: partial pivoting
    holds (|l_ij| <= 1 below the diagonal) and the scaled residual
    ||P A - L U||_1 / (k ||A||_1 eps32) stays within the LU tester's 100."""
    A0 = ora.gegen(m, n, 4242 + m + n, dtype=np.float32)
    F, piv, info = _sgetrf_tc(gb, A0, defer_rows, fuse)
    assert info == 0
    k = min(m, n)
    assert np.all(piv >= np.arange(k)) and np.all(piv < m)
    Lf = np.tril(F[:, :k].astype(np.float64), -1) + np.eye(m, k)
    Uf = np.triu(F[:k, :].astype(np.float64))
    assert np.abs(Lf).max() <= 1.0
    PA = A0.astype(np.float64)
    for i in range(k):
        if piv[i] != i:
            PA[[i, piv[i]]] = PA[[piv[i], i]]
    R = PA - Lf @ Uf
    resid = np.abs(R).sum(axis=0).max() / (k * np.abs(A0.astype(np.float64)).sum(axis=0).max() *
                                           np.finfo(np.float32).eps)
    assert resid <= 100.0, resid


def test_dgesv_mixed_paired_updates_converge(gb, ora):
    """The mixed solve with the factorization's steps paired down to 256 rows,
    and with the next-panel updates in the panel kernel or not: refinement
    converges to the FP64 backward error as with unpaired, separate steps."""
    n = 2049
    L = gb.lib()
    out = {}
    for rows, fuse in ((256, 1), (0, 1), (0, 0)):
        A, b = make_system(n, 1e4, 77)
        A0 = A.copy(order="F")
        X = np.zeros((n, 1), order="F")
        L.atlg_lu_defer_rows(rows)
        L.atlg_panel_fuse(fuse)
        try:
            info, berr, ferr, iters, status = gb.dgesv_mixed(A, np.zeros(n, dtype=np.int32), b.copy(order="F"), X)
        finally:
            L.atlg_lu_defer_rows(-1)
            L.atlg_panel_fuse(1)
        assert info == 0 and status == 0, (rows, fuse, status, iters)
        assert ora.backward_error(A0, X[:, 0], b[:, 0]) <= n * np.finfo(float).eps
        out[(rows, fuse)] = iters
    assert max(out.values()) <= min(out.values()) + 2, out


def _dlag2s_cases():
    rng = np.random.default_rng(5)
    parts = [rng.integers(0, 2**64, size=60000, dtype=np.uint64)]          # the whole double range, NaNs included
    # exponents around the float range, random mantissas, and exact ties
    # (the 29 bits dropped equal half a float ulp) with odd and even kept bits
    e = rng.integers(1023 - 160, 1023 + 130, size=60000).astype(np.uint64)
    m = rng.integers(0, 2**52, size=60000, dtype=np.uint64)
    s = rng.integers(0, 2, size=60000).astype(np.uint64) << np.uint64(63)
    parts.append(s | (e << np.uint64(52)) | m)
    mt = (m & ~np.uint64(0x1FFFFFFF)) | np.uint64(0x10000000)
    parts.append(s | (e << np.uint64(52)) | mt)
    f32max = float(np.finfo(np.float32).max)
    sub = 2.0 ** -149
    special = [0.0, -0.0, 5e-324, 2.0 ** -1022, sub, sub / 2, sub * 1.5, sub * 2.5, sub * 0.75, sub * 0.5000001,
               2.0 ** -126, 2.0 ** -126 - sub / 2, 2.0 ** -126 - sub, 1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24,
               1.0 + 2.0 ** -24 + 2.0 ** -52, f32max, f32max + 2.0 ** 103, f32max + 2.0 ** 103 - 2.0 ** 75,
               2.0 ** 128, 1e300, np.inf, -np.inf, -f32max, np.nan, -1.0 / 3.0, np.pi]
    parts.append(np.array(special, dtype=np.float64).view(np.uint64))
    return np.concatenate(parts).view(np.float64)


def test_dlag2s_rounds_to_nearest_even(gb):
    """atlg_dlag2s_dev, the mixed solver's FP64 -> FP32 copy (IEEE round to
    nearest even in integer arithmetic), against the host's conversion bit
    for bit: random bit patterns over the whole double range, random values
    and exact ties around the float range, the float subnormal range, the
    FLT_MAX rounding boundary, zeros and infinities; NaN stays NaN.  Returns 1
    when some |a| exceeds FLT_MAX, 0 otherwise; padding rows untouched."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    x = _dlag2s_cases()
    M, lda, ldsa = 997, 1000, 1003
    N = (x.size + M - 1) // M
    A = np.zeros((lda, N))
    flat = np.zeros(M * N)
    flat[:x.size] = x
    A[:M, :] = flat.reshape(N, M).T
    Ad = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    Sd = torch.full((N, ldsa), 7.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    assert L.atlg_dlag2s_dev(M, N, Ad.data_ptr(), lda, Sd.data_ptr(), ldsa, None) == 1
    S = Sd.cpu().numpy().T
    with np.errstate(over="ignore", invalid="ignore"):
        want = A[:M, :].astype(np.float32)
    got = S[:M, :]
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan)
    assert np.array_equal(got[~nan].view(np.uint32), want[~nan].view(np.uint32))
    assert np.all(S[M:, :] == 7.0)
    # in range: no overflow reported
    B = np.asfortranarray(np.random.default_rng(1).standard_normal((300, 200)))
    Bd = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    Td = torch.zeros((200, 300), dtype=torch.float32, device="cuda")
    assert L.atlg_dlag2s_dev(300, 200, Bd.data_ptr(), 300, Td.data_ptr(), 300, None) == 0
    assert np.array_equal(Td.cpu().numpy().T, B.astype(np.float32))
    assert L.atlg_dlag2s_dev(-1, 2, Bd.data_ptr(), 300, Td.data_ptr(), 300, None) == -1
