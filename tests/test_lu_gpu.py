"""LU path through the C ABI: clapack_dgetrf pivots bit-exact with the
reference (fixtures from its own getrfC/getrfR) and with the oracle, the
xdlutst residual (AtlasBase/Clint/atlas-tlp.base:1992-2058, threshold 100,
:2203), zero-pivot info, getrs/gesv against the oracle (xdslvtst residual,
threshold 100) and the full 8192 factorization."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
LU_THRESH = 100.0


@pytest.mark.parametrize("order", ["C", "R"])
def test_dgetrf_pivots_match_reference_fixtures(gb, ora, golden, order):
    for (M, N, lda) in golden["lu_cases"]:
        M, N, lda = int(M), int(N), int(lda)
        key = f"lu{order}_{M}x{N}_{lda}"
        rows, cols = (M, N) if order == "C" else (N, M)
        ld = max(lda, rows)
        A = ora.gegen(rows, cols, M * N + lda, lda=ld)
        ipiv = np.zeros(max(min(M, N), 1), dtype=np.int32)
        info = gb.clapack_dgetrf(102 if order == "C" else 101, M, N, A, ld, ipiv)
        assert info == int(golden[key + "_info"]), key
        assert np.array_equal(ipiv[: min(M, N)], golden[key + "_ipiv"]), key
        if key + "_lu" in golden:
            assert np.allclose(A[:rows, :cols], golden[key + "_lu"], rtol=0, atol=1e-11 * max(M, N)), key
        if ld > rows:
            assert (A[rows:, :] == -2.56e9).all()


@pytest.mark.parametrize("n", [2048, 4096, 8192])
def test_dgetrf_pivots_match_reference_at_headline_sizes(gb, ora, golden_large, n):
    """clapack_dgetrf on the xdlutst-seeded n x n matrix against the
    reference's own ATL_getrfC run on the same input (fixture): pivots bit
    for bit, the diagonal of U to rounding, and the dgetrs solution of the
    plain dgesv's right-hand side gegen(n, 1, n+1) against the reference's
    ATL_getrs."""
    A = ora.gegen(n, n, n * n + n)
    ipiv = np.zeros(n, dtype=np.int32)
    info = gb.clapack_dgetrf(102, n, n, A, n, ipiv)
    assert info == int(golden_large[f"lu_{n}_info"])
    ref = golden_large[f"lu_{n}_ipiv"]
    mism = np.nonzero(ipiv != ref)[0]
    assert mism.size == 0, f"pivot mismatch with the reference at columns {mism[:10]}"
    ud = golden_large[f"lu_{n}_udiag"]
    assert np.max(np.abs(np.diag(A) - ud)) <= 1e-9 * np.max(np.abs(ud))
    x = ora.gegen(n, 1, n + 1)
    gb.clapack_dgetrs(102, 111, n, 1, A, n, ipiv, x, n)
    xr = golden_large[f"lu_{n}_x"]
    assert np.linalg.norm(x[:, 0] - xr) <= 1e-8 * np.linalg.norm(xr)


def test_sgetrf_pivots_match_reference_at_4096(gb, ora, golden_large):
    """clapack_sgetrf (the reference semantics of the mixed solver's FP32
    factor) against the reference's own FP32 ATL_getrfC at n = 4096."""
    n = 4096
    A = ora.gegen(n, n, n * n + n, dtype=np.float32)
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_sgetrf(102, n, n, A, n, ipiv) == int(golden_large[f"slu_{n}_info"])
    mism = np.nonzero(ipiv != golden_large[f"slu_{n}_ipiv"])[0]
    assert mism.size == 0, f"pivot mismatch with the reference at columns {mism[:10]}"


@pytest.mark.parametrize("M,N,lda", [(500, 500, 500), (1000, 1000, 1001), (1537, 700, 1540), (300, 900, 300),
                                     (2048, 2048, 2048)])
def test_dgetrf_matches_oracle_and_residual(gb, ora, M, N, lda):
    seed = M * N + lda
    A = ora.gegen(M, N, seed, lda=lda)
    Ao = A.copy(order="F")
    ipiv = np.zeros(min(M, N), dtype=np.int32)
    info = gb.clapack_dgetrf(102, M, N, A, lda, ipiv)
    oinfo, opiv = ora.getrf(Ao, M, N)
    assert info == 0 and oinfo == 0
    assert np.array_equal(ipiv, opiv)
    r = ora.lu_resid(M, N, A, ipiv, seed)
    assert r <= LU_THRESH, r
    assert np.abs(A[:M] - Ao[:M]).max() < 1e-9


def test_dgetrf_singular_info(gb, ora, golden):
    for (n, zc) in ((8, 3), (50, 0), (64, 63), (100, 70)):
        A = np.asfortranarray(golden[f"sing_{n}_{zc}_a"].copy())
        ipiv = np.zeros(n, dtype=np.int32)
        info = gb.clapack_dgetrf(102, n, n, A, n, ipiv)
        assert info == int(golden[f"sing_{n}_{zc}_info"])
        assert np.array_equal(ipiv, golden[f"sing_{n}_{zc}_ipiv"])


def test_sgetrf_pivots(gb, ora, golden):
    for (M, N, lda) in golden["lu_cases"]:
        M, N, lda = int(M), int(N), int(lda)
        A = ora.gegen(M, N, M * N + lda, lda=max(lda, M), dtype=np.float32)
        ipiv = np.zeros(max(min(M, N), 1), dtype=np.int32)
        info = gb.clapack_sgetrf(102, M, N, A, max(lda, M), ipiv)
        assert info == int(golden[f"sluC_{M}x{N}_{lda}_info"])
        assert np.array_equal(ipiv[: min(M, N)], golden[f"sluC_{M}x{N}_{lda}_ipiv"])


@pytest.mark.parametrize("n,nrhs", [(700, 16), (1000, 64), (4096, 8)])
@pytest.mark.parametrize("trans", [111, 112])
def test_dgetrs_many_rhs_block_inverses(gb, ora, n, nrhs, trans):
    """ColMajor getrs with 8 or more right-hand sides applies 64 x 64
    diagonal-block inverses (formed once per triangle) instead of the
    substitution kernel: against the oracle's getrs to 1e-9, ragged last
    block included (700, 1000)."""
    A = ora.gegen(n, n, n * n + n)
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgetrf(102, n, n, A, n, ipiv) == 0
    B0 = ora.gegen(n, nrhs, 31 + nrhs, lda=n + 5)
    Bg = B0.copy(order="F")
    gb.clapack_dgetrs(102, trans, n, nrhs, A, n, ipiv, Bg, n + 5)
    Bo = B0.copy(order="F")
    ora.lib().ora_dgetrs(102, trans, n, nrhs, A, n, ipiv, Bo, n + 5)
    assert np.allclose(Bg[:n], Bo[:n], rtol=1e-9, atol=1e-9)
    assert (Bg[n:] == B0[n:]).all()


@pytest.mark.parametrize("order", [102, 101])
@pytest.mark.parametrize("trans", [111, 112])
def test_dgetrs_matches_oracle(gb, ora, order, trans):
    n, nrhs = 333, 7
    A = ora.gegen(n, n, n * n + n)
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgetrf(order, n, n, A, n, ipiv) == 0
    B0 = ora.gegen(n, nrhs, 99, lda=n + 3)
    Bg = B0.copy(order="F")
    gb.clapack_dgetrs(order, trans, n, nrhs, A, n, ipiv, Bg, n + 3)
    Bo = B0.copy(order="F")
    ora.lib().ora_dgetrs(order, trans, n, nrhs, A, n, ipiv, Bo, n + 3)
    assert np.allclose(Bg[:n], Bo[:n], rtol=1e-9, atol=1e-9)


def test_dgetrs_reference_fixtures(gb, ora, golden):
    for n, nrhs in ((60, 3), (129, 5)):
        A = ora.gegen(n, n, n * n + n)
        ipiv = np.zeros(n, dtype=np.int32)
        gb.clapack_dgetrf(102, n, n, A, n, ipiv)
        for trans in (111, 112):
            B = ora.gegen(n, nrhs, 77 + n)
            gb.clapack_dgetrs(102, trans, n, nrhs, A, n, ipiv, B, n)
            assert np.allclose(B, golden[f"getrs_{n}_{nrhs}_{trans}"], rtol=1e-10, atol=1e-10)


def test_dgesv_slvtst_residual(gb, ora):
    # xdslvtst: X known, B = A X, solve, ||X - Xc||_inf/(N eps ||A||_1 ||Xc||_inf) <= 100
    n, nrhs = 1000, 3
    A = ora.gegen(n, n, n * n + n)
    X = ora.gegen(n, nrhs, 1234)
    B = np.asfortranarray(A @ X)
    A0 = A.copy(order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgesv(102, n, nrhs, A, n, ipiv, B, n) == 0
    r = ora.lib().ora_dslv_resid(n, nrhs, A0, n, B, n, X, n)
    assert r <= LU_THRESH, r


def test_dgesv_singular_skips_solve(gb, ora):
    n = 64
    A = ora.gegen(n, n, 3)
    A[:, 10] = 0.0
    B = ora.gegen(n, 2, 4)
    B0 = B.copy()
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgesv(102, n, 2, A, n, ipiv, B, n) == 11
    assert np.array_equal(B, B0)


def test_dgetrf_full_size_8192(gb, ora):
    """The headline factorization: n=8192, xdlutst seed; pivots bit-exact with
    the oracle and the residual (computed with torch fp64 on the GPU as a
    checker) within the tester threshold."""
    torch = pytest.importorskip("torch")
    n = 8192
    seed = n * n + n
    A = ora.gegen(n, n, seed)
    ipiv = np.zeros(n, dtype=np.int32)
    info = gb.clapack_dgetrf(102, n, n, A, n, ipiv)
    assert info == 0
    ora.set_threads(0)
    Ao = ora.gegen(n, n, seed)
    oinfo, opiv = ora.getrf(Ao)
    mism = np.nonzero(ipiv != opiv)[0]
    assert mism.size == 0, f"pivot mismatch at columns {mism[:10]}"
    LU = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().T        # column-major view
    L = torch.tril(LU, -1) + torch.eye(n, dtype=torch.float64, device="cuda")
    U = torch.triu(LU)
    A0 = ora.gegen(n, n, seed)
    ora.laswp(n, A0, 0, n, ipiv, 1)
    PA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda().T
    D = PA - L @ U
    normA = float(torch.from_numpy(np.ascontiguousarray(ora.gegen(n, n, seed).T)).abs().sum(dim=1).max())
    resid = float(D.abs().sum(dim=0).max()) / (normA * np.finfo(float).eps * n)
    assert resid <= LU_THRESH, resid


@pytest.mark.parametrize("n", [1, 63, 64, 65, 1000, 3001])
@pytest.mark.parametrize("trans", [111, 112])
def test_dgetrs_one_rhs_lookback_trsv(gb, ora, n, trans):
    """One right-hand side takes the single-launch look-back triangular
    solves; edge sizes around the 64-row block."""
    A = ora.gegen(n, n, n * n + n)
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgetrf(102, n, n, A, n, ipiv) == 0
    b0 = ora.gegen(n, 1, 5 + n)
    bg = b0.copy(order="F")
    gb.clapack_dgetrs(102, trans, n, 1, A, n, ipiv, bg, n)
    bo = b0.copy(order="F")
    ora.lib().ora_dgetrs(102, trans, n, 1, A, n, ipiv, bo, n)
    assert np.allclose(bg, bo, rtol=1e-9, atol=1e-9 * np.abs(bo).max())
    assert gb.status() == 0


def test_dgetrf_sizes_in_sequence(gb):
    """A smaller factorization followed by larger ones in one process: the
    panel's candidate records are reused across columns and calls, and every
    pivot must still satisfy ipiv[j] >= j with a small LU residual."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    L = gb.lib()
    eps = np.finfo(float).eps
    n1 = lambda Z: float(Z.abs().sum(dim=0).max())
    for n in (4096, 6144, 2048, 8192):
        g = torch.Generator(device="cuda").manual_seed(13)
        A0 = torch.rand(n, n, device="cuda", dtype=torch.float64, generator=g) - 0.5
        A = A0.clone()
        piv = torch.zeros(n, dtype=torch.int32, device="cuda")
        info = torch.zeros(4, dtype=torch.int32, device="cuda")
        # the library stream does not wait for torch's stream
        torch.cuda.synchronize()
        L.atlg_dgetrf_dev(n, n, C.c_void_p(A.data_ptr()), n, C.c_void_p(piv.data_ptr()),
                          C.c_void_p(info.data_ptr()), None)
        torch.cuda.synchronize()
        assert int(info[0]) == 0 and gb.status() == 0
        p = piv.cpu().numpy()
        assert (p >= np.arange(n)).all() and (p < n).all(), n
        perm = np.arange(n)
        for i in range(n):
            perm[[i, p[i]]] = perm[[p[i], i]]
        F = A.T
        Lm = torch.tril(F, -1) + torch.eye(n, device="cuda", dtype=torch.float64)
        resid = n1(A0.T[torch.from_numpy(perm).cuda()] - Lm @ torch.triu(F)) / (n1(A0.T) * n * eps)
        assert resid <= 1.0, (n, resid)
        del A, A0, Lm, F
        torch.cuda.empty_cache()


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_cluster_panel_matches_grid_panel(gb, ora, dtype):
    """The cluster panel (distributed shared memory, hardware cluster barrier)
    and the cooperative-grid panel do the same arithmetic: bit-identical
    pivots and factors, for panels on both sides of the cluster's capacity
    (panels too tall for the cluster stay on the grid: the two-half split is
    switched off here)."""
    L = gb.lib()
    sizes = (700, 3000, 7100) if dtype == np.float64 else (700, 5000, 15000)
    L.atlg_panel_split(0)
    try:
        for n in sizes:
            A0 = ora.gegen(n, n, n * n + n, dtype=dtype)
            out = []
            for on in (1, 0):
                L.atlg_panel_cluster(on)
                A = A0.copy(order="F")
                piv = np.zeros(n, dtype=np.int32)
                f = gb.clapack_dgetrf if dtype == np.float64 else gb.clapack_sgetrf
                assert f(102, n, n, A, n, piv) == 0
                out.append((A, piv))
            assert np.array_equal(out[0][1], out[1][1]), n
            assert np.array_equal(out[0][0], out[1][0]), n
    finally:
        L.atlg_panel_cluster(1)
        L.atlg_panel_split(1)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_split_panel_matches_grid_panel(gb, ora, dtype):
    """Panels too tall for one cluster at 64 columns but not at 32 (FP64 above
    6816 rows, FP32 above 13248) run as two cluster halves: left half, its
    interchanges, triangular solve and update of the right half, right half,
    and one permutation record for the whole panel.  Against the grid panel
    (one launch per panel): the same pivots in FP64 (in FP32 the rounding
    differences of the two orders of operations flip near-ties in some
    column, after which the pivot sequences part: there every multiplier
    |l_ij| <= 1, the partial-pivoting property, is checked instead), and an
    LU residual |A(perm) - L U|_1 / (|A|_1 n eps) below 1 for both."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    n = 7100 if dtype == np.float64 else 14000
    eps = float(np.finfo(dtype).eps)
    A0 = ora.gegen(n, n, n * n + n, dtype=dtype)
    f = gb.clapack_dgetrf if dtype == np.float64 else gb.clapack_sgetrf
    out = []
    try:
        for on in (1, 0):
            L.atlg_panel_split(on)
            A = A0.copy(order="F")
            piv = np.zeros(n, dtype=np.int32)
            assert f(102, n, n, A, n, piv) == 0
            out.append((A, piv))
    finally:
        L.atlg_panel_split(1)
    if dtype == np.float64:
        assert np.array_equal(out[0][1], out[1][1])
    else:
        for F_np, p in out:
            assert (p >= np.arange(n)).all() and (p < n).all()
            assert float(np.abs(np.tril(F_np, -1)).max()) <= 1.0
    n1 = lambda Z: float(Z.abs().sum(dim=0).max())
    Ad = torch.from_numpy(np.asfortranarray(A0).astype(np.float64).T.copy()).cuda().T
    for F_np, p in out:
        perm = np.arange(n)
        for i in range(n):
            perm[[i, p[i]]] = perm[[p[i], i]]
        F = torch.from_numpy(F_np.astype(np.float64).T.copy()).cuda().T
        Lm = torch.tril(F, -1) + torch.eye(n, device="cuda", dtype=torch.float64)
        resid = n1(Ad[torch.from_numpy(perm).cuda()] - Lm @ torch.triu(F)) / (n1(Ad) * n * eps)
        assert resid <= 1.0, resid
        del F, Lm
    torch.cuda.empty_cache()


@pytest.mark.parametrize("m,n", [(64, 2000), (40, 517)])
def test_sgetrf_block_row_solve_matches_strsm(gb, ora, m, n):
    """The LU's solve for its top block row, U12 = inv(L11) A12 (FP32: a
    thread per column, the column in registers), gives the same bits as
    cblas_strsm (a warp per column) on the same operands.  With M <= 64 the
    factorization is one panel, its interchanges on A12 and this solve."""
    A0 = ora.gegen(m, n, 77 + n, dtype=np.float32)
    F = A0.copy(order="F")
    piv = np.zeros(m, dtype=np.int32)
    assert gb.clapack_sgetrf(102, m, n, F, m, piv) == 0
    B = np.asfortranarray(A0[:, m:])
    for i in range(m):
        B[[i, piv[i]]] = B[[piv[i], i]]
    L11 = np.asfortranarray(F[:, :m])
    gb.cblas_strsm(102, 141, 122, 111, 132, m, n - m, 1.0, L11, m, B, m)
    assert np.array_equal(B, F[:, m:])
