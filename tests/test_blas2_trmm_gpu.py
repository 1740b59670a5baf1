"""cblas_dtrmm / strmm, cblas_dgemv / sgemv and cblas_dtrsv / strsv through
the C ABI, against the reference-BLAS fixtures (trmm, gemv, trsv built from
the reference's basefiles) and the oracle: every Side/Uplo/Trans/Diag case,
both orders, lda gaps, negative increments."""
import ctypes as C
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ALL = list(itertools.product((141, 142), (121, 122), (111, 112), (131, 132)))


@pytest.mark.parametrize("side,uplo,ta,diag", ALL)
def test_dtrmm_matches_oracle(gb, ora, side, uplo, ta, diag):
    for (M, N, alpha) in ((45, 38, 1.5), (300, 131, -1.0), (64, 1, 1.0), (1, 70, 2.0), (257, 193, 0.5)):
        na = M if side == 141 else N
        A = ora.gegen(na, na, na * na + 11, lda=na + 1)
        B0 = ora.gegen(M, N, M * N + 3, lda=M + 2)
        Bg = B0.copy(order="F")
        gb.cblas_dtrmm(102, side, uplo, ta, diag, M, N, alpha, A, na + 1, Bg, M + 2)
        Bt = B0.copy(order="F")
        ora.lib().ora_dtrmm(side, uplo, ta, diag, M, N, alpha, A, na + 1, Bt, M + 2)
        assert np.abs(Bg[:M] - Bt[:M]).max() <= 1e-14 * na * (abs(alpha) + 1), (M, N)
        assert (Bg[M:] == -2.56e9).all()


def test_dtrmm_reference_fixtures(gb, ora, golden):
    for order in (101, 102):
        for (side, uplo, ta, diag) in ALL:
            M, N = 37, 29
            na = M if side == 141 else N
            rows, cols = (M, N) if order == 102 else (N, M)
            A = ora.gegen(na, na, na * na + 11)
            A += np.eye(na) * na
            B = ora.gegen(rows, cols, M * N + 3)
            gb.cblas_dtrmm(order, side, uplo, ta, diag, M, N, 1.5, A, na, B, rows)
            ref = golden[f"trmm_{order}_{side}_{uplo}_{ta}_{diag}"]
            assert np.abs(B - ref).max() <= 1e-12 * na, (order, side, uplo, ta, diag)


def test_dtrmm_large_equals_dense_product(gb, ora):
    # the triangular-operand GEMM skips k-tiles: compare with the dense
    # product of the explicit triangle at a size with many tiles
    M, N = 1000, 700
    A = ora.gegen(M, M, 5)
    B0 = ora.gegen(M, N, 6)
    for uplo, ta, diag in itertools.product((121, 122), (111, 112), (131, 132)):
        T = np.triu(A) if uplo == 121 else np.tril(A)
        if diag == 132:
            np.fill_diagonal(T, 1.0)
        op = T if ta == 111 else T.T
        Bg = B0.copy(order="F")
        gb.cblas_dtrmm(102, 141, uplo, ta, diag, M, N, 1.0, A, M, Bg, M)
        assert np.abs(Bg - op @ B0).max() <= 1e-13 * M, (uplo, ta, diag)
        Br = ora.gegen(N, M, 7)
        Bg = Br.copy(order="F")
        gb.cblas_dtrmm(102, 142, uplo, ta, diag, N, M, 1.0, A, M, Bg, N)
        assert np.abs(Bg - Br @ op).max() <= 1e-13 * M, (uplo, ta, diag)


def test_dtrmm_alpha_zero_and_cp_async_loader(gb, ora):
    M, N = 50, 40
    A = ora.gegen(M, M, 1)
    B = ora.gegen(M, N, 2)
    gb.cblas_dtrmm(102, 141, 121, 111, 131, M, N, 0.0, A, M, B, M)
    assert (B == 0).all()
    # an odd leading dimension keeps the GEMM off TMA (cp.async loader)
    A = ora.gegen(M, M, 3, lda=M + 1)
    B0 = ora.gegen(M, N, 4, lda=M + 1)
    Bg = B0.copy(order="F")
    lib = gb.lib()
    torch = pytest.importorskip("torch")
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(Bg.T)).cuda()
    assert lib.atlg_dtrmm_dev(141, 122, 112, 131, M, N, 1.0, C.c_void_p(dA.data_ptr()), M + 1,
                              C.c_void_p(dB.data_ptr()), M + 1, None) == 0
    torch.cuda.synchronize()
    got = dB.cpu().numpy().T
    Bt = B0.copy(order="F")
    ora.lib().ora_dtrmm(141, 122, 112, 131, M, N, 1.0, A, M + 1, Bt, M + 1)
    assert np.abs(got[:M] - Bt[:M]).max() <= 1e-13


def test_strmm(gb, ora):
    M, N = 150, 40
    A = ora.gegen(M, M, 9, dtype=np.float32)
    B0 = ora.gegen(M, N, 10, dtype=np.float32)
    Bg = B0.copy(order="F")
    gb.cblas_strmm(102, 141, 122, 111, 131, M, N, 1.0, A, M, Bg, M)
    Bt = B0.copy(order="F")
    ora.lib().ora_strmm(141, 122, 111, 131, M, N, 1.0, A, M, Bt, M)
    assert np.allclose(Bg, Bt, rtol=1e-4, atol=1e-4)


def test_dgemv_reference_fixtures(gb, ora, golden):
    for order in (101, 102):
        for ta in (111, 112):
            for incx, incy in ((1, 1), (-2, 3), (2, -3)):
                M, N = 33, 21
                A = ora.gegen(M, N, 7) if order == 102 else ora.gegen(N, M, 7)
                lx, ly = (N, M) if ta == 111 else (M, N)
                x = ora.gegen(lx * abs(incx), 1, 8)[:, 0].copy()
                y = ora.gegen(ly * abs(incy), 1, 9)[:, 0].copy()
                y0 = y.copy()
                gb.cblas_dgemv(order, ta, M, N, 0.7, A, A.shape[0], x, incx, 0.3, y, incy)
                assert np.abs(y - golden[f"gemv_{order}_{ta}_{incx}_{incy}"]).max() <= 1e-14 * lx
                if abs(incy) > 1:
                    mask = np.ones(len(y), bool)
                    mask[::abs(incy)] = False
                    assert np.array_equal(y[mask], y0[mask])


@pytest.mark.parametrize("order,ta", list(itertools.product((101, 102), (111, 112))))
def test_dgemv_matches_oracle(gb, ora, order, ta):
    for (M, N, alpha, beta) in ((1000, 700, 1.0, 0.0), (31, 2049, -0.5, 2.0), (4097, 5, 1.5, 1.0),
                                (300, 200, 0.0, 3.0)):
        A = ora.gegen(M, N, 7, lda=M + 3) if order == 102 else ora.gegen(N, M, 7, lda=N + 3)
        lx, ly = (N, M) if ta == 111 else (M, N)
        x = np.random.default_rng(1).uniform(-1, 1, lx)
        y0 = np.random.default_rng(2).uniform(-1, 1, ly)
        yg = y0.copy()
        gb.cblas_dgemv(order, ta, M, N, alpha, A, A.shape[0], x, 1, beta, yg, 1)
        yt = y0.copy()
        ora.gemv(ta, M, N, alpha, A, x, 1, beta, yt, 1, order=order)
        assert np.abs(yg - yt).max() <= 1e-14 * lx + 1e-15, (M, N)


def test_sgemv(gb, ora):
    M, N = 500, 300
    A = ora.gegen(M, N, 3, dtype=np.float32)
    x = np.ones(N, dtype=np.float32)
    y = np.zeros(M, dtype=np.float32)
    gb.cblas_sgemv(102, 111, M, N, 1.0, A, M, x, 1, 0.0, y, 1)
    assert np.allclose(y, A.astype(np.float64).sum(axis=1), rtol=1e-4, atol=1e-4)


def test_dtrsv_reference_fixtures(gb, ora, golden):
    for order in (101, 102):
        for uplo in (121, 122):
            for ta in (111, 112):
                for diag in (131, 132):
                    for incx in (1, -2):
                        n = 40
                        A = ora.gegen(n, n, 5)
                        A += np.eye(n) * n
                        x = ora.gegen(n * abs(incx), 1, 6)[:, 0].copy()
                        gb.cblas_dtrsv(order, uplo, ta, diag, n, A, n, x, incx)
                        ref = golden[f"trsv_{order}_{uplo}_{ta}_{diag}_{incx}"]
                        assert np.allclose(x, ref, rtol=1e-12, atol=1e-14), (order, uplo, ta, diag, incx)


@pytest.mark.parametrize("uplo,ta,diag", list(itertools.product((121, 122), (111, 112), (131, 132))))
def test_dtrsv_matches_oracle(gb, ora, uplo, ta, diag):
    for n in (1, 63, 64, 65, 1000, 3001):
        # off-diagonal entries scaled by 1/n keep the unit-diagonal solves bounded
        A = ora.gegen(n, n, n + 5, lda=n + 1)
        A[:n, :n] = A[:n, :n] / n + np.eye(n)
        x0 = np.random.default_rng(n).uniform(-1, 1, n)
        xg = x0.copy()
        gb.cblas_dtrsv(102, uplo, ta, diag, n, A, n + 1, xg, 1)
        xt = x0.copy()
        ora.trsv(uplo, ta, diag, n, A, xt, 1)
        assert np.abs(xg - xt).max() <= 1e-12 * max(1.0, np.abs(xt).max()), n


def test_strsv(gb, ora):
    n = 300
    A = ora.gegen(n, n, 2, dtype=np.float32)
    A += np.eye(n, dtype=np.float32) * n
    x0 = np.ones(n, dtype=np.float32)
    xg = x0.copy()
    gb.cblas_strsv(102, 122, 111, 131, n, A, n, xg, 1)
    xt = x0.copy()
    ora.trsv(122, 111, 131, n, A, xt, 1)
    assert np.allclose(xg, xt, rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("n", [1, 100, 128, 129, 1000, 2500])
@pytest.mark.parametrize("uplo,diag", [(122, 132), (121, 131)])
def test_strsv_chain_on_lu_factors(gb, n, uplo, diag):
    """The chained FP32 TRSV (block inverses prepared once, then solves)
    on the factors of a partial-pivoting LU: against an FP64 triangular solve
    of the same FP32 factors, to FP32 accuracy; two solves with one
    preparation give identical results."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    g = torch.Generator(device="cuda").manual_seed(n + uplo)
    A = torch.randn(n, n, device="cuda", dtype=torch.float64, generator=g)
    LU, _ = torch.linalg.lu_factor(A)
    T = LU.float()                                       # row-major n x n holding the factors
    Tcm = T.t().contiguous()                             # column-major storage
    ws = torch.empty(max(1, L.atlg_strsv_chain_ws(n) // 4), dtype=torch.float32, device="cuda")
    b = torch.randn(n, device="cuda", dtype=torch.float32, generator=g)
    x1, x2 = b.clone(), b.clone()
    torch.cuda.synchronize()
    assert L.atlg_strsv_chain_prepare_dev(uplo, diag, n, Tcm.data_ptr(), n, ws.data_ptr(), None) == 0
    assert L.atlg_strsv_chain_dev(uplo, n, Tcm.data_ptr(), n, ws.data_ptr(), x1.data_ptr(), None) == 0
    assert L.atlg_strsv_chain_dev(uplo, n, Tcm.data_ptr(), n, ws.data_ptr(), x2.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert L.atlg_status() == 0
    assert torch.equal(x1, x2)
    Td = T.double()
    if uplo == 122:
        Tt = torch.tril(Td, -1) + torch.eye(n, dtype=torch.float64, device="cuda")
    else:
        Tt = torch.triu(Td)
    ref = torch.linalg.solve_triangular(Tt, b.double().unsqueeze(1), upper=(uplo == 121),
                                        unitriangular=(diag == 132)).squeeze(1)
    err = float((x1.double() - ref).abs().max() / ref.abs().max())
    assert err < 2e-2, err       # FP32 forward error of a Gaussian matrix's factors (bugs give O(1))


def test_strsv_chain_rejects_bad_arguments(gb):
    L = gb.lib()
    assert L.atlg_strsv_chain_prepare_dev(122, 132, -1, None, 1, None, None) == -1
    assert L.atlg_strsv_chain_prepare_dev(123, 132, 10, None, 10, None, None) == -1
    assert L.atlg_strsv_chain_dev(122, 10, None, 5, None, None, None) == -1


@pytest.mark.parametrize("M,K,incx,beta", [(5000, 3000, 1, 0.5), (2048, 1024, 3, 0.0), (4097, 1500, 1, -1.0)])
def test_dgemv_large_tiled_form(gb, M, K, incx, beta):
    """NoTrans GEMV with M >= 2048 and K >= 1024 takes the tiled form (column
    tiles summed in a fixed order by a second kernel): against torch FP64,
    beta = 0 never reading y (NaN there stays out of the result), and the
    same bits on a repeated call."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    g = torch.Generator(device="cuda").manual_seed(M + K)
    A = torch.randn(K, M, device="cuda", dtype=torch.float64, generator=g)     # column-major M x K
    xs = torch.randn(K * incx, device="cuda", dtype=torch.float64, generator=g)
    y0 = torch.randn(M, device="cuda", dtype=torch.float64, generator=g)
    if beta == 0.0:
        y0[::7] = float("nan")
    outs = []
    for _ in range(2):
        y = y0.clone()
        torch.cuda.synchronize()
        assert L.atlg_dgemv_dev(111, M, K, 1.25, A.data_ptr(), M, xs.data_ptr(), incx, beta, y.data_ptr(), None) == 0
        torch.cuda.synchronize()
        outs.append(y)
    ref = 1.25 * (A.T @ xs[::incx]) + (beta * y0 if beta != 0.0 else 0.0)
    assert torch.isfinite(outs[0]).all()
    err = float((outs[0] - ref).abs().max() / ref.abs().max())
    assert err < 1e-13, err
    assert torch.equal(outs[0], outs[1])
