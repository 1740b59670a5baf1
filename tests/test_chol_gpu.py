"""SYRK and the Cholesky path (cblas_dsyrk, clapack_dpotrf / dpotrs / dposv
and the single-precision variants) through the C ABI, against the reference
fixtures (ATL_potrf / ATL_potrs / reference-BLAS syrk built from the
reference's basefiles) and the oracle.  Info indices are compared exactly;
factors and solutions to rounding, scaled by the problem size."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def spd(n, seed, lda=None, dtype=np.float64):
    """G G^T + n I for a seeded uniform G; the lda gap holds -2.56e9."""
    lda = n if lda is None else lda
    G = np.asfortranarray(np.random.default_rng(seed).uniform(-0.5, 0.5, (n, n)))
    A = np.full((lda, n), -2.56e9, order="F")
    S = G @ G.T + n * np.eye(n)
    A[:n, :n] = 0.5 * (S + S.T)
    return A.astype(dtype, order="F")


@pytest.mark.parametrize("order,uplo,trans", list(itertools.product((101, 102), (121, 122), (111, 112))))
def test_dsyrk_matches_oracle(gb, ora, order, uplo, trans):
    for (N, K, alpha, beta) in ((37, 29, 1.5, 0.5), (300, 130, -1.0, 1.0), (129, 1, 2.0, 0.0),
                                (65, 700, 1.0, -2.0)):
        nt = (trans == 111) == (order == 102)
        rows, cols = (N, K) if nt else (K, N)
        A = ora.gegen(rows, cols, 99 + N + K, lda=rows + 3)
        C0 = ora.gegen(N, N, 5 + N, lda=N + 1)
        Cg = C0.copy(order="F")
        gb.cblas_dsyrk(order, uplo, trans, N, K, alpha, A, rows + 3, beta, Cg, N + 1)
        Ct = C0.copy(order="F")
        ora.syrk(uplo, trans, N, K, alpha, A, beta, Ct, order=order)
        tol = 1e-15 * K * 4 * (abs(alpha) + 1) + 1e-14
        assert np.abs(Cg[:N] - Ct[:N]).max() <= tol, (N, K)
        # the other triangle and the ldc gap are left as they were
        eff_upper = (uplo == 121) == (order == 102)
        other = np.tril_indices(N, -1) if eff_upper else np.triu_indices(N, 1)
        assert np.array_equal(Cg[:N][other], C0[:N][other])
        assert (Cg[N:] == C0[N:]).all()


def test_dsyrk_reference_fixtures(gb, ora, golden):
    for (uplo, tr, N, K) in golden["syrk_cases"]:
        uplo, tr, N, K = int(uplo), int(tr), int(N), int(K)
        for order in (101, 102):
            nt = (tr == 111) == (order == 102)
            lda, cols = (N, K) if nt else (K, N)
            A = ora.gegen(lda, cols, 99 + N + K)
            Cm = ora.gegen(N, N, 5 + N)
            gb.cblas_dsyrk(order, uplo, tr, N, K, 1.5, A, lda, 0.5, Cm, N)
            ref = golden[f"syrk_{order}_{uplo}_{tr}_{N}_{K}"]
            assert np.abs(Cm - ref).max() <= 1e-14 * K + 1e-15, (order, uplo, tr)


def test_dsyrk_alpha_zero_scales_triangle(gb, ora):
    N = 70
    A = ora.gegen(N, 5, 1)
    C0 = ora.gegen(N, N, 2)
    for beta in (0.0, 3.0):
        Cg = C0.copy(order="F")
        gb.cblas_dsyrk(102, 122, 111, N, 5, 0.0, A, N, beta, Cg, N)
        low = np.tril_indices(N)
        assert np.array_equal(Cg[low], beta * C0[low])
        assert np.array_equal(Cg[np.triu_indices(N, 1)], C0[np.triu_indices(N, 1)])


@pytest.mark.parametrize("order", [101, 102])
def test_dgemm_a_at_takes_the_syrk_shortcut(gb, ora, order):
    # cblas_dgemm with B == A, TA != TB, beta == 0 is a SYRK plus a mirror;
    # the result is exactly symmetric and equals the GEMM to rounding
    M, K = 200, 90
    A = ora.gegen(M, K, 17)
    for ta, tb in ((111, 112), (112, 111)):
        if order == 102:
            lda = M if ta == 111 else K
            X = A if ta == 111 else np.asfortranarray(A.T)
        else:
            lda = K if ta == 111 else M
            X = np.asfortranarray(A.T) if ta == 111 else A
        Cg = np.full((M, M), 7.0, order="F")
        gb.cblas_dgemm(order, ta, tb, M, M, K, 1.25, X, lda, X, lda, 0.0, Cg, M)
        ref = 1.25 * (A @ A.T)
        assert np.array_equal(Cg, Cg.T)
        assert np.abs(Cg - ref).max() <= 1e-13 * K


@pytest.mark.parametrize("uplo,order", list(itertools.product((121, 122), (101, 102))))
def test_dpotrf_dpotrs_reference_fixtures(gb, ora, golden, uplo, order):
    for (n, lda) in golden["chol_cases"]:
        n, lda = int(n), int(lda)
        key = f"chol_{n}_{lda}_{uplo}_{order}"
        F = golden[f"chol_{n}_{lda}_a"].copy(order="F")
        info = gb.clapack_dpotrf(order, uplo, n, F, lda)
        assert info == int(golden[key + "_info"]) == 0
        assert (F[n:] == -2.56e9).all()
        if key + "_f" not in golden:
            continue
        ref = golden[key + "_f"]
        # only the factored triangle is compared; the other is never written
        eff_upper = (uplo == 121) == (order == 102)
        tri = np.triu_indices(n) if eff_upper else np.tril_indices(n)
        assert np.abs(F[:n][tri] - ref[:n][tri]).max() <= 1e-13 * n, key
        other = np.tril_indices(n, -1) if eff_upper else np.triu_indices(n, 1)
        assert np.array_equal(F[:n][other], golden[f"chol_{n}_{lda}_a"][:n][other])
        B = ora.gegen(n, 3, 77 + n)
        assert gb.clapack_dpotrs(order, uplo, n, 3, F, lda, B, n) == 0
        assert np.allclose(B, golden[key + "_x"], rtol=1e-10, atol=1e-12), key


def test_dpotrf_info_matches_reference(gb, golden):
    for (n, lda, bad) in golden["chol_bad"]:
        n, lda, bad = int(n), int(lda), int(bad)
        for uplo in (121, 122):
            A = golden[f"chol_{n}_{lda}_a"].copy(order="F")
            A[bad, bad] = -1.0
            info = gb.clapack_dpotrf(102, uplo, n, A, lda)
            assert info == int(golden[f"cholbad_{n}_{bad}_{uplo}_info"]) == bad + 1
            # columns before the failing block are a finished factor
            done = (bad // 64) * 64
            if done:
                L = np.tril(A[:done, :done]) if uplo == 122 else np.triu(A[:done, :done]).T
                A0 = golden[f"chol_{n}_{lda}_a"][:done, :done]
                assert np.abs(L @ L.T - A0).max() <= 1e-12 * n


@pytest.mark.parametrize("uplo", [121, 122])
def test_dpotrf_large_residual_and_oracle(gb, ora, uplo):
    for n in (1000, 2048 + 17):
        A0 = spd(n, n, lda=n + 2)
        F = A0.copy(order="F")
        assert gb.clapack_dpotrf(102, uplo, n, F, n + 2) == 0
        Ft = A0.copy(order="F")
        assert ora.potrf(Ft, uplo=uplo, N=n) == 0
        L = np.tril(F[:n]) if uplo == 122 else np.triu(F[:n]).T
        Lt = np.tril(Ft[:n]) if uplo == 122 else np.triu(Ft[:n]).T
        eps = np.finfo(np.float64).eps
        resid = np.abs(L @ L.T - A0[:n]).sum(axis=0).max() / (np.abs(A0[:n]).sum(axis=0).max() * n * eps)
        assert resid <= 10.0, resid
        assert np.abs(L - Lt).max() <= 1e-12 * np.abs(Lt).max()


@pytest.mark.parametrize("uplo,order", list(itertools.product((121, 122), (101, 102))))
def test_dposv_solves(gb, ora, uplo, order):
    n, nrhs = 777, 5
    A0 = spd(n, 3 + n, lda=n + 1)
    B0 = np.asfortranarray(np.random.default_rng(5).uniform(-1, 1, (n, nrhs)))
    A = A0.copy(order="F")
    B = B0.copy(order="F")
    assert gb.clapack_dposv(order, uplo, n, nrhs, A, n + 1, B, n) == 0
    At = A0.copy(order="F")
    Bt = B0.copy(order="F")
    assert ora.lib().ora_dposv(order, uplo, n, nrhs, At, n + 1, Bt, n) == 0
    assert np.abs(B - Bt).max() <= 1e-11 * np.abs(Bt).max()
    # row-major B holds the right-hand sides as rows of length n, so both
    # orders solve A X = B for the symmetric A
    assert np.abs(A0[:n] @ B - B0).max() <= 1e-10 * n


def test_dposv_not_positive_definite_leaves_b(gb):
    n = 300
    A = spd(n, 9)
    A[150, 150] = -5.0
    B = np.ones((n, 2), order="F")
    assert gb.clapack_dposv(102, 122, n, 2, A, n, B, n) == 151
    assert (B == 1.0).all()


def test_spotrf_sposv(gb, ora):
    n = 513
    A0 = spd(n, 4, dtype=np.float32)
    F = A0.copy(order="F")
    assert gb.clapack_spotrf(102, 122, n, F, n) == 0
    L = np.tril(F).astype(np.float64)
    rel = np.abs(L @ L.T - A0).max() / np.abs(A0).max()
    assert rel <= 1e-5
    B0 = np.ones((n, 2), dtype=np.float32, order="F")
    A = A0.copy(order="F")
    B = B0.copy(order="F")
    assert gb.clapack_sposv(102, 121, n, 2, A, n, B, n) == 0
    assert np.abs(A0.astype(np.float64) @ B - 1.0).max() <= 1e-3


def test_dpotrf_device_api(gb):
    torch = pytest.importorskip("torch")
    import ctypes as C
    n = 640
    A0 = spd(n, 21)
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()      # row-major A^T = column-major A
    info = gb.lib().atlg_dpotrf_dev(122, n, C.c_void_p(dA.data_ptr()), n, None)
    torch.cuda.synchronize()
    assert info == 0
    L = torch.tril(dA.T)
    A0t = torch.from_numpy(A0).cuda()
    assert float((L @ L.T - A0t).abs().max()) <= 1e-12 * n
    dB = torch.ones((1, n), dtype=torch.float64, device="cuda")   # column-major n x 1
    rc = gb.lib().atlg_dpotrs_dev(102, 122, n, 1, C.c_void_p(dA.data_ptr()), n, C.c_void_p(dB.data_ptr()), n,
                                  None)
    torch.cuda.synchronize()
    assert rc == 0
    x = dB.reshape(n)
    assert float((A0t @ x - 1.0).abs().max()) <= 1e-10
