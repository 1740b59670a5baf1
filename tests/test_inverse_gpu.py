"""clapack_dtrtri / strtri and clapack_dgetri / sgetri through the C ABI,
against the fixtures from the reference's ATL_trtri and clapack_getri (built
from its basefiles) and the oracle: both triangles, orders and diagonals,
singular info, and inverse residuals at sizes with many 64-column blocks."""
import ctypes as C
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tri_of(T, eff_upper, unit):
    X = np.triu(T) if eff_upper else np.tril(T)
    if unit:
        np.fill_diagonal(X, 1.0)
    return X


@pytest.mark.parametrize("uplo,order,diag", list(itertools.product((121, 122), (101, 102), (131, 132))))
def test_dtrtri_reference_fixtures(gb, ora, golden, uplo, order, diag):
    for n in (1, 2, 3, 4, 5, 50):
        T = ora.gegen(n, n, 3 + n)
        T += np.eye(n) * n
        T0 = T.copy(order="F")
        key = f"trtri_{uplo}_{order}_{diag}_{n}"
        assert gb.clapack_dtrtri(order, uplo, diag, n, T, n) == int(golden[key + "_info"]) == 0
        ref = golden[key]
        assert np.abs(T - ref).max() <= 1e-13 * n * max(1.0, np.abs(ref).max()), key
        # the other triangle (and a unit diagonal) is not touched
        eff_upper = (uplo == 121) == (order == 102)
        other = np.tril_indices(n, -1) if eff_upper else np.triu_indices(n, 1)
        assert np.array_equal(T[other], T0[other])
        if diag == 132:
            assert np.array_equal(np.diag(T), np.diag(T0))


@pytest.mark.parametrize("uplo,diag", list(itertools.product((121, 122), (131, 132))))
def test_dtrtri_large_residual_and_oracle(gb, ora, uplo, diag):
    for n in (200, 1000, 2049):
        T = ora.gegen(n, n, 5 + n, lda=n + 3)
        T[:n, :n] = T[:n, :n] / n + 2.0 * np.eye(n)     # well conditioned for both diagonals
        T0 = T.copy(order="F")
        assert gb.clapack_dtrtri(102, uplo, diag, n, T, n + 3) == 0
        Tt = T0.copy(order="F")
        assert ora.trtri(Tt, uplo, diag, N=n) == 0
        eff_upper = uplo == 121
        X = tri_of(T[:n], eff_upper, diag == 132)
        Xt = tri_of(Tt[:n], eff_upper, diag == 132)
        A = tri_of(T0[:n], eff_upper, diag == 132)
        assert np.abs(X @ A - np.eye(n)).max() <= 1e-13 * n
        assert np.abs(X - Xt).max() <= 1e-13 * np.abs(Xt).max()
        assert (T[n:] == T0[n:]).all()


def test_dtrtri_singular_info(gb, ora, golden):
    for (n, z) in ((10, 0), (50, 37), (130, 129)):
        T = ora.gegen(n, n, 3 + n)
        T += np.eye(n) * n
        T[z, z] = 0.0
        T0 = T.copy(order="F")
        assert gb.clapack_dtrtri(102, 121, 131, n, T, n) == int(golden[f"trtri_sing_{n}_{z}_info"]) == z + 1
        assert np.array_equal(T, T0)
        # a unit diagonal is never inspected
        assert gb.clapack_dtrtri(102, 121, 132, n, T, n) == 0


@pytest.mark.parametrize("order", [101, 102])
def test_dgetri_reference_fixtures(gb, golden, order):
    for n in (1, 2, 3, 5, 17, 64, 65, 100):
        key = f"getri_{n}_{order}"
        A = golden[key + "_lu"].copy(order="F")
        piv = golden[key + "_piv"].astype(np.int32)
        assert gb.clapack_dgetri(order, n, A, n, piv) == int(golden[key + "_info"]) == 0
        ref = golden[key + "_inv"]
        assert np.abs(A - ref).max() <= 1e-12 * n * max(1.0, np.abs(ref).max()), key


@pytest.mark.parametrize("order", [101, 102])
def test_dgetri_large_after_dgetrf(gb, ora, order):
    for n in (700, 2048 + 33):
        A0 = ora.gegen(n, n, n * n + n, lda=n + 1)
        A = A0.copy(order="F")
        piv = np.zeros(n, dtype=np.int32)
        assert gb.clapack_dgetrf(order, n, n, A, n + 1, piv) == 0
        F = A.copy(order="F")
        assert gb.clapack_dgetri(order, n, A, n + 1, piv) == 0
        M0 = A0[:n] if order == 102 else A0[:n].T     # the matrix the caller means
        X = A[:n] if order == 102 else A[:n].T
        # ||X A - I||_1 / (n eps ||A||_1 ||X||_1), the inverse tester's residual
        eps = np.finfo(float).eps
        n1 = lambda Z: np.abs(Z).sum(axis=0).max()
        resid = n1(X @ M0 - np.eye(n)) / (n1(X) * n1(M0) * n * eps)
        assert resid <= 1.0, resid
        Ft = F.copy(order="F")
        assert ora.getri(Ft, piv, N=n, order=order) == 0
        assert np.abs(A[:n] - Ft[:n]).max() <= 1e-10 * np.abs(Ft[:n]).max()
        assert (A[n:] == A0[n:]).all()


def test_sgetri_strtri(gb, ora):
    n = 300
    A0 = ora.gegen(n, n, 7, dtype=np.float32)
    A0 += np.eye(n, dtype=np.float32) * 4
    A = A0.copy(order="F")
    piv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_sgetrf(102, n, n, A, n, piv) == 0
    assert gb.clapack_sgetri(102, n, A, n, piv) == 0
    assert np.abs(A.astype(np.float64) @ A0 - np.eye(n)).max() <= 1e-3
    T = ora.gegen(n, n, 8, dtype=np.float32)
    T = np.asfortranarray(T / n + 2 * np.eye(n, dtype=np.float32))
    T0 = T.copy(order="F")
    assert gb.clapack_strtri(102, 122, 131, n, T, n) == 0
    assert np.abs(np.tril(T).astype(np.float64) @ np.tril(T0) - np.eye(n)).max() <= 1e-4


def test_dgetri_device_api(gb, ora):
    torch = pytest.importorskip("torch")
    n = 513
    A0 = ora.gegen(n, n, 99)
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
    piv = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(4, dtype=torch.int32, device="cuda")
    L = gb.lib()
    assert L.atlg_dgetrf_dev(n, n, C.c_void_p(dA.data_ptr()), n, C.c_void_p(piv.data_ptr()),
                             C.c_void_p(info.data_ptr()), None) == 0
    assert L.atlg_dgetri_dev(n, C.c_void_p(dA.data_ptr()), n, C.c_void_p(piv.data_ptr()), None) == 0
    torch.cuda.synchronize()
    X = dA.cpu().numpy().T
    assert np.abs(X @ A0 - np.eye(n)).max() <= 1e-10
