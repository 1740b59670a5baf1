"""The split-DGEMM form of dgesv (dgesv_split: FP64 LU whose trailing updates
run on the split-precision tensor-core DGEMM): the tester's LU residual and
valid pivots, FP64-level backward error at condition numbers where the
mixed-precision solve must fall back, agreement with the oracle's solve, and
the zero-pivot info."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [700, 1500, 2049])
def test_split_lu_residual_and_pivots(gb, ora, n):
    seed = n * n + n
    A = ora.gegen(n, n, seed)
    piv = np.zeros(n, dtype=np.int32)
    B = np.zeros((n, 1), order="F")
    assert gb.dgesv_split(n, 0, A, n, piv, B, n) == 0
    assert (piv >= np.arange(n)).all() and (piv < n).all()
    # xdlutst: ||PA - LU||_1 / (||A||_1 eps n) <= 100
    assert ora.lu_resid(n, n, A, piv, seed) <= 100.0


def test_split_dgesv_matches_oracle_solve(gb, ora):
    n = 1800
    A0 = ora.gegen(n, n, 11)
    b0 = ora.gegen(n, 2, 12)
    A = A0.copy(order="F")
    b = b0.copy(order="F")
    piv = np.zeros(n, dtype=np.int32)
    assert gb.dgesv_split(n, 2, A, n, piv, b, n) == 0
    At = A0.copy(order="F")
    bt = b0.copy(order="F")
    info, ip = ora.getrf(At)
    ora.getrs(At, ip, bt)
    assert np.abs(b - bt).max() <= 1e-9 * np.abs(bt).max()
    for j in range(2):
        assert ora.backward_error(A0, b[:, j], b0[:, j]) <= n * np.finfo(float).eps


@pytest.mark.parametrize("kappa", [1e2, 1e10, 1e14])
def test_split_dgesv_backward_error_any_condition(gb, ora, kappa):
    n = 1024
    rng = np.random.default_rng(3)
    U, _ = np.linalg.qr(rng.standard_normal((n, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.logspace(0, -np.log10(kappa), n)
    A0 = np.asfortranarray((U * s) @ V.T)
    b0 = np.asfortranarray(rng.standard_normal((n, 1)))
    A = A0.copy(order="F")
    b = b0.copy(order="F")
    piv = np.zeros(n, dtype=np.int32)
    assert gb.dgesv_split(n, 1, A, n, piv, b, n) == 0
    berr = ora.backward_error(A0, b[:, 0], b0[:, 0])
    assert berr <= n * np.finfo(float).eps, berr


def test_split_lu_zero_pivot_info(gb, ora):
    n = 1100
    A = ora.gegen(n, n, 5)
    A[:, 700] = 0.0
    piv = np.zeros(n, dtype=np.int32)
    B = np.ones((n, 1), order="F")
    info = gb.dgesv_split(n, 1, A, n, piv, B, n)
    assert info == 701
    assert (B == 1.0).all()


@pytest.mark.parametrize("leaf", [256, 512])
def test_split_lu_narrow_leaves(gb, ora, leaf):
    # 1024-wide outer blocks factored recursively with narrower FP64 leaves
    # (split products inside the block column); same residual bound, and the
    # zero-pivot info from inside a recursive block
    lib = gb.lib()
    lib.atlg_split_lu_leaf(leaf)
    try:
        n = 2300
        A = ora.gegen(n, n, 77)
        piv = np.zeros(n, dtype=np.int32)
        B = np.zeros((n, 1), order="F")
        assert gb.dgesv_split(n, 0, A, n, piv, B, n) == 0
        assert (piv >= np.arange(n)).all() and (piv < n).all()
        assert ora.lu_resid(n, n, A, piv, 77) <= 100.0
        A = ora.gegen(n, n, 78)
        A[:, 1500] = 0.0
        assert gb.dgesv_split(n, 0, A, n, piv, B, n) == 1501
    finally:
        lib.atlg_split_lu_leaf(0)
