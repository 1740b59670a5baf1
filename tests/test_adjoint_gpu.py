"""dgesv_adjoint through the C ABI and a torch.autograd.Function test
harness around it: X = A^{-1} B; for an upstream gX, gB = A^{-T} gX and
gA = -gB X^T.  Checked against central finite differences (h = 1e-6, 32
random directions) and against the gradient built from the oracle's CPU
solve, at a small size and at the workload's own size (n = 4096, nrhs = 64),
where the solve is also repeated through the mixed-precision path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.standard_normal((n, n)) / np.sqrt(n) + 4.0 * np.eye(n))
    B = np.asfortranarray(rng.standard_normal((n, nrhs)))
    gX = np.asfortranarray(rng.standard_normal((n, nrhs)))
    return A, B, gX


def solve(gb, A, B):
    n, nrhs = B.shape
    LU = A.copy(order="F")
    X = B.copy(order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    assert gb.clapack_dgesv(102, n, nrhs, LU, n, ipiv, X, n) == 0
    return LU, ipiv, X


def test_adjoint_matches_oracle_gradient(gb, ora):
    n, nrhs = 512, 16
    A, B, gX = make(n, nrhs, 3)
    LU, ipiv, X = solve(gb, A, B)
    gA, gB = gb.dgesv_adjoint(LU, ipiv, X, gX)
    # oracle: gB = A^{-T} gX by the CPU transposed solve, gA = -gB X^T
    Lo = A.copy(order="F")
    info, opiv = ora.getrf(Lo)
    gBo = gX.copy(order="F")
    ora.getrs(Lo, opiv, gBo, trans=ora.Trans)
    gAo = -gBo @ X.T
    assert np.abs(gB - gBo).max() <= 1e-12 * np.abs(gBo).max()
    assert np.abs(gA - gAo).max() <= 1e-12 * np.abs(gAo).max()


def test_autograd_function_against_finite_differences(gb):
    torch = pytest.importorskip("torch")

    class Solve(torch.autograd.Function):
        """Test harness only: forward = clapack_dgesv, backward = dgesv_adjoint."""

        @staticmethod
        def forward(ctx, A, B):
            An = np.asfortranarray(A.detach().numpy())
            Bn = np.asfortranarray(B.detach().numpy())
            LU, ipiv, X = solve(gb, An, Bn)
            ctx.saved = (LU, ipiv, X)
            return torch.from_numpy(np.ascontiguousarray(X))

        @staticmethod
        def backward(ctx, gX):
            LU, ipiv, X = ctx.saved
            gA, gB = gb.dgesv_adjoint(LU, ipiv, X, np.asfortranarray(gX.numpy()))
            return torch.from_numpy(np.ascontiguousarray(gA)), torch.from_numpy(np.ascontiguousarray(gB))

    n, nrhs = 96, 8
    A, B, gX = make(n, nrhs, 11)
    At = torch.tensor(A, requires_grad=True)
    Bt = torch.tensor(B, requires_grad=True)
    X = Solve.apply(At, Bt)
    X.backward(torch.from_numpy(gX))
    gA, gB = At.grad.numpy(), Bt.grad.numpy()
    rng = np.random.default_rng(5)
    h = 1e-6
    for _ in range(32):
        dA = rng.standard_normal((n, n))
        dB = rng.standard_normal((n, nrhs))
        Xp = solve(gb, np.asfortranarray(A + h * dA), np.asfortranarray(B + h * dB))[2]
        Xm = solve(gb, np.asfortranarray(A - h * dA), np.asfortranarray(B - h * dB))[2]
        fd = np.sum(gX * (Xp - Xm)) / (2 * h)
        an = np.sum(gA * dA) + np.sum(gB * dB)
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)


def _mixed_solve(gb, A, B):
    n, nrhs = B.shape
    X = np.zeros((n, nrhs), order="F")
    ipiv = np.zeros(n, dtype=np.int32)
    info, berr, ferr, iters, status = gb.dgesv_mixed(A.copy(order="F"), ipiv, B.copy(order="F"), X)
    assert info == 0
    return X, status


def test_adjoint_at_n4096_nrhs64(gb, ora):
    """The differentiable-solve workload at its stated size: A = G/sqrt(n) + 4I,
    B and gX Gaussian.  gA, gB against the gradient built from the oracle's
    CPU solve and against central finite differences (h = 1e-6, 32 random
    directions); then the forward and the transposed solve repeated through
    the mixed-precision path, whose gradient must agree with the FP64 one to
    the refinement's accuracy."""
    n, nrhs = 4096, 64
    A, B, gX = make(n, nrhs, 2024)
    LU, ipiv, X = solve(gb, A, B)
    gA, gB = gb.dgesv_adjoint(LU, ipiv, X, gX)
    ora.set_threads(0)
    Lo = A.copy(order="F")
    info, opiv = ora.getrf(Lo)
    assert info == 0
    Xo = B.copy(order="F")
    ora.getrs(Lo, opiv, Xo)
    gBo = gX.copy(order="F")
    ora.getrs(Lo, opiv, gBo, trans=ora.Trans)
    gAo = -gBo @ Xo.T
    assert np.abs(gB - gBo).max() <= 1e-12 * np.abs(gBo).max()
    assert np.abs(gA - gAo).max() <= 1e-12 * np.abs(gAo).max()
    rng = np.random.default_rng(8)
    h = 1e-6
    for _ in range(32):
        dA = rng.standard_normal((n, n))
        dB = rng.standard_normal((n, nrhs))
        Xp = solve(gb, np.asfortranarray(A + h * dA), np.asfortranarray(B + h * dB))[2]
        Xm = solve(gb, np.asfortranarray(A - h * dA), np.asfortranarray(B - h * dB))[2]
        fd = np.sum(gX * (Xp - Xm)) / (2 * h)
        an = np.sum(gA * dA) + np.sum(gB * dB)
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)
    Xmx, st1 = _mixed_solve(gb, A, B)
    gBm, st2 = _mixed_solve(gb, np.asfortranarray(A.T), gX)
    gAm = -gBm @ Xmx.T
    assert st1 == 0 and st2 == 0                     # refinement converged, no FP64 fallback
    assert np.abs(gBm - gB).max() <= 1e-12 * np.abs(gB).max()
    assert np.abs(gAm - gA).max() <= 1e-12 * np.abs(gA).max()
