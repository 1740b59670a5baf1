"""DTRSM through the C ABI: all Side/Uplo/Trans/Diag cases against the
oracle and the reference-BLAS fixtures; A diagonally dominant as in
xdl3blastst's trsmtst (AtlasBase/Antoine/atlbinblas.base:12761-12890)."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ALL = list(itertools.product((141, 142), (121, 122), (111, 112), (131, 132)))


@pytest.mark.parametrize("side,uplo,ta,diag", ALL)
def test_dtrsm_matches_oracle(gb, ora, side, uplo, ta, diag):
    for (M, N, alpha) in ((45, 38, 1.5), (200, 131, -1.0), (64, 1, 1.0), (1, 70, 2.0)):
        na = M if side == 141 else N
        A = ora.gegen(na, na, na * na + 11, lda=na + 1)
        A[:na, :na] += np.eye(na) * na
        B0 = ora.gegen(M, N, M * N + 3, lda=M + 2)
        Bg = B0.copy(order="F")
        gb.cblas_dtrsm(102, side, uplo, ta, diag, M, N, alpha, A, na + 1, Bg, M + 2)
        Bt = B0.copy(order="F")
        ora.lib().ora_dtrsm(side, uplo, ta, diag, M, N, alpha, A, na + 1, Bt, M + 2)
        scale = np.abs(Bt[:M]).max() + 1
        assert np.abs(Bg[:M] - Bt[:M]).max() <= 1e-12 * scale * max(M, N), (M, N)
        assert (Bg[M:] == -2.56e9).all()


def test_dtrsm_reference_fixtures(gb, ora, golden):
    for (side, uplo, ta, diag) in ALL:
        M, N = 45, 38
        na = M if side == 141 else N
        A = ora.gegen(na, na, na * na + 11)
        A += np.eye(na) * na
        B = ora.gegen(M, N, M * N + 3)
        gb.cblas_dtrsm(102, side, uplo, ta, diag, M, N, 1.5, A, na, B, M)
        assert np.allclose(B, golden[f"trsm_{side}_{uplo}_{ta}_{diag}"], rtol=1e-9, atol=1e-9)


def test_dtrsm_rowmajor_equals_transposed_colmajor(gb, ora):
    M, N = 90, 70
    A = ora.gegen(N, N, 4)
    A += np.eye(N) * N
    B = ora.gegen(M, N, 5)
    # row-major B (M x N, ldb=N) is the column-major B^T
    Bt = np.asfortranarray(B.T.copy())
    At = np.asfortranarray(A.T.copy())
    gb.cblas_dtrsm(101, 142, 121, 111, 131, M, N, 1.0, At, N, Bt, N)
    ref = B.copy(order="F")
    ora.lib().ora_dtrsm(142, 121, 111, 131, M, N, 1.0, A, N, ref, M)
    assert np.allclose(Bt.T, ref, rtol=1e-12, atol=1e-12)


def test_strsm(gb, ora):
    M, N = 150, 40
    A = ora.gegen(M, M, 9, dtype=np.float32)
    A += np.eye(M, dtype=np.float32) * M
    B0 = ora.gegen(M, N, 10, dtype=np.float32)
    Bg = B0.copy(order="F")
    gb.cblas_strsm(102, 141, 122, 111, 131, M, N, 1.0, A, M, Bg, M)
    Bt = B0.copy(order="F")
    ora.lib().ora_strsm(141, 122, 111, 131, M, N, 1.0, A, M, Bt, M)
    assert np.allclose(Bg, Bt, rtol=1e-4, atol=1e-5)
