"""Split-precision DGEMM (integer slices on tcgen05 tensor cores, FP64
recombination) through the C ABI.

1. Exactness of the tensor-core path: integer operands whose rows/columns
   peak at 127 are carried by the first slice alone, so the result must equal
   the exact integer product bit for bit -- with every entry +-127, each FP32
   chunk accumulator reaches 1024 * 127^2 = 16.5e6 (< 2^24) and K spans
   several 1024-chunks and a ragged tail.
2. Accuracy on the configuration's distribution (uniform[-1,1] * 2^e,
   e in [-16, 16] per element): against the double-double oracle on sampled
   entries and against the FP64 DGEMM.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def int_operands(M, N, K, seed, worst=False):
    rng = np.random.default_rng(seed)
    if worst:
        A = 127.0 * np.where(rng.random((M, K)) < 0.5, -1.0, 1.0)
        B = 127.0 * np.where(rng.random((K, N)) < 0.5, -1.0, 1.0)
    else:
        A = rng.integers(-127, 128, (M, K)).astype(np.float64)
        B = rng.integers(-127, 128, (K, N)).astype(np.float64)
        A[:, 0] = 127.0
        B[0, :] = -127.0
    return np.asfortranarray(A), np.asfortranarray(B)


@pytest.mark.parametrize("M,N,K,worst,ns", [(300, 200, 3000, False, 1), (256, 384, 4096, True, 1),
                                             (129, 130, 1025, False, 7), (64, 1000, 64, True, 3)])
def test_split_dgemm_integer_exact(gb, M, N, K, worst, ns):
    A, B = int_operands(M, N, K, M + N + K, worst)
    Cm = np.zeros((M, N), order="F")
    gb.dgemm_split(111, 111, 1.0, A, B, 0.0, Cm, nslices=ns)
    exact = (A.astype(np.int64) @ B.astype(np.int64)).astype(np.float64)
    assert np.array_equal(Cm, exact)


def config3_operands(M, N, K, seed):
    rng = np.random.default_rng(seed)
    A = rng.uniform(-1, 1, (M, K)) * np.exp2(rng.integers(-16, 17, (M, K)))
    B = rng.uniform(-1, 1, (K, N)) * np.exp2(rng.integers(-16, 17, (K, N)))
    return np.asfortranarray(A), np.asfortranarray(B)


@pytest.mark.parametrize("M,N,K", [(1024, 1024, 1024), (777, 555, 1333)])
def test_split_dgemm_accuracy_vs_double_double(gb, ora, M, N, K):
    A, B = config3_operands(M, N, K, 3)
    C7 = np.zeros((M, N), order="F")
    gb.dgemm_split(111, 111, 1.0, A, B, 0.0, C7, nslices=7)
    C64 = np.zeros((M, N), order="F")
    gb.dgemm(111, 111, 1.0, A, B, 0.0, C64)
    rng = np.random.default_rng(1)
    ii = rng.integers(0, M, 400)
    jj = rng.integers(0, N, 400)
    hi, lo = ora.dd_samples(111, 111, M, N, K, A, B, ii, jj)
    ref = hi + lo
    absab = np.array([np.abs(A[i, :]) @ np.abs(B[:, j]) for i, j in zip(ii, jj)])
    rowmax = np.abs(A).max(axis=1)[ii]
    colmax = np.abs(B).max(axis=0)[jj]
    err7 = np.abs(C7[ii, jj] - ref)
    err64 = np.abs(C64[ii, jj] - ref)
    # truncation after 7 x 7 bits of the row / column maxima (error-free split + dropped pairs)
    assert (err7 <= K * 2.0 ** -47 * rowmax * colmax).all()
    # normwise: comparable with the FP64 DGEMM's own rounding
    assert err7.max() <= 64 * max(err64.max(), np.finfo(float).eps * absab.max())


@pytest.mark.parametrize("ta,tb", [(111, 112), (112, 111), (112, 112)])
def test_split_dgemm_transposes_alpha_beta(gb, ta, tb):
    M, N, K = 200, 150, 300
    rng = np.random.default_rng(ta + tb)
    A = np.asfortranarray(rng.standard_normal((M, K) if ta == 111 else (K, M)))
    B = np.asfortranarray(rng.standard_normal((K, N) if tb == 111 else (N, K)))
    C0 = np.asfortranarray(rng.standard_normal((M, N)))
    Cs = C0.copy(order="F")
    gb.dgemm_split(ta, tb, -1.5, A, B, 0.5, Cs, nslices=8)
    opA = A if ta == 111 else A.T
    opB = B if tb == 111 else B.T
    ref = -1.5 * (opA @ opB) + 0.5 * C0
    assert np.abs(Cs - ref).max() <= 1e-12 * np.abs(ref).max()
