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


def split_emulation(A, B, alpha, beta, C0, ns):
    """The split DGEMM's arithmetic restated in numpy: per-row / per-column
    exponents (frexp of the max), 7-bit digits by the exact FP64 recurrence
    x *= 128, d = trunc(x), x -= d, exact integer diagonal sums, and the FP64
    recombination smallest diagonal first (C = beta C + v for the first
    diagonal, C += v after it, v = (acc * alpha 2^(ea - 7(d+2))) * 2^eb)."""
    def expo(v):
        m = np.abs(v).max(axis=1)
        return np.where(m > 0, np.frexp(m)[1], 0)

    def digits(V, e):
        x = np.ldexp(V, -e[:, None])
        out = []
        for _ in range(ns):
            x = x * 128.0
            d = np.trunc(x)
            x = x - d
            out.append(d)
        return out

    ea, eb = expo(A), expo(B.T)
    At, Bt = digits(A, ea), digits(B.T, eb)
    C = C0.copy()
    first = True
    for d in range(ns - 1, -1, -1):
        # digit products < 2^14, sums < 2^53: exact in FP64 in any order
        acc = sum(At[t] @ Bt[d - t].T for t in range(d + 1))
        fr = np.ldexp(alpha, ea - 7 * (d + 2))
        v = (acc * fr[:, None]) * np.ldexp(1.0, eb)[None, :]
        if first and beta == 0.0:
            C = v
        else:
            C = C + v
        first = False
    return C


@pytest.mark.parametrize("alpha,beta,ns", [(1.0, 0.0, 8), (-0.75, 1.0, 8), (1.0 / 3.0, 0.0, 5), (-1.0, 1.0, 3)])
def test_split_dgemm_bit_exact_vs_emulation(gb, alpha, beta, ns):
    # every step of the split scheme, bit for bit: mixed magnitudes and signs,
    # an all-zero row and column, subnormal entries, exact powers of two
    M, N, K = 190, 300, 1100
    rng = np.random.default_rng(ns)
    A = rng.uniform(-1, 1, (M, K)) * np.exp2(rng.integers(-30, 31, (M, K)))
    B = rng.uniform(-1, 1, (K, N)) * np.exp2(rng.integers(-30, 31, (K, N)))
    A[5, :] = 0.0
    B[:, 7] = 0.0
    A[9, :10] = 5e-310
    A[9, 10] = 1.0
    B[3, 11] = -4.9e-324
    A[11, 12] = -2.0 ** 40
    A = np.asfortranarray(A)
    B = np.asfortranarray(B)
    C0 = np.asfortranarray(rng.standard_normal((M, N)))
    Cg = C0.copy(order="F")
    gb.dgemm_split(111, 111, alpha, A, B, beta, Cg, nslices=ns)
    ref = split_emulation(A, B, alpha, beta, C0, ns)
    assert np.array_equal(Cg, ref)
