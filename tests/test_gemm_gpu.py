"""DGEMM/SGEMM through the C ABI against the oracle and the reference-BLAS
fixtures, with the xdl3blastst residual (AtlasBase/Antoine/atlbinblas.base:
11910-11930): resid = ||C-C0||_1 / (max(||A||,1) max(||B||,1) max(||C||,1)
eps max(M,N,K)) <= 50."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
THRESH = 50.0


def gen_operands(ora, ta, tb, M, N, K, pad=0, dtype=np.float64):
    mA, nA = (M, K) if ta == 111 else (K, M)
    mB, nB = (K, N) if tb == 111 else (N, K)
    A = ora.gegen(mA, nA, mA * nA + 513 * 7 + 90, lda=mA + pad, dtype=dtype)
    B = ora.gegen(mB, nB, mB * nB + 127 * 50 + 77, lda=mB + pad, dtype=dtype)
    Cm = ora.gegen(M, N, M * N + 101 * 2 + 53, lda=M + pad, dtype=dtype)
    return A, B, Cm


CASES = [
    (111, 111, 1024, 1024, 1024, 1.0, 0.0, 0),     # the headline DGEMM shape
    (111, 111, 1, 1, 1, 1.0, 0.0, 0),
    (111, 111, 33, 17, 5, 1.0, 1.0, 3),
    (111, 112, 129, 65, 257, -1.0, 0.5, 1),
    (112, 111, 200, 300, 64, 2.5, -1.0, 0),
    (112, 112, 77, 1, 190, 0.75, 0.0, 2),
    (111, 111, 1000, 3, 700, 1.0, 1.0, 0),
    (111, 111, 5, 2000, 40, -0.5, 0.25, 5),
]


@pytest.mark.parametrize("ta,tb,M,N,K,alpha,beta,pad", CASES)
def test_dgemm_matches_oracle(gb, ora, ta, tb, M, N, K, alpha, beta, pad):
    A, B, C0 = gen_operands(ora, ta, tb, M, N, K, pad)
    Cin = C0.copy(order="F")
    Cg = C0.copy(order="F")
    gb.cblas_dgemm(102, ta, tb, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta, Cg, Cg.shape[0])
    Ct = C0.copy(order="F")
    ora.lib().ora_dgemm(ta, tb, M, N, K, alpha, A, A.shape[0], B, B.shape[0], beta, Ct, Ct.shape[0])
    r = ora.gemm_resid(ta, tb, M, N, K, alpha, A, B, beta, Cin, Cg, Ct)
    assert r <= THRESH, r
    eps = np.finfo(float).eps
    bound = 2 * K * eps * (abs(alpha) * K * np.abs(A).max() * np.abs(B).max() + abs(beta) * np.abs(Cin[:M]).max())
    assert np.abs(Cg[:M] - Ct[:M]).max() <= bound
    if pad:
        assert (Cg[M:] == -2.56e9).all(), "lda gap was written"


def test_dgemm_reference_fixtures(gb, ora, golden):
    for (ta, tb, M, N, K, al, be) in golden["gemm_cases"]:
        ta, tb, M, N, K = int(ta), int(tb), int(M), int(N), int(K)
        A, B, Cm = gen_operands(ora, ta, tb, M, N, K)
        gb.cblas_dgemm(102, ta, tb, M, N, K, al, A, A.shape[0], B, B.shape[0], be, Cm, M)
        assert np.abs(Cm - golden[f"gemm_{ta}_{tb}_{M}_{N}_{K}"]).max() <= 1e-13 * K * 4


def test_dgemm_rowmajor(gb, ora):
    M, N, K = 70, 45, 33
    A = np.asfortranarray(ora.gegen(K, M, 1).T.copy())        # any data
    Ar = np.ascontiguousarray(ora.gegen(M, K, 11).reshape(-1))  # row-major M x K, lda=K
    Br = np.ascontiguousarray(ora.gegen(K, N, 12).reshape(-1))  # row-major K x N, ldb=N
    Cr = np.zeros(M * N)
    a2 = np.asfortranarray(Ar.reshape(1, -1).T)
    b2 = np.asfortranarray(Br.reshape(1, -1).T)
    c2 = np.asfortranarray(Cr.reshape(1, -1).T)
    gb.lib().cblas_dgemm(101, 111, 111, M, N, K, 1.0, a2, K, b2, N, 0.0, c2, N)
    ref = Ar.reshape(M, K) @ Br.reshape(K, N)
    assert np.allclose(c2.reshape(M, N), ref, rtol=0, atol=1e-13 * K)
    del A


def test_dgemm_symmetric_product_is_exactly_symmetric(gb, ora):
    # cblas_dgemm with A==B, TA!=TB, beta==0 is the reference's syrk shortcut
    # (AtlasBase/Clint/cblas.base:221-231): the result must be symmetric.
    n, k = 300, 120
    A = ora.gegen(n, k, 5)
    Cm = np.zeros((n, n), order="F")
    gb.cblas_dgemm(102, 111, 112, n, n, k, 1.0, A, n, A, n, 0.0, Cm, n)
    assert np.array_equal(Cm, Cm.T)


def test_alpha_zero_and_k_zero_scale_c(gb, ora):
    M, N = 40, 30
    A = ora.gegen(M, 8, 1)
    B = ora.gegen(8, N, 2)
    C0 = ora.gegen(M, N, 3)
    Cm = C0.copy(order="F")
    gb.cblas_dgemm(102, 111, 111, M, N, 8, 0.0, A, M, B, 8, 2.0, Cm, M)
    assert np.array_equal(Cm, 2.0 * C0)
    Cm = C0.copy(order="F")
    gb.cblas_dgemm(102, 111, 111, M, N, 0, 1.0, A, M, B, 8, 0.0, Cm, M)
    assert (Cm == 0).all()


def test_beta_zero_ignores_nan_in_c(gb, ora):
    M, N, K = 64, 64, 64
    A, B, _ = gen_operands(ora, 111, 111, M, N, K)
    Cm = np.full((M, N), np.nan, order="F")
    gb.cblas_dgemm(102, 111, 111, M, N, K, 1.0, A, M, B, K, 0.0, Cm, M)
    assert np.isfinite(Cm).all()


def test_tma_and_cpasync_loaders_agree_bitwise(gb, ora):
    torch = pytest.importorskip("torch")
    M, N, K = 517, 263, 301
    A, B, _ = gen_operands(ora, 111, 111, M, N, K)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()  # column-major storage
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    outs = []
    for tma in (1, 0):
        dC = torch.zeros((N, M + 1), dtype=torch.float64, device="cuda")   # ldc = M+1 (odd)
        gb.lib().atlg_dgemm_dev_opts(111, 111, M, N, K, 1.0, dA.data_ptr(), M, dB.data_ptr(), K, 0.0,
                                     dC.data_ptr(), M + 1, tma, None)
        torch.cuda.synchronize()
        outs.append(dC.cpu().numpy()[:, :M].copy())
    assert np.array_equal(outs[0], outs[1])
    ref = A @ B
    assert np.abs(outs[0].T - ref).max() < 1e-12


@pytest.mark.parametrize("ta,tb,M,N,K", [(111, 111, 300, 200, 150), (112, 112, 129, 1, 77),
                                         (111, 112, 1024, 1024, 1024)])
def test_sgemm_matches_oracle(gb, ora, ta, tb, M, N, K):
    A, B, C0 = gen_operands(ora, ta, tb, M, N, K, dtype=np.float32)
    Cg = C0.copy(order="F")
    gb.cblas_sgemm(102, ta, tb, M, N, K, 1.5, A, A.shape[0], B, B.shape[0], -0.5, Cg, M)
    Ct = C0.copy(order="F")
    ora.lib().ora_sgemm(ta, tb, M, N, K, 1.5, A, A.shape[0], B, B.shape[0], -0.5, Ct, M)
    eps = np.finfo(np.float32).eps
    assert np.abs(Cg - Ct).max() <= 2 * K * eps * (np.abs(A).max() * np.abs(B).max() * 1.5 + 1)


def test_dgemm_1024_matches_reference_blas(gb, ora, golden_large):
    """cblas_dgemm at 1024^3 (NoTrans/NoTrans, alpha 1, beta 0, gemmtst
    seeds) against the reference BLAS product of the same operands: 16384
    sampled entries within the elementwise bound 2 K eps K max|A| max|B| and
    every column 1-norm to 1e-12."""
    n = 1024
    A, B, Cm = gen_operands(ora, 111, 111, n, n, n)
    gb.cblas_dgemm(102, 111, 111, n, n, n, 1.0, A, n, B, n, 0.0, Cm, n)
    idx = golden_large["gemm_1024_idx"]
    ref = golden_large["gemm_1024_val"]
    got = Cm.reshape(-1, order="F")[idx]
    bound = 2 * n * np.finfo(float).eps * n * np.abs(A).max() * np.abs(B).max()
    assert np.max(np.abs(got - ref)) <= bound
    cn = golden_large["gemm_1024_colnrm1"]
    assert np.max(np.abs(np.abs(Cm).sum(axis=0) - cn) / cn) <= 1e-12
