"""Row interchanges (ATL_laswp, AtlasBase/Clint/atlas-lp.base:1053-1166)
through the C ABI, bit-exact: against the reference's own laswp output
(fixtures, forward and backward) and against the oracle on the three ways the
device applies a permutation -- the dense column form (most rows of the span
move), the sparse pair-list form (a few hundred interchanges in a tall
column, as for one block column of the split LU) and the gather/copy form
for tables too large for shared memory -- and on the ways it builds the
row-content table: the parallel form for pivots that look down (getrf's),
the one-thread chain for other pivot vectors and for long chains."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, gb, A, N, K1, K2, piv, inci, nrows):
    """Apply atlg_dlaswp_dev to a column-major copy of A; return the result."""
    L = gb.lib()
    m, lda = A.shape[0], A.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dpiv = torch.from_numpy(np.ascontiguousarray(piv, dtype=np.int32)).cuda()
    torch.cuda.synchronize()
    assert L.atlg_dlaswp_dev(N, dA.data_ptr(), lda, K1, K2, dpiv.data_ptr(), inci, nrows, None) == 0
    torch.cuda.synchronize()
    assert gb.status() == 0
    return dA.cpu().numpy().T


def test_laswp_matches_reference_fixtures(gb, ora, golden):
    torch = pytest.importorskip("torch")
    for (m, n, k1, k2) in ((40, 70, 0, 40), (100, 33, 5, 77), (64, 64, 0, 64)):
        piv = golden[f"laswp_{m}_{n}_{k1}_{k2}_piv"]
        for inci in (1, -1):
            A = ora.gegen(m, n, m * n)
            got = _run(torch, gb, A, n, k1, k2, piv, inci, m)
            assert np.array_equal(got, golden[f"laswp_{m}_{n}_{k1}_{k2}_{inci}"]), (m, n, k1, k2, inci)


@pytest.mark.parametrize("m,N,K1,K2,inci,form", [
    (8192, 300, 0, 8192, 1, "dense"),          # a full LU pivot vector
    (8192, 7, 0, 8192, -1, "dense"),
    (1000, 1, 3, 900, 1, "dense"),             # one right-hand side
    (16384, 40, 0, 512, 1, "sparse"),          # one 512-wide block column of a tall matrix
    (16384, 3, 100, 356, -1, "sparse"),
    (12000, 25, 0, 64, 1, "sparse"),
    (20000, 3, 0, 20000, 1, "gather"),         # table beyond the shared-memory form
    (13000, 5, 0, 13000, -1, "one-thread chain"),  # too many interchanges for the parallel table
])
def test_laswp_forms_match_oracle(gb, ora, m, N, K1, K2, inci, form):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(m + N + K1)
    piv = np.arange(m, dtype=np.int32)
    piv[K1:K2] = [rng.integers(i, m) for i in range(K1, K2)]
    A = ora.gegen(m, N, m * N + 3)
    got = _run(torch, gb, A, N, K1, K2, piv, inci, m)
    ref = A.copy(order="F")
    ora.laswp(N, ref, K1, K2, piv, inci)
    assert np.array_equal(got, ref), form


def test_laswp_no_interchange_is_identity(gb, ora):
    torch = pytest.importorskip("torch")
    m, N = 500, 9
    piv = np.arange(m, dtype=np.int32)
    A = ora.gegen(m, N, 17)
    got = _run(torch, gb, A, N, 0, m, piv, 1, m)
    assert np.array_equal(got, A)


@pytest.mark.parametrize("inci", [1, -1])
def test_laswp_pivots_that_look_up(gb, ora, inci):
    """Pivot vectors with ipiv[i] < i (not from getrf) take the one-thread
    interchange chain; the result is still the reference's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    m, N, K1, K2 = 3000, 20, 10, 2900
    piv = rng.integers(0, m, size=m).astype(np.int32)
    A = ora.gegen(m, N, 99)
    got = _run(torch, gb, A, N, K1, K2, piv, inci, m)
    ref = A.copy(order="F")
    ora.laswp(N, ref, K1, K2, piv, inci)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("kind", ["one target", "few targets", "clustered"])
@pytest.mark.parametrize("inci", [1, -1])
def test_laswp_table_buckets_and_crowded_targets(gb, ora, kind, inci):
    """Pivots that look down with many sources per target: the table's
    counting sort sorts each target's sources in one thread up to 64 of them
    and falls back to the warp scan beyond; both give the reference's
    permutation."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(len(kind) + inci)
    m, N, K1, K2 = 4096, 6, 0, 4000
    piv = np.arange(m, dtype=np.int32)
    if kind == "one target":          # every interchange with the last row
        piv[K1:K2] = m - 1
    elif kind == "few targets":       # about 50 sources per target, around the bucket limit
        tg = np.sort(rng.choice(np.arange(K2, m), size=80, replace=False))
        piv[K1:K2] = [tg[rng.integers(0, 80)] for _ in range(K1, K2)]
    else:                             # targets just below each source
        piv[K1:K2] = [min(m - 1, i + int(rng.integers(0, 4))) for i in range(K1, K2)]
    A = ora.gegen(m, N, 5 * m + N)
    got = _run(torch, gb, A, N, K1, K2, piv, inci, m)
    ref = A.copy(order="F")
    ora.laswp(N, ref, K1, K2, piv, inci)
    assert np.array_equal(got, ref), kind
