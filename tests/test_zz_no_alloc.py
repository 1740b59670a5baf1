"""atlg_dlaswp_noalloc: the row-interchange entry point for callers that
cannot let a library allocate device memory (their own pool owns it, or they
cannot take the synchronisation of cudaMalloc/cudaFree).  Its scratch is a
fixed array in the library, so this checks, through the C ABI, that two calls
in a row give exactly the result of the allocating entry point
atlg_dlaswp_dev (a permutation: bit-exact), including a table too large for
shared memory (kept in the fixed array before the gathered rows); that with
stream NULL it runs on the library's own stream, ordered after a
factorization launched there; and that bad ranges and calls needing more
than the fixed scratch are refused before any work is queued.  The file is
named to be collected last."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(torch, ora, m, n, seed, rng):
    A = ora.gegen(m, n, seed)
    piv = np.array([rng.integers(i, m) for i in range(m)], dtype=np.int32)
    dA1 = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dA2 = dA1.clone()
    dpiv = torch.from_numpy(piv).cuda()
    return A, piv, dA1, dA2, dpiv


# (rows, columns, K1, K2, inci, seed); 60000 rows exceed the 49152-entry
# shared-memory table, so the table lives in the fixed array
CASES = ((300, 17, 0, 300, 1, 11), (1000, 5, 3, 900, -1, 12), (60000, 2, 0, 60000, 1, 13),
         (60000, 1, 7, 59000, -1, 14))


def test_noalloc_matches_allocating_laswp_twice(gb, ora):
    torch = pytest.importorskip("torch")
    L = gb.lib()
    rng = np.random.default_rng(7)
    for (m, n, k1, k2, inci, seed) in CASES:
        A, piv, dA1, dA2, dpiv = _case(torch, ora, m, n, seed, rng)
        torch.cuda.synchronize()
        assert L.atlg_dlaswp_dev(n, dA1.data_ptr(), m, k1, k2, dpiv.data_ptr(), inci, m, None) == 0
        assert L.atlg_dlaswp_noalloc(n, dA2.data_ptr(), m, k1, k2, dpiv.data_ptr(), inci, m, None) == 0
        torch.cuda.synchronize()
        got = dA2.cpu().numpy().T
        assert np.array_equal(got, dA1.cpu().numpy().T)
        ref = A.copy(order="F")
        ora.laswp(n, ref, k1, k2, piv, inci)
        assert np.array_equal(got, ref)


def test_noalloc_null_stream_follows_a_factorization_on_the_library_stream(gb, ora):
    """dgetrf and the interchanges both on stream NULL, no synchronisation in
    between: the interchanges must see the pivots and factors the
    factorization wrote."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    n = 1024                           # 8 MiB of gathered rows: within the fixed scratch
    A = ora.gegen(n, n, n * n + n)
    dA1 = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dA2 = dA1.clone()
    piv1 = torch.zeros(n, dtype=torch.int32, device="cuda")
    piv2 = torch.zeros(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    # reference result: factor, wait, then interchange on the host
    assert L.atlg_dgetrf_dev(n, n, dA1.data_ptr(), n, piv1.data_ptr(), info.data_ptr(), None) == 0
    torch.cuda.synchronize()
    expect = dA1.cpu().numpy().T.copy(order="F")
    ora.laswp(n, expect, 0, n, piv1.cpu().numpy(), -1)
    # the same two steps queued back to back on the library stream
    assert L.atlg_dgetrf_dev(n, n, dA2.data_ptr(), n, piv2.data_ptr(), info[1:].data_ptr(), None) == 0
    assert L.atlg_dlaswp_noalloc(n, dA2.data_ptr(), n, 0, n, piv2.data_ptr(), -1, n, None) == 0
    torch.cuda.synchronize()
    assert int(info[0]) == 0 and int(info[1]) == 0
    assert np.array_equal(piv2.cpu().numpy(), piv1.cpu().numpy())
    assert np.array_equal(dA2.cpu().numpy().T, expect)


def test_noalloc_rejects_sizes_beyond_its_scratch(gb):
    L = gb.lib()
    # 4096 rows x 600 columns need 19.7 MB > 16 MiB: refused before touching memory
    rc = L.atlg_dlaswp_noalloc(600, None, 4096, 0, 4096, None, 1, 4096, None)
    assert rc == -2


def test_noalloc_rejects_interchange_ranges_outside_the_rows(gb):
    L = gb.lib()
    # K1 < 0 or K2 > nrows would index past the row-content table: -1, no work
    assert L.atlg_dlaswp_noalloc(4, None, 100, -1, 50, None, 1, 100, None) == -1
    assert L.atlg_dlaswp_noalloc(4, None, 100, 0, 101, None, 1, 100, None) == -1
    assert L.atlg_dlaswp_noalloc(4, None, 99, 0, 10, None, 1, 100, None) == -1
