"""atlg_dlaswp_noalloc: the row-interchange entry point for callers that
cannot let a library allocate device memory (their own pool owns it, or they
cannot take the synchronisation of cudaMalloc/cudaFree).  Its scratch is a
fixed array in the library, so this checks, through the C ABI, that two calls
in a row give exactly the result of the allocating entry point
atlg_dlaswp_dev (a permutation: bit-exact), and that a call needing more than
the fixed scratch is refused before any work is queued.  The file is named to
be collected last."""
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


def test_noalloc_matches_allocating_laswp_twice(gb, ora):
    torch = pytest.importorskip("torch")
    L = gb.lib()
    rng = np.random.default_rng(7)
    for (m, n, k1, k2, inci, seed) in ((300, 17, 0, 300, 1, 11), (1000, 5, 3, 900, -1, 12)):
        A, piv, dA1, dA2, dpiv = _case(torch, ora, m, n, seed, rng)
        assert L.atlg_dlaswp_dev(n, dA1.data_ptr(), m, k1, k2, dpiv.data_ptr(), inci, m, None) == 0
        assert L.atlg_dlaswp_noalloc(n, dA2.data_ptr(), m, k1, k2, dpiv.data_ptr(), inci, m, None) == 0
        torch.cuda.synchronize()
        got = dA2.cpu().numpy().T
        assert np.array_equal(got, dA1.cpu().numpy().T)
        ref = A.copy(order="F")
        ora.laswp(n, ref, k1, k2, piv, inci)
        assert np.array_equal(got, ref)


def test_noalloc_rejects_sizes_beyond_its_scratch(gb):
    L = gb.lib()
    # 4096 rows x 600 columns need 19.7 MB > 16 MiB: refused before touching memory
    rc = L.atlg_dlaswp_noalloc(600, None, 4096, 0, 4096, None, 1, 4096, None)
    assert rc == -2
