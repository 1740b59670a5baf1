"""cblas_idamax / cblas_isamax through the C ABI, exactly: against the
reference's own ATL_i?amax results (fixtures: ties, zeros, infinities, NaN
runs, unit and strided; AtlasBase/Clint/atlas-lvl1.base:1148-1340) through
the host-pointer entry points, and against the oracle on device-resident
vectors long enough to span many CTAs, with the deciding elements placed on
chunk boundaries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fixture_cases(golden):
    for k in sorted(golden.files):
        if k.startswith("iamax_") and k.endswith("_meta"):
            pre, idx = k.split("_")[1:3]
            N, inc, res = (int(v) for v in golden[k])
            yield k, pre, golden[f"iamax_{pre}_{idx}_x"], N, inc, res


def test_host_iamax_matches_reference_fixtures(gb, golden):
    n = 0
    for k, pre, x, N, inc, res in _fixture_cases(golden):
        f = gb.cblas_idamax if pre == "d" else gb.cblas_isamax
        assert f(N, x, inc) == res, k
        n += 1
    assert n >= 100
    assert gb.status() == 0


def _dev(torch, gb, x, N, inc):
    L = gb.lib()
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    res = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    f = L.atlg_idamax_dev if x.dtype == np.float64 else L.atlg_isamax_dev
    assert f(N, dx.data_ptr(), inc, res.data_ptr(), None) == 0
    torch.cuda.synchronize()
    return int(res.item())


def test_device_iamax_matches_reference_fixtures(gb, golden):
    torch = pytest.importorskip("torch")
    for k, pre, x, N, inc, res in _fixture_cases(golden):
        if x.size == 0:
            continue
        assert _dev(torch, gb, x, N, inc) == res, k


def _long_cases(rng, n):
    nan = np.nan
    base = rng.standard_normal(n)
    out = []
    a = base.copy()                      # one maximum deep inside
    a[n // 3 + 5] = 50.0
    out.append(("single max", a))
    a = base.copy()                      # equal magnitudes in several chunks: the first wins
    for p in (n - 1, n // 2, 777777, 4095, 4096):
        a[p] = -60.0 if p % 2 else 60.0
    out.append(("ties", a))
    out.append(("all zero", np.zeros(n)))
    a = base.copy()                      # a NaN late, then an ordered value and a later maximum
    a[n - 5000] = nan
    a[n - 4999] = -0.5
    a[n - 10] = 9.0
    out.append(("nan then ordered", a))
    a = base.copy()                      # NaN, then an inverted run across many chunks
    p = 4096 * 3 - 2
    a[p] = nan
    a[p + 1] = 3.0                       # (P, Q) = (-3, 3): inverted
    run = -(3.0 - 1e-5 * np.arange(1, 40001))
    a[p + 2:p + 2 + run.size] = run      # shrinking negatives keep it inverted
    a[p + 2 + run.size:] = 0.0           # ordered again at the first zero, with m = 0 ...
    out.append(("nan inverted run", a))
    a = a.copy()
    a[n - 3] = 1e-30                     # ... and a later positive magnitude
    out.append(("nan inverted run, later max", a))
    a = base.copy()                      # several NaNs, the last one near the end
    a[[10, 99999, n - 2]] = nan
    out.append(("nan near the end", a))
    a = base.copy()
    a[[5, 9]] = [np.inf, -np.inf]
    out.append(("infinities", a))
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_device_iamax_long_vectors_match_oracle(gb, ora, dtype):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(99)
    n = (1 << 22) + 3
    for name, a in _long_cases(rng, n):
        x = a.astype(dtype)
        for inc in (1, 2):
            if inc == 2:
                buf = np.full(2 * (n - 1) + 1, 1e30, dtype=dtype)
                buf[::2] = x
            else:
                buf = x
            exp = ora.cblas_iamax(n, buf, inc)
            assert _dev(torch, gb, buf, n, inc) == exp, (name, inc)
    assert gb.status() == 0


def test_device_iamax_back_to_back_calls(gb, ora):
    """The merge counter is reset by each call: many calls in a row on one
    stream stay exact."""
    torch = pytest.importorskip("torch")
    L = gb.lib()
    rng = np.random.default_rng(5)
    n = 1 << 20
    xs = [rng.standard_normal(n) for _ in range(6)]
    dxs = [torch.from_numpy(x).cuda() for x in xs]
    res = torch.zeros(len(xs), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i, dx in enumerate(dxs):
        assert L.atlg_idamax_dev(n, dx.data_ptr(), 1, res.data_ptr() + 4 * i, None) == 0
    torch.cuda.synchronize()
    assert res.cpu().tolist() == [ora.cblas_iamax(n, x, 1) for x in xs]
