"""The reference's own tester programs run against the GPU library.

xdlutst (`lutst`, AtlasBase/Clint/atlas-tlp.base:1782-2260, built with
-DTimeC so it factors through clapack_dgetrf; residual threshold 100 at
:2203) and xdl3blastst (`l3blastst`, AtlasBase/Antoine/atlbinblas.base, built
with -DUSE_L3_REFERENCE so the trusted GEMM is the reference BLAS; threshold
50 at :11091) are extracted from the reference's basefiles and linked against
libatlas_gb300.so by oracle/ref_build.sh (oracle/_ref/xdlutst,
oracle/_ref/xdl3blastst).  Each case here runs one tester invocation as a
subprocess and requires the tester's own verdict: every case PASS, and for
xdlutst every printed residual at most 100.  The testers exist only where the
reference tree (or an extraction of it in oracle/_ref/src) was available when
the copy was built; elsewhere these tests skip."""
import os
import re
import subprocess

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFDIR = os.path.join(ROOT, "oracle", "_ref")
LU_THRESH = 100.0


def _run(prog, args, timeout=900):
    path = os.path.join(REFDIR, prog)
    if not os.access(path, os.X_OK):
        pytest.skip(f"{prog} not built: no reference tree or extraction where this copy was built")
    p = subprocess.run([path] + args, capture_output=True, text=True, timeout=timeout)
    print(p.stdout)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    return p.stdout


def _lu_rows(out):
    """(order, M, N, lda, npiv, resid) of every case line of xdlutst."""
    rows = []
    for line in out.splitlines():
        f = line.split()
        if len(f) == 9 and f[1] in ("Col", "Row"):
            rows.append((f[1], int(f[2]), int(f[3]), int(f[4]), int(f[5]), float(f[8])))
    return rows


@pytest.mark.parametrize("args,ncases", [
    (["-n", "8192", "-O", "1", "C"], 1),                                   # the headline factorization
    (["-N", "100", "1000", "300", "-O", "2", "C", "R"], 8),                 # square, both orders
    (["-M", "500", "500", "1", "-N", "300", "900", "600", "-O", "2", "C", "R"], 4),   # rectangular
])
def test_xdlutst_against_gpu_dgetrf(args, ncases):
    out = _run("xdlutst", args)
    rows = _lu_rows(out)
    assert len(rows) == ncases, out
    for (order, M, N, lda, npiv, resid) in rows:
        assert 0.0 <= resid <= LU_THRESH, (order, M, N, resid)
    assert f"ALL {ncases} CASES PASSED" in out


def _l3_verdict(out):
    m = re.search(r"(\d+) tests run, (\d+) passed", out)
    assert m, out
    return int(m.group(1)), int(m.group(2))


@pytest.mark.parametrize("args,ntests", [
    # the headline DGEMM: 1024^3 NoTrans/NoTrans, alpha 1, beta 0
    (["-R", "gemm", "-A", "1", "N", "-B", "1", "N", "-m", "1024", "-n", "1024", "-k", "1024",
      "-a", "1", "1.0", "-b", "1", "0.0"], 1),
    (["-R", "gemm", "-A", "2", "N", "T", "-B", "2", "N", "T", "-m", "333", "-n", "257", "-k", "129",
      "-a", "2", "1.0", "-0.5", "-b", "2", "0.0", "1.5"], 16),
    (["-R", "trsm", "-S", "2", "L", "R", "-U", "2", "L", "U", "-A", "2", "N", "T", "-D", "2", "N", "U",
      "-m", "300", "-n", "200", "-a", "1", "1.5"], 16),
    (["-R", "trmm", "-S", "2", "L", "R", "-U", "2", "L", "U", "-A", "2", "N", "T", "-D", "2", "N", "U",
      "-m", "300", "-n", "200", "-a", "1", "1.5"], 16),
    (["-R", "syrk", "-U", "2", "L", "U", "-A", "2", "N", "T", "-n", "300", "-k", "200",
      "-a", "1", "1.5", "-b", "1", "0.5"], 4),
])
def test_xdl3blastst_against_gpu_blas(args, ntests):
    out = _run("xdl3blastst", args + ["-F", "0"])
    run, passed = _l3_verdict(out)
    assert run == ntests and passed == ntests, out
