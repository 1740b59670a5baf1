"""The C ABI without a GPU: the library loads, exports every function that
include/atlas_gb300.h declares, and rejects bad arguments the way the
reference does (message on stderr, exit status -1) before touching a GPU."""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "atlas_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(cblas_\w+|clapack_\w+|atlg_\w+|dgesv_\w+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_reference_entry_points():
    names = declared_functions()
    for n in ("cblas_dgemm", "cblas_sgemm", "cblas_dtrsm", "clapack_dgetrf", "clapack_dgetrs",
              "clapack_dgesv", "clapack_sgetrf"):
        assert n in names


def test_library_exports_every_declared_symbol(gb):
    L = gb.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def _run(code):
    env = dict(os.environ)
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                          timeout=120)


PRE = ("import sys, numpy as np; sys.path.insert(0, %r); import atlas_gb300 as G; "
       % os.path.join(ROOT, "math-atlas_gb300"))


@pytest.mark.parametrize("call,param,rout", [
    ("G.cblas_dgemm(102, 111, 111, -1, 2, 2, 1.0, A, 4, A, 4, 0.0, A, 4)", 4, "cblas_dgemm"),
    ("G.cblas_dgemm(102, 111, 111, 4, 2, 2, 1.0, A, 3, A, 4, 0.0, A, 4)", 9, "cblas_dgemm"),
    ("G.cblas_dgemm(102, 119, 111, 4, 2, 2, 1.0, A, 4, A, 4, 0.0, A, 4)", 2, "cblas_dgemm"),
    ("G.cblas_dgemm(100, 111, 111, 4, 2, 2, 1.0, A, 4, A, 4, 0.0, A, 4)", 1, "cblas_dgemm"),
    ("G.cblas_dgemm(101, 111, 111, 4, 4, 2, 1.0, A, 4, A, 4, 0.0, A, 3)", 14, "cblas_dgemm"),
    ("G.cblas_dtrsm(102, 141, 121, 111, 131, 4, 4, 1.0, A, 3, A, 4)", 10, "cblas_dtrsm"),
    ("G.cblas_dtrsm(102, 141, 125, 111, 131, 4, 4, 1.0, A, 4, A, 4)", 3, "cblas_dtrsm"),
    ("G.clapack_dgetrf(102, 4, 4, A, 3, p)", 6, "clapack_dgetrf"),
    ("G.clapack_dgetrf(102, -1, 4, A, 4, p)", 2, "clapack_dgetrf"),
    ("G.clapack_dgesv(102, 4, -2, A, 4, p, A, 4)", 3, "clapack_dgesv"),
    ("G.clapack_dgetrs(102, 120, 4, 1, A, 4, p, A, 4)", 2, "clapack_dgetrs"),
    # the widened rows: AtlasBase/Clint/cblas.base:356-449 (syrk), :611-677 (trmm),
    # cblas-lvl2.base:21-93 (gemv), :273-357 (trsv), atlas-clp.base:115-452
    ("G.cblas_dsyrk(102, 125, 111, 4, 2, 1.0, A, 4, 0.0, A, 4)", 2, "cblas_dsyrk"),
    ("G.cblas_dsyrk(102, 121, 111, 4, 2, 1.0, A, 3, 0.0, A, 4)", 8, "cblas_dsyrk"),
    ("G.cblas_dsyrk(101, 121, 111, 4, 2, 1.0, A, 4, 0.0, A, 3)", 11, "cblas_dsyrk"),
    ("G.cblas_dtrmm(102, 140, 121, 111, 131, 4, 4, 1.0, A, 4, A, 4)", 2, "cblas_dtrmm"),
    ("G.cblas_dtrmm(102, 141, 121, 111, 131, 4, 4, 1.0, A, 3, A, 4)", 10, "cblas_dtrmm"),
    ("G.cblas_dgemv(102, 111, 4, 4, 1.0, A, 4, x, 0, 0.0, x, 1)", 9, "cblas_dgemv"),
    ("G.cblas_dgemv(102, 111, 4, 4, 1.0, A, 3, x, 1, 0.0, x, 1)", 7, "cblas_dgemv"),
    ("G.cblas_dgemv(102, 118, 4, 4, 1.0, A, 4, x, 1, 0.0, x, 1)", 2, "cblas_dgemv"),
    ("G.cblas_dtrsv(102, 121, 111, 133, 4, A, 4, x, 1)", 4, "cblas_dtrsv"),
    ("G.cblas_dtrsv(102, 121, 111, 131, 4, A, 4, x, 0)", 9, "cblas_dtrsv"),
    ("G.clapack_dpotrf(102, 125, 4, A, 4)", 2, "clapack_dpotrf"),
    ("G.clapack_dpotrf(102, 121, 4, A, 3)", 5, "clapack_dpotrf"),
    ("G.clapack_dpotrs(102, 121, 4, -1, A, 4, A, 4)", 4, "clapack_dpotrs"),
    ("G.clapack_dpotrs(102, 121, 4, 1, A, 4, A, 3)", 8, "clapack_dpotrs"),
    ("G.clapack_dposv(102, 121, 4, 1, A, 3, A, 4)", 6, "clapack_dposv"),
    ("G.clapack_dtrtri(102, 121, 130, 4, A, 4)", 3, "clapack_dtrtri"),
    ("G.clapack_dtrtri(102, 121, 131, 4, A, 3)", 6, "clapack_dtrtri"),
    ("G.clapack_dgetri(102, 4, A, 3, p)", 4, "clapack_dgetri"),
    ("G.dgesv_split(4, 1, A, 3, p, A, 4)", 4, "dgesv_split"),
])
def test_bad_argument_reports_and_exits(gb, call, param, rout):
    code = PRE + ("A = np.zeros((4, 4), order='F'); p = np.zeros(4, dtype=np.int32); x = np.zeros(4); "
                  + call)
    r = _run(code)
    assert r.returncode == 255, (r.returncode, r.stderr)
    assert f"Parameter {param} to routine {rout} was incorrect" in r.stderr


def test_quick_returns_need_no_gpu(gb):
    code = PRE + ("import numpy as np; A = np.ones((4, 4), order='F'); p = np.zeros(4, dtype=np.int32); "
                  "G.cblas_dgemm(102, 111, 111, 0, 4, 4, 1.0, A, 4, A, 4, 0.0, A, 4); "
                  "print(G.clapack_dgetrf(102, 0, 4, A, 4, p)); print(A.sum())")
    r = _run(code)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["0", "16.0"]
