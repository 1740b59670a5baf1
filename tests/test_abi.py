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
])
def test_bad_argument_reports_and_exits(gb, call, param, rout):
    code = PRE + "A = np.zeros((4, 4), order='F'); p = np.zeros(4, dtype=np.int32); " + call
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
