"""The boundary from C: a C99 program that includes include/atlas_gb300.h,
takes the address of every function the header declares, links against
libatlas_gb300.so and runs calls that return before any device work
(cblas_i?amax with N < 2, clapack_dgetrf with N = 0).  No GPU needed."""
import os
import shutil
import subprocess

import pytest

from test_abi import declared_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "math-atlas_gb300")


def test_c_program_links_every_entry_point_and_runs(gb, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = declared_functions()
    src = ['#include <stdio.h>', '#include "atlas_gb300.h"', "int main(void) {",
           "  const void *fns[] = {"]
    src += [f"    (const void *){n}," for n in names]
    src += ["  };",
            "  double x[1] = {3.0};",
            "  float xs[1] = {3.0f};",
            "  int piv[1];",
            "  size_t i;",
            "  for (i = 0; i < sizeof fns / sizeof fns[0]; ++i) if (!fns[i]) return 2;",
            "  if (cblas_idamax(1, x, 1) != 0 || cblas_isamax(1, xs, 1) != 0) return 3;",
            "  if (cblas_idamax(5, x, -1) != 0) return 4;",
            "  if (clapack_dgetrf(CblasColMajor, 0, 0, x, 1, piv) != 0) return 5;",
            '  printf("%d\\n", (int)(sizeof fns / sizeof fns[0]));',
            "  return 0;", "}"]
    c = tmp_path / "abi.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "abi"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(c),
                        "-L", LIBDIR, "-latlas_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, (run.returncode, run.stderr)
    assert int(run.stdout.strip()) == len(names)
