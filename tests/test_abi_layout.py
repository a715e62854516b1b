"""The ctypes mirrors in tailor_gb300/_lib.py against the C ABI header: a C
program compiled with gcc from include/tailor_gb300.h prints the size of
every struct and the offset of every field the Python side declares, and
both sides must agree (a field added on one side only would shift every
later field).  Needs gcc, no GPU."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

from tailor_gb300 import _lib as L

ROOT = Path(__file__).resolve().parents[1]
PAIRS = [
    ("tlr_recipe", L.Recipe), ("tlr_rule", L.Rule), ("tlr_metric_diag", L.MetricDiag),
    ("tlr_deriv_diag", L.DerivDiag), ("tlr_operator_diag", L.OperatorDiag),
    ("tlr_bc_diag", L.BcDiag), ("tlr_solve_opts", L.SolveOpts), ("tlr_eig_diag", L.EigDiag),
    ("tlr_grid_class", L.GridClass), ("tlr_sweep_point", L.SweepPoint),
    ("tlr_sweep_opts", L.SweepOpts), ("tlr_sweep_diag", L.SweepDiag),
    ("tlr_symbolic_info", L.SymbolicInfo),
]


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "tailor_gb300.h"',
             "int main(void) {"]
    for cname, py in PAIRS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("abi")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run([gcc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}


@pytest.mark.parametrize("cname,py", PAIRS, ids=[c for c, _ in PAIRS])
def test_struct_layout_matches_the_header(c_layout, cname, py):
    assert ctypes.sizeof(py) == c_layout[(cname, "size")], cname
    for fname, _ in py._fields_:
        assert getattr(py, fname).offset == c_layout[(cname, fname)], (cname, fname)
