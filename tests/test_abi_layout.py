"""The ctypes mirror of the C ABI structs has the C layout: a small C
program compiled against include/rheogpu.h prints sizeof and every field's
offsetof, which must equal the ctypes Structure's (no GPU needed; skipped
when no C compiler is present)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from rheotool_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CNAME = {"lambda_": "lambda"}   # Python keywords renamed in the mirror
STRUCTS = ["rt_mesh_desc", "rt_bc_desc", "rt_model_params", "rt_solver_ctl", "rt_solver_perf",
           "rt_case_ctl", "rt_step_perf"]


def test_struct_layouts_match_c(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rheogpu.h"', 'int main(void) {']
    for s in STRUCTS:
        st = getattr(abi, s)
        lines.append(f'printf("{s} sizeof %zu\\n", sizeof({s}));')
        for name, _ in st._fields_:
            lines.append(f'printf("{s} {name} %zu\\n", offsetof({s}, {CNAME.get(name, name)}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")
    for line in filter(None, out):
        s, name, v = line.split()
        st = getattr(abi, s)
        got = C.sizeof(st) if name == "sizeof" else getattr(st, name).offset
        assert got == int(v), (s, name, got, int(v))
