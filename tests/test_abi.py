"""CPU-side checks of the drop-in boundary: the C-ABI library loads, exports
every entry point include/rheogpu.h declares, and its structs have the layout
ctypes assumes.  No compute call is made (there may be no GPU)."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from rheotool_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def headers():
    return sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def test_library_exports_every_declared_symbol():
    lib = abi.load_library()
    for h in headers():
        for name in abi.header_symbols(h):
            assert hasattr(lib, name), f"{name} declared in {os.path.basename(h)} is not exported"


def test_header_constants_match_the_bindings():
    """Every integer #define of the headers (with or without a trailing
    comment) has the same value in abi.py."""
    seen = 0
    for h in headers():
        for name, val in re.findall(r"^#define\s+(RT_\w+)\s+(-?\d+)\s*(?:/\*.*)?$", open(h).read(), re.M):
            assert hasattr(abi, name), f"{name} missing from abi.py"
            assert getattr(abi, name) == int(val), name
            seen += 1
    assert seen > 10


def test_struct_layouts_match_the_c_compiler():
    from oracle import pyoracle
    L = pyoracle.lib()
    out = (C.c_int * 8)()
    L.or_abi_sizes(out)
    sizes = [C.sizeof(t) for t in (abi.rt_mesh_desc, abi.rt_bc_desc, abi.rt_model_params,
                                   abi.rt_solver_ctl, abi.rt_solver_perf, abi.rt_case_ctl,
                                   abi.rt_step_perf, abi.rt_thermo_desc)]
    assert list(out) == sizes


def test_status_strings():
    lib = abi.load_library()
    assert lib.rt_status_string(abi.RT_EINVAL) == b"RT_EINVAL"
    assert lib.rt_status_string(abi.RT_OK) == b"RT_OK"


def test_null_context_is_rejected():
    lib = abi.load_library()
    assert lib.rt_ctx_destroy(None) == abi.RT_EINVAL
    assert lib.rt_step(None, 1, None) == abi.RT_EINVAL
    assert lib.rt_ctx_create(None, 0) == abi.RT_EINVAL


def test_product_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "rheotool_gb300")
    for path in glob.glob(os.path.join(pkg, "**", "*"), recursive=True):
        if path.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            txt = open(path).read()
            for bad in ("pyoracle", "liboracle", "from oracle", "import oracle", "oracle.c"):
                assert bad not in txt, (path, bad)


def test_case_descriptors_roundtrip():
    from rheotool_gb300.case import cavity_case, contraction_case
    from rheotool_gb300.mesh import contraction_mesh
    c = cavity_case(6)
    md, bd, mp, ctl = c.descriptors()
    assert md.nCells == 36 and md.nPatches == 2 and list(md.solveDir) == [1, 1, 0]
    assert ctl.needReference == 1 and mp.model == abi.RT_MODEL_OLDROYDB_LOG
    c2 = contraction_case(contraction_mesh(4, 4, 2, 1, 2, 1.0, 1.0))
    md, bd, mp, ctl = c2.descriptors()
    assert ctl.needReference == 0 and mp.model == abi.RT_MODEL_GIESEKUS_LOG
    assert abs(mp.lambda_ - 2.0) < 1e-15 and abs(mp.etaS - 1 / 9) < 1e-15
