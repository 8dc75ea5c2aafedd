"""rt_residual_noalloc: the residual entry point for callers that cannot
allocate device memory (a callback inside another library's Krylov loop, where
a cudaMalloc would synchronise the device mid-loop; a host whose device memory
is all owned by its own pool allocator).  The inputs live in device memory the test allocates; the
library allocates nothing and keeps its reduction scratch in a static device
array.  Its result must equal rt_residual's (host arrays) to the round-off of
a different reduction order, on two calls in a row (the second call reuses
the shared scratch left by the first).

The inputs are written on a stream of the caller's own, as such a caller
would: the call runs on the context's stream, so the caller completes the
writes on its stream first (here: synchronises that stream, not the device).
The library's device-memory counter is unchanged by the calls; a mesh above
the 2,097,152-cell limit and pointers that are not device memory of the
context's device are refused with RT_EINVAL before any kernel runs.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(mesh, seed):
    rng = np.random.default_rng(seed)
    F, N = mesh.nFaces, mesh.nCells
    phi = rng.normal(size=F) * mesh.magSf
    u = (phi >= 0).astype(float)
    g = mesh.magSf * mesh.deltaCoeffs * (1.0 + rng.random(F))
    lower = -u * phi - g
    upper = (1 - u) * phi - g
    diag = np.zeros(N)
    np.subtract.at(diag, mesh.owner, lower)
    np.subtract.at(diag, mesh.neighbour, upper)
    diag += 3.0 * mesh.V
    b = rng.normal(size=N) * mesh.V
    x = rng.normal(size=N)
    return diag, upper, lower, b, x


def _device_bytes(lib):
    n = C.c_int64()
    assert lib.rt_device_bytes(C.byref(n)) == 0
    return n.value


def test_residual_noalloc_matches_rt_residual():
    torch = pytest.importorskip("torch")
    from rheotool_gb300 import abi
    from rheotool_gb300.mesh import contraction_mesh
    from rheotool_gb300.runtime import Context

    mesh = contraction_mesh(10, 8, 6, 4, 5, 4.0, 4.0)
    ctx = Context(0)
    try:
        ctx.upload_mesh(mesh)
        side = torch.cuda.Stream(device="cuda:0")
        for call, seed in enumerate((101, 202)):
            diag, upper, lower, b, x = _system(mesh, seed)
            ref = ctx.residual(diag, upper, lower, b, x)
            with torch.cuda.stream(side):
                dev = [torch.tensor(a, dtype=torch.float64, device="cuda:0") for a in (diag, upper, lower, b, x)]
            side.synchronize()            # the caller's writes are complete; no device-wide sync
            before = _device_bytes(ctx.lib)
            out = C.c_double(-1.0)
            st = ctx.lib.rt_residual_noalloc(ctx._ctx, *[C.c_void_p(t.data_ptr()) for t in dev], C.byref(out))
            assert st == abi.RT_OK, ctx.lib.rt_last_error(ctx._ctx)
            assert _device_bytes(ctx.lib) == before
            assert ref > 0
            assert abs(out.value - ref) <= 1e-12 * ref, (call, out.value, ref)
        # host memory is not device memory: refused before any kernel runs
        diag, upper, lower, b, x = _system(mesh, 303)
        host = [np.ascontiguousarray(a) for a in (diag, upper, lower, b, x)]
        out = C.c_double(-1.0)
        st = ctx.lib.rt_residual_noalloc(ctx._ctx, *[C.c_void_p(a.ctypes.data) for a in host], C.byref(out))
        assert st == abi.RT_EINVAL
        assert b"not device memory" in ctx.lib.rt_last_error(ctx._ctx) or b"not a CUDA pointer" in \
            ctx.lib.rt_last_error(ctx._ctx)
        assert out.value == -1.0
    finally:
        ctx.close()


def test_residual_noalloc_refuses_meshes_above_its_limit():
    torch = pytest.importorskip("torch")
    from rheotool_gb300 import abi
    from rheotool_gb300.mesh import cavity_mesh
    from rheotool_gb300.runtime import Context

    mesh = cavity_mesh(1449)             # 2,099,601 cells > 2,097,152
    mesh.cellIJK = None                  # unstructured upload (the limit is about the cells)
    ctx = Context(0)
    try:
        ctx.upload_mesh(mesh)
        N, F = mesh.nCells, mesh.nFaces
        dev = [torch.zeros(n, dtype=torch.float64, device="cuda:0") for n in (N, F, F, N, N)]
        torch.cuda.synchronize()
        out = C.c_double(-1.0)
        st = ctx.lib.rt_residual_noalloc(ctx._ctx, *[C.c_void_p(t.data_ptr()) for t in dev], C.byref(out))
        assert st == abi.RT_EINVAL
        assert b"2097152" in ctx.lib.rt_last_error(ctx._ctx)
        assert out.value == -1.0
    finally:
        ctx.close()
