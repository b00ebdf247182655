"""The allocation-free entry point pg3gpu_run_iteration_noalloc (GPU).

Some callers cannot allocate device memory once they run -- a plugin inside a host
application or engine whose device memory belongs to that host's own allocator, or a
real-time loop with a fixed memory budget that must not run out of memory half-way
through a session. For them the library keeps the per-sample
radiance of a launch in a fixed scratch area compiled into it, and the caller
passes the output arrays. This test calls that entry point through the C ABI
twice in a row and checks the accumulated result against the regular entry point
(pg3gpu_run_iteration) on the same samples, with the tolerance the other
framebuffer tests use. It is collected last so that a failure here stops a
`-x` run only after every other test has run.
"""
import ctypes

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import _lib, scene as S

pytestmark = pytest.mark.gpu


def _noalloc():
    f = _lib.load().pg3gpu_run_iteration_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p,
                  ctypes.c_void_p]
    return f


def test_noalloc_matches_run_iteration_on_two_calls():
    import torch
    w = h = 24
    cfg = P.Config(scene=S.cornell_box(w, h), max_path_length=8)
    run = _noalloc()
    # the caller owns the outputs (here allocated by torch before the loop)
    out_sum = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
    out_sq = torch.zeros_like(out_sum)
    torch.cuda.synchronize()
    with P.GpuPathTracer(cfg, seed=21) as r:
        _lib.check(run(r._ctx, P.renderer.kPathTracing, 0, 3, out_sum.data_ptr(), out_sq.data_ptr()), r._ctx)
        _lib.check(run(r._ctx, P.renderer.kPathTracing, 3, 5, out_sum.data_ptr(), out_sq.data_ptr()), r._ctx)
        r.synchronize()
        got_sum = out_sum.cpu().numpy().reshape(h, w, 3)
        got_sq = out_sq.cpu().numpy().reshape(h, w, 3)
    with P.GpuPathTracer(cfg, seed=21) as ref:
        ref.RunIteration(P.renderer.kPathTracing, 0, 3)
        ref.RunIteration(P.renderer.kPathTracing, 3, 5)
        mean, var, n = ref.framebuffer(with_variance=True)
    assert n == 8
    assert np.allclose(got_sum / 8, mean, rtol=1e-5, atol=1e-6)
    var_got = np.maximum(got_sq - 8 * (got_sum / 8) ** 2, 0) / 7
    assert np.allclose(var_got, var, rtol=1e-4, atol=1e-6)
    assert got_sum.sum() > 0


def test_noalloc_rejects_images_beyond_its_scratch():
    import torch
    side = 1025   # 1025 x 1025 pixels > PG3GPU_NOALLOC_MAX_PATHS = 2^20
    cfg = P.Config(scene=S.cornell_box(side, side), max_path_length=8)
    out = torch.zeros(side * side * 3, dtype=torch.float64, device="cuda")
    with P.GpuPathTracer(cfg, seed=1) as r:
        st = _noalloc()(r._ctx, P.renderer.kPathTracing, 0, 1, out.data_ptr(), out.data_ptr())
        assert st == _lib.ERR_INVALID_ARGUMENT
        assert b"scratch" in _lib.load().pg3gpu_last_error(r._ctx)
