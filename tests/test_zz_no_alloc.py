"""The allocation-free entry point pg3gpu_run_iteration_noalloc (GPU).

Some callers cannot allocate device memory once they run -- a plugin inside a host
application or engine whose device memory belongs to that host's own allocator, or a
real-time loop with a fixed memory budget that must not run out of memory half-way
through a session. For them the library keeps the per-sample
radiance of a launch in a fixed scratch area compiled into it, and the caller
passes the output arrays. This test calls that entry point through the C ABI
twice in a row and checks the accumulated result against the regular entry point
(pg3gpu_run_iteration) on the same samples, with the tolerance the other
framebuffer tests use: on the area-light box, on the environment-map box with the
steerable sampler and roulette, and on an image large enough that one call runs
several launch chunks through the shared scratch area. It also checks that the
call refuses what the regular entry point refuses. It is collected last so that a
failure here stops a `-x` run only after every other test has run.
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


def _noalloc_render(cfg, calls, seed):
    """Runs the (iteration, spp) calls through the allocation-free entry point into caller-owned
    device arrays; returns the summed radiance and sum of squares as (h, w, 3) arrays."""
    import torch
    w, h = cfg.scene.camera.width, cfg.scene.camera.height
    out_sum = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
    out_sq = torch.zeros_like(out_sum)
    torch.cuda.synchronize()
    run = _noalloc()
    with P.GpuPathTracer(cfg, seed=seed) as r:
        for it, spp in calls:
            _lib.check(run(r._ctx, P.renderer.kPathTracing, it, spp, out_sum.data_ptr(), out_sq.data_ptr()), r._ctx)
        r.synchronize()
    return out_sum.cpu().numpy().reshape(h, w, 3), out_sq.cpu().numpy().reshape(h, w, 3)


def _regular_render(cfg, calls, seed):
    with P.GpuPathTracer(cfg, seed=seed) as r:
        for it, spp in calls:
            r.RunIteration(P.renderer.kPathTracing, it, spp)
        mean, var, n = r.framebuffer(with_variance=True)
    return mean, var, n


def test_noalloc_environment_map_steerable_matches_run_iteration():
    # the benchmark's sampler setup (steerable, projected weights, roulette from length 4) on a
    # small image: the same paths as the regular call on the megakernel pipeline, which is the
    # pipeline the allocation-free call runs
    calls = [(0, 3), (3, 5)]
    scene = S.cornell_env(32, 32, 128, 64)
    kw = dict(scene=scene, max_path_length=12, rr_min_path_length=4, em_sampler=P.renderer.EM_STEERABLE)
    got_sum, got_sq = _noalloc_render(P.Config(**kw), calls, seed=5)
    mean, var, n = _regular_render(P.Config(pipeline=P.renderer.PIPELINE_MEGAKERNEL, **kw), calls, seed=5)
    assert n == 8
    assert np.allclose(got_sum / 8, mean, rtol=1e-5, atol=1e-6)
    var_got = np.maximum(got_sq - 8 * (got_sum / 8) ** 2, 0) / 7
    assert np.allclose(var_got, var, rtol=1e-4, atol=1e-6)
    # against the default (wavefront) pipeline: the two pipelines draw the same random numbers
    # and differ only where float rounding flips a decision, in a small share of the samples
    mean_w, _, _ = _regular_render(P.Config(**kw), calls, seed=5)
    same = np.isclose(got_sum / 8, mean_w, rtol=1e-5, atol=1e-6).mean()
    assert same >= 0.97, same


def test_noalloc_several_launch_chunks_per_call():
    # 512 x 512 pixels: the 2^20-path scratch area holds 4 samples per pixel, so a call of 5 runs
    # two launch chunks that reuse the area (sample offsets 0..3, then 4), and the next call again
    calls = [(0, 5), (5, 2)]
    cfg = P.Config(scene=S.cornell_box(512, 512), max_path_length=8)
    got_sum, got_sq = _noalloc_render(cfg, calls, seed=9)
    cfg_m = P.Config(scene=S.cornell_box(512, 512), max_path_length=8, pipeline=P.renderer.PIPELINE_MEGAKERNEL)
    mean, var, n = _regular_render(cfg_m, calls, seed=9)
    assert n == 7
    assert np.allclose(got_sum / 7, mean, rtol=1e-5, atol=1e-6)
    var_got = np.maximum(got_sq - 7 * (got_sum / 7) ** 2, 0) / 6
    assert np.allclose(var_got, var, rtol=1e-4, atol=1e-6)


def test_noalloc_refuses_what_run_iteration_refuses():
    import torch
    # the SRA layered material: the path tracers refuse it (the reference stops with a fatal error)
    scene = S.cornell_mixed(16, 16, sra=True)
    out = torch.zeros(16 * 16 * 3, dtype=torch.float64, device="cuda")
    run = _noalloc()
    with P.GpuPathTracer(P.Config(scene=scene, max_path_length=6), seed=1) as r:
        for alg in (P.renderer.kPathTracing, P.renderer.kPathTracingNaive):
            st = run(r._ctx, alg, 0, 1, out.data_ptr(), out.data_ptr())
            assert st == _lib.ERR_UNSUPPORTED
            assert b"SRA" in _lib.load().pg3gpu_last_error(r._ctx)
            with pytest.raises(P.Pg3Error):
                r.RunIteration(alg, 0, 1)
        # a one-hit algorithm renders the material, like the regular call
        _lib.check(run(r._ctx, P.renderer.kDirectIllumMis, 0, 2, out.data_ptr(), out.data_ptr()), r._ctx)
        r.synchronize()
    assert float(out.sum()) > 0
    # splitting keeps per-thread frame stacks in device memory: refused
    cfg = P.Config(scene=S.cornell_box(16, 16), max_path_length=6, splitting_budget=4)
    with P.GpuPathTracer(cfg, seed=1) as r:
        st = run(r._ctx, P.renderer.kPathTracing, 0, 1, out.data_ptr(), out.data_ptr())
        assert st == _lib.ERR_UNSUPPORTED
