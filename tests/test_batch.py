"""Batched rendering (pg3gpu_batch_*): many scene instances on one persistent wavefront.

Every instance of a batch renders the same paths as a context created from its scene and
options (same pixel/sample/vertex keyed random numbers, same stage code), so its
framebuffer must equal that context's up to the order of the fp64 sums. The CPU tests cover
argument validation, which happens before any CUDA call.
"""
import ctypes

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import _lib, scene as S

R = P.renderer


def _variants(n, side=(16, 40), spp=(2, 5), base_seed=100):
    cfgs, spps = [], []
    for i in range(n):
        s, k = S.random_variant(base_seed + i, em_width=64, em_height=32, side_range=side, spp_range=spp,
                                max_spheres=4)
        cfgs.append(P.Config(scene=s, max_path_length=0, base_seed=7 + i))
        spps.append(k)
    return cfgs, spps


def _reference_images(cfgs, spps, runs=1):
    out = []
    for c, k in zip(cfgs, spps):
        with P.GpuPathTracer(c) as r:
            for run in range(runs):
                r.RunIteration(R.kPathTracing, run * k, k)
            out.append(r.framebuffer(with_variance=True))
    return out


def _create_raw(cfgs, spps):
    L = _lib.load()
    n = len(cfgs)
    descs = (_lib.SceneDesc * max(n, 1))(*[_lib.scene_desc(c.scene) for c in cfgs])
    opts = (_lib.Options * max(n, 1))(*[c.options() for c in cfgs])
    sp = (ctypes.c_uint32 * max(n, 1))(*spps)
    h = ctypes.c_void_p()
    st = L.pg3gpu_batch_create(descs, opts, sp, n, 0, ctypes.byref(h))
    if st == 0:
        L.pg3gpu_batch_destroy(h)
    return st, L.pg3gpu_batch_last_error(None).decode()


def test_batch_argument_validation():
    cfgs, spps = _variants(2)
    st, err = _create_raw([], [])
    assert st == _lib.ERR_INVALID_ARGUMENT and "instances" in err
    st, err = _create_raw(cfgs, [spps[0], 0])
    assert st == _lib.ERR_INVALID_ARGUMENT and "spp" in err
    cfgs[1].algorithm = R.kPathTracingNaive
    st, err = _create_raw(cfgs, spps)
    assert st == _lib.ERR_UNSUPPORTED and "algorithm 7" in err
    big = [cfgs[0]] * (_lib.BATCH_MAX_INSTANCES + 1)
    st, err = _create_raw(big, [1] * len(big))
    assert st == _lib.ERR_INVALID_ARGUMENT


def _assert_same(batch_img, ref_img):
    m_b, v_b, it_b = batch_img
    m_r, v_r, it_r = ref_img
    assert it_b == it_r
    scale = max(float(np.abs(m_r).max()), 1e-6)
    np.testing.assert_allclose(m_b, m_r, rtol=2e-6, atol=1e-7 * scale)
    # sums of squares: the single-scene accumulation adds squares of up to 32 samples in fp32
    # before going to fp64, the batch adds each sample's square in fp64
    np.testing.assert_allclose(v_b, v_r, rtol=1e-2, atol=1e-6 * max(float(v_r.max()), 1e-6))


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [1, 0])
def test_batch_matches_single_scene_contexts(use_graph):
    cfgs, spps = _variants(6)
    refs = _reference_images(cfgs, spps, runs=2)
    with P.GpuBatch(cfgs, spps) as b:
        b.set_tuning(use_graph=use_graph)
        b.run()
        b.run()
        b.synchronize()
        for i in range(len(cfgs)):
            _assert_same(b.framebuffer(i, with_variance=True), refs[i])
        st = b.stats()
        assert st["paths"] == 2 * sum(h * w * k for (h, w), k in zip(b.sizes, spps))


@pytest.mark.gpu
def test_batch_with_phong_smooth_materials_and_point_lights():
    # instances of different material kinds: the batch launches the shade kernels of every kind
    # that any instance holds (Phong, the smooth pair) next to the Lambert/GGX ones
    cfgs, spps = _variants(2, base_seed=500)
    cfgs.append(P.Config(scene=S.cornell_mixed(20, 20), max_path_length=0, base_seed=11))
    cfgs.append(P.Config(scene=S.cornell_mixed(24, 16, area=False), max_path_length=8, base_seed=12))
    spps += [3, 4]
    refs = _reference_images(cfgs, spps)
    with P.GpuBatch(cfgs, spps) as b:
        b.run()
        b.synchronize()
        for i in range(len(cfgs)):
            _assert_same(b.framebuffer(i, with_variance=True), refs[i])


@pytest.mark.gpu
def test_batch_slot_reuse_with_tiny_capacity():
    # 1024 slots for tens of thousands of paths: every slot is refilled many times and
    # instances of different sizes share the slots within one step
    cfgs, spps = _variants(5, side=(8, 48), spp=(1, 6), base_seed=300)
    refs = _reference_images(cfgs, spps)
    with P.GpuBatch(cfgs, spps) as b:
        for thr in (0.25, 0.875):
            b.clear()
            b.set_tuning(capacity=1024, regen_threshold=thr, block_size=128)
            b.run()
            b.synchronize()
            for i in range(len(cfgs)):
                _assert_same(b.framebuffer(i, with_variance=True), refs[i])


@pytest.mark.gpu
def test_batch_autotune_keeps_results_and_clears():
    cfgs, spps = _variants(4, base_seed=500)
    refs = _reference_images(cfgs, spps)
    with P.GpuBatch(cfgs, spps) as b:
        t = b.autotune(max_trials=6)
        assert t["block_size"] in (128, 256) and 0 < t["regen_threshold"] <= 0.875 and t["capacity"] >= 1024
        assert b.framebuffer(0)[2] == 0          # trial runs cleared
        b.run()
        b.synchronize()
        for i in range(len(cfgs)):
            _assert_same(b.framebuffer(i, with_variance=True), refs[i])
