"""Wavefront pipeline parity (GPU tests): the stage kernels draw the same Philox
numbers as the megakernel, so the two pipelines agree sample by sample up to
float rounding; the wavefront also matches the oracle path by path and the
reference's golden images statistically."""
import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import scene as S

from _util import load_golden, scene_from_golden, z_ok, zscores

pytestmark = pytest.mark.gpu

R = P.renderer


def _samples(scene, maxpl, pipeline, sampler=R.EM_CDF, spp=8, seed=31, rr=0, cap=0):
    cfg = P.Config(scene=scene, max_path_length=maxpl, em_sampler=sampler, pipeline=pipeline,
                   rr_min_path_length=rr, max_paths_in_flight=cap)
    with P.GpuPathTracer(cfg, seed=seed) as r:
        out = r.render_samples(R.kPathTracing, 0, spp)
        st = r.stats()
    return out, st


def _match(a, b, tol=1e-3):
    return float(np.mean(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b))))


@pytest.mark.parametrize("case", ["area", "area_rr", "env_cdf", "env_cos", "env_rr3"])
def test_wavefront_matches_megakernel(case):
    if case.startswith("area"):
        scene, maxpl, sampler = S.cornell_box(32, 32), (0 if case == "area_rr" else 8), R.EM_CDF
        rr = 0
    else:
        scene, maxpl = S.cornell_env(32, 32, 64, 32), 12
        sampler = R.EM_COSINE if case == "env_cos" else R.EM_CDF
        rr = 4 if case == "env_rr3" else 0
    a, sa = _samples(scene, maxpl, R.PIPELINE_MEGAKERNEL, sampler, rr=rr)
    b, sb = _samples(scene, maxpl, R.PIPELINE_WAVEFRONT, sampler, rr=rr)
    frac = _match(b, a)
    assert frac >= 0.995, "wavefront/megakernel sample match %.4f" % frac
    assert sa["paths"] == sb["paths"]
    # identical random decisions -> (nearly) identical ray counts
    assert abs(sa["extension_rays"] - sb["extension_rays"]) <= 1e-3 * sa["extension_rays"]
    assert abs(sa["shadow_rays"] - sb["shadow_rays"]) <= 1e-3 * sa["shadow_rays"]


def test_wavefront_small_capacity_chunks():
    # more paths than one wavefront chunk holds: chunks must not interfere
    scene = S.cornell_box(16, 16)
    a, _ = _samples(scene, 8, R.PIPELINE_WAVEFRONT, spp=6)
    b, _ = _samples(scene, 8, R.PIPELINE_MEGAKERNEL, spp=6)
    assert _match(a, b) >= 0.995


def test_multi_chunk_call_accumulates_every_chunk():
    # chunks of 2 samples per pixel: the call accumulates chunk k on a side stream while chunk
    # k + 1 renders into the other output set; the framebuffer is the mean of the same samples
    scene = S.cornell_box(16, 16)
    cfg = P.Config(scene=scene, max_path_length=8, max_paths_in_flight=2 * 16 * 16)
    with P.GpuPathTracer(cfg, seed=13) as r:
        samples = r.render_samples(R.kPathTracing, 0, 10)
        r.RunIteration(R.kPathTracing, 0, 10)
        r.RunIteration(R.kPathTracing, 10, 6)       # a second call reuses both output sets
        mean, var, n = r.framebuffer(with_variance=True)
        tail = r.render_samples(R.kPathTracing, 10, 6)
    assert n == 16
    want = np.concatenate([samples, tail]).astype(np.float64)
    assert np.allclose(mean, want.mean(axis=0), rtol=1e-6, atol=1e-7)
    assert np.allclose(var, want.var(axis=0, ddof=1), rtol=1e-4, atol=1e-7)


@pytest.mark.parametrize("name", ["cornell_area_32", "cornell_env_32_cdf"])
def test_wavefront_against_reference_golden(name):
    d, text, td = load_golden(name)
    scene = scene_from_golden(d)
    cfg = P.Config(scene=scene, max_path_length=int(d["max_path_length"]), pipeline=R.PIPELINE_WAVEFRONT)
    spp = max(16384, int(d["spp"]))   # the benchmark scenes' goldens: 65536 samples per pixel
    with P.GpuPathTracer(cfg, seed=77) as r:
        r.RunIteration(R.kPathTracing, 0, spp)
        mean, var, n = r.framebuffer(with_variance=True)
    frac, zm, zs = z_ok(zscores(mean, var / spp, d["mean"], d["var_mean"]))
    assert frac >= 0.999 and abs(zm) < 0.25 and 0.7 < zs < 1.3, (frac, zm, zs)


@pytest.mark.parametrize("sampler", [R.EM_STEERABLE, R.EM_CDF])
def test_small_calls_replay_a_render_graph(sampler):
    # Calls of up to 2^22 paths in one launch chunk (the reference's RunIteration pattern: one
    # sample per pixel per call) replay a captured graph of the chunk's launches, with the call's
    # first sample index set in its head node. The image is the one of the same samples launched
    # directly (pg3gpu_render_samples), summed per pixel in sample order: bit for bit.
    scene = S.cornell_env(48, 40, 128, 64)
    cfg = P.Config(scene=scene, max_path_length=12, rr_min_path_length=4, em_sampler=sampler)
    with P.GpuPathTracer(cfg, seed=3) as r:
        for k in range(12):
            r.RunIteration(R.kPathTracing, k, 1)
        r.RunIteration(R.kPathTracing, 12, 3)      # another sample count: captured anew
        r.RunIteration(R.kPathTracing, 15, 1)
        mean, var, n = r.framebuffer(with_variance=True)
        st = r.stats()
    with P.GpuPathTracer(cfg, seed=3) as d:
        samples = d.render_samples(R.kPathTracing, 0, 16).astype(np.float64)
    assert n == 16
    acc = np.zeros(samples.shape[1:])
    for k in range(16):
        acc += samples[k]
    assert np.array_equal(mean, acc / 16)
    assert st["paths"] == 16 * 48 * 40
    assert st["kernel_launches"] > 14 * 40      # every replay counts its stage launches
