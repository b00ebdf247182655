"""The reference-side renderer class (pg3render_gb300/shim/gpu_path_tracer.hxx) compiled against
the reference's own headers, in the reference's own program flow.

``oracle/_ref/pg3render_gpu`` (built by oracle/build_ref.py) parses the reference's command
line with the reference's Config, builds the scene with the reference's Scene::LoadCornellBox,
creates GpuPathTracer (an AbstractRenderer, src/renderer.hxx:232-278) and calls
RunIteration(algorithm, iteration) once per iteration, as Render() does
(src/pg3render.cxx:84-128); the image comes back through AbstractRenderer::GetFramebuffer.

* CPU: the scene GpuPathTracer translates from the reference's objects equals the library's
  own restatement of the same built-in scene (pg3render_gb300.presets), for all 39 -s ids.
* GPU: the images of that program z-test against the reference renderer's goldens of the
  same scenes, and batching the iterations (RunIterations) changes nothing.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from pg3render_gb300 import presets as PR
from pg3render_gb300 import scene as S

from _util import load_golden, z_ok, zscores

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "oracle", "_ref", "pg3render_gpu")

needs_exe = pytest.mark.skipif(not os.path.exists(EXE), reason="reference headers not available: "
                               "oracle/_ref/pg3render_gpu is not built")


def _dump(sid, tmp_path, w=32, h=32):
    p = str(tmp_path / ("scene%d.json" % sid))
    subprocess.run([EXE, "-s", str(sid), "-q", "--res", str(w), str(h), "--dump-scene", p], check=True,
                   capture_output=True)
    with open(p) as f:
        return json.load(f)


def _close(a, b, rtol=1e-6, atol=1e-7):
    return np.allclose(np.asarray(a, np.float64), np.asarray(b, np.float64), rtol=rtol, atol=atol)


@needs_exe
@pytest.mark.parametrize("sid", range(39))
def test_translated_scene_equals_the_restated_preset(sid, tmp_path):
    d = _dump(sid, tmp_path)
    ref = PR.reference_scene(sid, 32, 32)
    cam = ref.camera
    assert _close(d["camera"]["position"], cam.position) and _close(d["camera"]["forward"], cam.forward / np.linalg.norm(cam.forward))
    up = np.asarray(cam.up, np.float64)
    f = np.asarray(cam.forward, np.float64) / np.linalg.norm(cam.forward)
    up_perp = up - f * (up @ f)
    assert _close(d["camera"]["up"], up_perp / np.linalg.norm(up_perp), rtol=1e-5, atol=1e-5)
    assert (d["camera"]["width"], d["camera"]["height"]) == (32, 32)
    assert abs(d["camera"]["hfov_deg"] - cam.hfov_deg) < 1e-4

    assert len(d["materials"]) == len(ref.materials)
    for got, m in zip(d["materials"], ref.materials):
        assert got["kind"] == m.kind
        if m.kind in (S.MAT_LAMBERT, S.MAT_PHONG):
            assert _close(got["albedo"], m.albedo)
        if m.kind == S.MAT_PHONG:
            assert _close(got["glossy"], m.glossy) and _close(got["phong_exponent"], m.phong_exponent)
        if m.kind in (S.MAT_GGX_CONDUCTOR, S.MAT_GGX_DIELECTRIC, S.MAT_SRA_LAYERED):
            assert _close(got["alpha"], min(max(m.alpha, 0.001), 1.0))
        if m.kind not in (S.MAT_LAMBERT, S.MAT_PHONG):
            assert _close(got["ior"], m.ior / m.ior_outer)
        if m.kind in (S.MAT_GGX_CONDUCTOR, S.MAT_SMOOTH_CONDUCTOR):
            assert _close(got["absorb"], m.absorb)
        if m.kind == S.MAT_SRA_LAYERED:
            assert got["inner_kind"] == m.inner_kind
            assert _close(got["medium_attenuation"], m.medium_attenuation)
            assert _close(got["medium_thickness"], m.medium_thickness)

    assert len(d["triangles"]) == len(ref.triangles)
    for got, (p0, p1, p2, mat) in zip(d["triangles"], ref.triangles):
        assert _close(got["p"], np.concatenate([p0, p1, p2])) and got["material"] == mat
    assert len(d["spheres"]) == len(ref.spheres)
    for got, (c, r, mat) in zip(d["spheres"], ref.spheres):
        assert _close(got["center"], c) and _close(got["radius"], r) and got["material"] == mat

    # light order may differ (picking is by contribution; the ids only name the lights)
    got_area = {a["triangle"]: a["radiance"] for a in d["area_lights"]}
    ref_area = {t: rad for t, rad in ref.area_lights}
    assert sorted(got_area) == sorted(ref_area)
    for t in ref_area:
        assert _close(got_area[t], ref_area[t], rtol=1e-5)
    assert len(d["point_lights"]) == len(ref.point_lights)
    for got, (pos, power) in zip(d["point_lights"], ref.point_lights):
        assert _close(got["position"], pos) and _close(got["power"], power, rtol=1e-5)
    if ref.env_map is not None:
        assert d["background"] == 2
    elif ref.background_const is not None:
        assert d["background"] == 1 and _close(d["background_radiance"], ref.background_const)
    else:
        assert d["background"] == 0


def _render(sid, iters, tmp_path, batch=1, algorithm="pt", extra=()):
    out = str(tmp_path / ("img%d_%d.bin" % (sid, batch)))
    res = subprocess.run([EXE, "-s", str(sid), "-a", algorithm, "-minpl", "1", "-maxpl", "8", "-sb", "1", "-iic", "0",
                          "-i", str(iters), "-q", "--res", "32", "32", "--out", out, "--batch", str(batch)]
                         + list(extra), check=True, capture_output=True, text=True)
    timing = json.loads(res.stdout.strip().splitlines()[-1])
    with open(out, "rb") as f:
        w, h, n = np.frombuffer(f.read(12), np.uint32)
        mean = np.frombuffer(f.read(int(w * h * 3) * 8), np.float64).reshape(h, w, 3)
        var = np.frombuffer(f.read(int(w * h * 3) * 8), np.float64).reshape(h, w, 3)
    return mean, var, int(n), timing


@needs_exe
@pytest.mark.gpu
@pytest.mark.parametrize("name", ["preset_03", "preset_07", "preset_12", "preset_16", "preset_29", "preset_38"])
def test_reference_program_with_gpu_renderer_matches_golden(name, tmp_path):
    d, text, td = load_golden(name)
    sid = int(name.split("_")[1])
    iters = 8192
    mean, var, n, timing = _render(sid, iters, tmp_path)
    assert n == iters and timing["iterations"] == iters
    z = zscores(mean, var / n, d["mean"], d["var_mean"])
    frac, zm, zs = z_ok(z, stochastic=(var / n + d["var_mean"]) > 1e-10 * d["mean"] ** 2)
    assert frac >= 0.999 and abs(zm) < 0.25 and 0.7 < zs < 1.3, (name, frac, zm, zs)


@needs_exe
@pytest.mark.gpu
def test_batched_iterations_equal_per_iteration_calls(tmp_path):
    a, va, na, _ = _render(3, 96, tmp_path, batch=1)
    b, vb, nb, _ = _render(3, 96, tmp_path, batch=32)
    assert na == nb == 96
    assert np.allclose(a, b, rtol=1e-12, atol=0) and np.allclose(va, vb, rtol=1e-9, atol=1e-15)


@needs_exe
@pytest.mark.gpu
def test_one_hit_algorithm_through_the_reference_program(tmp_path):
    d, text, td = load_golden("preset_12_dmis")
    mean, var, n, _ = _render(12, 4096, tmp_path, algorithm="dmis")
    z = zscores(mean, var / n, d["mean"], d["var_mean"])
    frac, zm, zs = z_ok(z, stochastic=(var / n + d["var_mean"]) > 1e-10 * d["mean"] ** 2)
    assert frac >= 0.999, (frac, zm, zs)
