"""The C ABI library on the host (CPU tests, no kernel launches).

* libpg3gpu.so loads and exports every function include/pg3gpu.h declares;
* scene/option validation runs before any CUDA call and returns the documented
  statuses (the reference's fatal errors become status codes);
* the Python scene builders produce what the oracle/harness text format needs.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import _lib, scene as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pg3gpu.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg3gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = header_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) <= set(names)


def test_status_strings_and_version():
    L = _lib.load()
    assert L.pg3gpu_version().startswith(b"pg3gpu")
    assert L.pg3gpu_status_string(0) == b"ok"
    assert L.pg3gpu_status_string(2) == b"unsupported"


def _create(scene, **opt):
    L = _lib.load()
    desc = _lib.scene_desc(scene)
    cfg = P.Config(scene=scene, max_path_length=8)
    o = cfg.options()
    for k, v in opt.items():
        setattr(o, k, v)
    h = ctypes.c_void_p()
    st = L.pg3gpu_create(ctypes.byref(desc), ctypes.byref(o), 0, ctypes.byref(h))
    if st == 0:
        L.pg3gpu_destroy(h)
    return st, L.pg3gpu_last_error(None).decode()


@pytest.mark.parametrize("opt,status,msg", [
    (dict(splitting_budget=0), _lib.ERR_INVALID_ARGUMENT, "splitting budget"),
    (dict(splitting_budget=65), _lib.ERR_INVALID_ARGUMENT, "splitting budget"),
    (dict(splitting_level=1.5), _lib.ERR_INVALID_ARGUMENT, "splitting level"),
    (dict(light_to_bsdf_ratio=0.0), _lib.ERR_INVALID_ARGUMENT, "ratio"),
    (dict(indirect_clipping=-1.0), _lib.ERR_INVALID_ARGUMENT, "clipping"),
    (dict(algorithm=8), _lib.ERR_INVALID_ARGUMENT, "unknown algorithm"),
    (dict(min_path_length=9), _lib.ERR_INVALID_ARGUMENT, "min path length"),
    (dict(min_path_length=0), _lib.ERR_INVALID_ARGUMENT, "min_path_length"),
    (dict(max_path_length=0, min_path_length=2), _lib.ERR_INVALID_ARGUMENT, "Russian roulette"),
    (dict(em_sampler=9), _lib.ERR_INVALID_ARGUMENT, "sampler"),
])
def test_option_validation(opt, status, msg):
    st, err = _create(S.cornell_box(8, 8), **opt)
    assert st == status and msg in err, (st, err)


def test_scene_validation():
    s = S.cornell_box(8, 8)
    s.triangles[0] = (s.triangles[0][0], s.triangles[0][1], s.triangles[0][2], 999)
    st, err = _create(s)
    assert st == _lib.ERR_INVALID_ARGUMENT and "material" in err
    s = S.cornell_box(8, 8)
    s.spheres[0] = (s.spheres[0][0], -1.0, s.spheres[0][2])
    assert _create(s)[0] == _lib.ERR_INVALID_ARGUMENT
    s = S.cornell_box(8, 8)
    p = s.triangles[0][0]
    s.triangles[0] = (p, p, p, 0)                            # degenerate
    assert _create(s)[0] == _lib.ERR_INVALID_ARGUMENT
    s = S.cornell_box(8, 8)
    s.env_map = np.ones((4, 8, 3), np.float32)               # environment map + area lights: valid
    st, err = _create(s)
    assert st == _lib.ERR_CUDA and "device" in err           # (validation passed; no GPU here)
    for bad in (np.nan, np.inf, -1e-30):                     # map texels: finite and non-negative
        s = S.cornell_env(8, 8, 16, 8)
        s.env_map[3, 5, 1] = bad
        assert _create(s)[0] == _lib.ERR_INVALID_ARGUMENT, bad
    s = S.cornell_env(8, 8, 16, 8)
    s.env_map[3, 5, 1] = -0.0                                # negative zero is zero
    st, err = _create(s)
    assert st == _lib.ERR_CUDA and "device" in err
    s = S.cornell_box(0, 8)
    assert _create(s)[0] == _lib.ERR_INVALID_ARGUMENT


def test_phong_smooth_and_point_light_validation():
    s = S.cornell_mixed(8, 8)
    st, err = _create(s)
    assert st == _lib.ERR_CUDA and "device" in err           # valid (no GPU here)
    for kind, field, value, msg in [(S.MAT_PHONG, "phong_exponent", -1.0, "exponent"),
                                    (S.MAT_PHONG, "glossy", (0.1, -0.2, 0.1), "Phong reflectances"),
                                    (S.MAT_PHONG, "albedo", (np.inf, 0.2, 0.1), "Phong reflectances"),
                                    (S.MAT_SMOOTH_DIELECTRIC, "ior", np.nan, "refraction")]:
        s = S.cornell_mixed(8, 8)
        i = next(k for k, m in enumerate(s.materials) if m.kind == kind)
        setattr(s.materials[i], field, value)
        st, err = _create(s)
        assert st == _lib.ERR_INVALID_ARGUMENT and msg in err, (field, st, err)
    s = S.cornell_mixed(8, 8)
    s.point_lights[0] = ((0.0, np.nan, 0.5), (1.0, 1.0, 1.0))
    st, err = _create(s)
    assert st == _lib.ERR_INVALID_ARGUMENT and "point light" in err
    s = S.cornell_mixed(8, 8)
    s.materials[0].kind = 7
    st, err = _create(s)
    assert st == _lib.ERR_INVALID_ARGUMENT and "unknown kind" in err


def test_sra_layered_validation():
    s = S.cornell_mixed(8, 8, sra=True)
    st, err = _create(s, algorithm=5)
    assert st == _lib.ERR_CUDA and "device" in err           # valid (no GPU here)
    i = next(k for k, m in enumerate(s.materials) if m.kind == S.MAT_SRA_LAYERED)
    for field, value, msg in [("inner_kind", S.MAT_PHONG, "inner layer"), ("medium_thickness", -1.0, "medium"),
                              ("medium_attenuation", (0.0, np.nan, 1.0), "medium")]:
        s = S.cornell_mixed(8, 8, sra=True)
        setattr(s.materials[i], field, value)
        st, err = _create(s, algorithm=5)
        assert st == _lib.ERR_INVALID_ARGUMENT and msg in err, (field, st, err)
    assert "sra 0.05 1.51 1.000277 lambert" in S.cornell_mixed(8, 8, sra=True).to_text()


def test_phong_constructor_halves_diffuse_with_glossy_lobe():
    m = S.phong((0.8, 0.6, 0.4), (0.5, 0.5, 0.5), 90)
    assert m.albedo == (0.4, 0.3, 0.2) and m.glossy == (0.5, 0.5, 0.5) and m.phong_exponent == 90
    m = S.phong((0.8, 0.6, 0.4), (0.5, 0.5, 0.5), 90, use_glossy=False)
    assert m.albedo == (0.8, 0.6, 0.4) and m.glossy == (0.0, 0.0, 0.0)
    s = S.cornell_mixed(8, 8)
    assert s.num_lights == 3 and "point_light 0.0 0.0 0.6 20.0 20.0 20.0" in s.to_text()


def test_null_arguments():
    L = _lib.load()
    h = ctypes.c_void_p()
    assert L.pg3gpu_create(None, None, 0, ctypes.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert L.pg3gpu_run_iteration(None, 7, 0, 1) == _lib.ERR_INVALID_ARGUMENT
    assert L.pg3gpu_read_framebuffer(None, None, None, None) == _lib.ERR_INVALID_ARGUMENT
    assert L.pg3gpu_destroy(None) == _lib.ERR_INVALID_ARGUMENT


def test_valid_scene_without_gpu_reports_cuda_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    st, err = _create(S.cornell_box(8, 8))
    assert st == _lib.ERR_CUDA and "device" in err


def test_scene_builders():
    c1 = S.cornell_box(64, 64)
    assert len(c1.triangles) == 12 and len(c1.spheres) == 2 and len(c1.area_lights) == 2
    # every box wall faces inwards (normal towards the centre) and the light faces down
    for p0, p1, p2, mat in c1.triangles:
        n = np.cross(np.subtract(p1, p0), np.subtract(p2, p0))
        c = (np.array(p0) + p1 + p2) / 3
        assert np.dot(n, -c) > 0
    c2 = S.cornell_env(32, 32, 64, 32)
    assert len(c2.triangles) == 8 and c2.env_map.shape == (32, 64, 3) and c2.num_lights == 1
    text = c2.to_text(em_path="/x/em.bin", max_path_length=12)
    assert "background_em /x/em.bin" in text and text.strip().endswith("options pt 1 12")
    sky = S.synthetic_sky(128, 64, seed=1)
    assert np.isfinite(sky).all() and sky.min() >= 0
    assert np.array_equal(sky, S.synthetic_sky(128, 64, seed=1))


def test_env_map_file_roundtrip(tmp_path):
    em = np.random.default_rng(0).random((8, 16, 3)).astype(np.float32)
    p = str(tmp_path / "e.bin")
    S.write_env_map(p, em)
    assert np.array_equal(S.read_env_map(p), em)
