#!/usr/bin/env python3
"""Generates the golden images in tests/golden/ from the reference renderer's
own code (oracle/_ref/pg3ref_* built by oracle/build_ref.py from the reference
sources). Run here, where the reference checkout exists; the fixtures are
committed so that tests on other machines need neither the reference nor its
build.

Each fixture ``<name>.npz`` holds
  scene_text   the scene in the oracle/harness text format (EM path placeholder)
  env_map      float32 [H, W, 3] or empty
  mean         float64 [h, w, 3]  mean over K*N reference iterations
  var_mean     float64 [h, w, 3]  variance of that mean (var of one renderer's mean / K)
  spp          K*N
and the options the scene was rendered with.
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from pg3render_gb300 import scene as S  # noqa: E402

CASES = {
    # name: (builder, max_path_length, em_sampler, algorithm, renderers, iterations)
    # the two benchmark scenes at 65536 samples per pixel (64 renderers x 1024 iterations)
    "cornell_area_32": (lambda: S.cornell_box(32, 32), 8, "cdf", "pt", 64, 1024),
    "cornell_area_32_naive": (lambda: S.cornell_box(32, 32), 8, "cdf", "ptn", 64, 128),
    "cornell_area_32_rr": (lambda: S.cornell_box(32, 32), 0, "cdf", "pt", 64, 128),
    "cornell_env_32_cdf": (lambda: S.cornell_env(32, 32, 64, 32), 12, "cdf", "pt", 64, 1024),
    "cornell_env_32_cos": (lambda: S.cornell_env(32, 32, 64, 32), 12, "cosine", "pt", 64, 128),
    # the environment-map benchmark scene with its full 1024x512 sky (sun lobes of 1-3 degrees,
    # peak 1e4 x the sky mean) at 64x64 pixels and 65536 samples per pixel (256 renderers x 256
    # iterations): the image the benchmark's own sampler setup (steerable, roulette) must match
    "cornell_env_64_sky1024_cdf": (lambda: S.cornell_env(64, 64, 1024, 512), 12, "cdf", "pt", 256, 256),
    # direct illumination, eye light, normal visualiser (one hit; src/direct_illumination.hxx,
    # src/eye_light.hxx, src/normal_visualiser.hxx)
    "cornell_area_32_dbs": (lambda: S.cornell_box(32, 32), 8, "cdf", "dbs", 64, 128),
    "cornell_area_32_dlsa": (lambda: S.cornell_box(32, 32), 8, "cdf", "dlsa", 64, 128),
    "cornell_area_32_dlss": (lambda: S.cornell_box(32, 32), 8, "cdf", "dlss", 64, 128),
    "cornell_area_32_dmis": (lambda: S.cornell_box(32, 32), 8, "cdf", "dmis", 64, 128),
    "cornell_env_32_dmis_cdf": (lambda: S.cornell_env(32, 32, 64, 32), 12, "cdf", "dmis", 64, 128),
    "cornell_env_32_dbs": (lambda: S.cornell_env(32, 32, 64, 32), 12, "cdf", "dbs", 64, 128),
    "cornell_area_32_el": (lambda: S.cornell_box(32, 32), 8, "cdf", "el", 16, 512),
    "cornell_area_32_nv": (lambda: S.cornell_box(32, 32), 8, "cdf", "nv", 16, 512),
    # splitting budget / level / light-to-BSDF ratio and indirect clipping (src/path_tracer.hxx:
    # 240-265, 400-402, 432-454); the first two are the reference's default options (-sb 4 -iic 16)
    "cornell_area_32_sb4_iic16": (lambda: S.cornell_box(32, 32), 0, "cdf", "pt", 64, 64, (4, 1.0, 1.0, 16.0)),
    "cornell_env_32_sb4_iic16": (lambda: S.cornell_env(32, 32, 64, 32), 0, "cdf", "pt", 64, 64, (4, 1.0, 1.0, 16.0)),
    "cornell_area_32_sb3_lvl05_r2": (lambda: S.cornell_box(32, 32), 8, "cdf", "pt", 64, 64, (3, 0.5, 2.0, 0.0)),
    # area lights and a background light in one scene (picking includes the background's estimate)
    "cornell_envarea_32_cdf": (lambda: S.cornell_env_area(32, 32, 64, 32), 12, "cdf", "pt", 64, 128),
    "cornell_envarea_32_dmis": (lambda: S.cornell_env_area(32, 32, 64, 32), 12, "cdf", "dmis", 64, 128),
    "cornell_areabg_32": (lambda: S.cornell_box_bg(32, 32), 8, "cdf", "pt", 64, 128),
    # Phong, smooth conductor and smooth dielectric materials and a point light
    # (src/materials.hxx:353-780, src/lights.hxx:232-343); glossy lobes and caustics are
    # heavy-tailed: 256 renderers for the per-pixel variance of the mean
    "cornell_mixed_32": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "pt", 256, 128),
    "cornell_mixed_32_rr": (lambda: S.cornell_mixed(32, 32), 0, "cdf", "pt", 256, 128),
    "cornell_mixed_32_point": (lambda: S.cornell_mixed(32, 32, area=False), 8, "cdf", "pt", 256, 128),
    "cornell_mixed_32_naive": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "ptn", 256, 128),
    "cornell_mixed_32_dmis": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "dmis", 256, 128),
    "cornell_mixed_32_dlsa": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "dlsa", 256, 128),
    "cornell_mixed_32_dlss": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "dlss", 256, 128),
    "cornell_mixed_32_dbs": (lambda: S.cornell_mixed(32, 32), 8, "cdf", "dbs", 256, 128),
    "cornell_mixed_32_sb4_iic16": (lambda: S.cornell_mixed(32, 32), 0, "cdf", "pt", 256, 64, (4, 1.0, 1.0, 16.0)),
    "cornell_envmixed_32_cdf": (lambda: S.cornell_env_mixed(32, 32, 64, 32), 12, "cdf", "pt", 256, 128),
    "cornell_mixedsra_32_dmis": (lambda: S.cornell_mixed(32, 32, sra=True), 8, "cdf", "dmis", 256, 128),
    "cornell_mixedsra_32_dbs": (lambda: S.cornell_mixed(32, 32, sra=True), 8, "cdf", "dbs", 256, 128),
}

# The reference's own built-in scenes (Scene::LoadCornellBox, -s ids of src/config.hxx:45-115):
# the reference renders the scene it builds itself, the tests render pg3render_gb300.presets' build
# name: (scene id, max_path_length, algorithm, renderers, iterations)
PRESET_CASES = {
    "preset_00": (0, 8, "pt", 64, 128),      # point light, Phong diffuse box
    "preset_01": (1, 8, "pt", 256, 128),     # point light, Phong glossy box
    "preset_03": (3, 8, "pt", 64, 128),      # ceiling light, glossy
    "preset_05": (5, 8, "pt", 256, 128),      # light box, glossy
    "preset_07": (7, 8, "pt", 64, 128),      # constant environment, glossy
    "preset_12": (12, 8, "pt", 64, 128),     # point + light box + environment
    "preset_16": (16, 8, "pt", 256, 128),    # point light, smooth conductor spheres
    "preset_19": (19, 8, "pt", 256, 128),     # light box, smooth conductors, glossy walls
    "preset_29": (29, 8, "pt", 64, 128),     # environment, rectangles, GGX dielectric
    "preset_31": (31, 8, "pt", 256, 128),    # light box, smooth dielectric sphere in the box
    "preset_38": (38, 8, "pt", 256, 128),     # layered sphere (GGX dielectric around a GGX conductor)
    "preset_12_dmis": (12, 8, "dmis", 64, 128),
    # the SRA layered sphere: the reference renders it with the one-hit algorithms only
    "preset_27_dmis": (27, 8, "dmis", 64, 128),
    "preset_27_dlss": (27, 8, "dlss", 64, 128),
}

EM_TOKEN = "@EM@"


def make(name):
    build, maxpl, sampler, alg, K, N = CASES[name][:6]
    splitting = CASES[name][6] if len(CASES[name]) > 6 else None
    scene = build()
    with tempfile.TemporaryDirectory() as td:
        em_path = os.path.join(td, "em.bin")
        if scene.env_map is not None:
            scene.write_env_map(em_path)
        text = scene.to_text(em_path=em_path, algorithm=alg, max_path_length=maxpl, splitting=splitting)
        r = O.reference_render(text, renderers=K, iters=N, seed=4321, em_sampler=sampler)
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        scene_text=np.array(text.replace(em_path, EM_TOKEN)),
        env_map=(scene.env_map if scene.env_map is not None else np.zeros((0, 0, 3), np.float32)),
        mean=r["mean"], var_mean=r["var_of_renderer_mean"] / K, spp=np.array(K * N),
        max_path_length=np.array(maxpl), em_sampler=np.array(sampler), algorithm=np.array(alg),
        splitting=np.array(splitting if splitting is not None else (1, 1.0, 1.0, 0.0), np.float64))
    print(name, "done", r["timing"])


def make_preset(name):
    from pg3render_gb300 import presets as PR
    sid, maxpl, alg, K, N = PRESET_CASES[name]
    scene = PR.reference_scene(sid, 32, 32)
    text = scene.to_text(algorithm=alg, max_path_length=maxpl)
    opts = "options %s 1 %d\n" % (alg, maxpl)
    r = O.reference_render(opts, renderers=K, iters=N, seed=4321, extra=("--preset", str(sid), "32", "32", "0"))
    np.savez_compressed(
        os.path.join(HERE, name + ".npz"),
        scene_text=np.array(text), env_map=np.zeros((0, 0, 3), np.float32),
        mean=r["mean"], var_mean=r["var_of_renderer_mean"] / K, spp=np.array(K * N),
        max_path_length=np.array(maxpl), em_sampler=np.array("cdf"), algorithm=np.array(alg),
        splitting=np.array((1, 1.0, 1.0, 0.0), np.float64))
    print(name, "done", r["timing"])


def make_image_writer():
    """image_writer.npz: one reference renderer's framebuffer (16x12 Cornell box, 4 iterations)
    and the files the reference's own Framebuffer::SaveBMP (gamma 2.2) and SaveHDR wrote from it."""
    scene = S.cornell_box(16, 12)
    text = scene.to_text(max_path_length=8)
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for ext in ("bmp", "hdr"):
            p = os.path.join(td, "img." + ext)
            O.reference_render(text, renderers=1, iters=4, seed=777, extra=("--save-image", p))
            with open(p, "rb") as f:
                out[ext] = np.frombuffer(f.read(), np.uint8).copy()
            out["fb_" + ext] = np.fromfile(p + ".fb", np.float64).reshape(12, 16, 3)
    assert np.array_equal(out["fb_bmp"], out["fb_hdr"])
    np.savez_compressed(os.path.join(HERE, "image_writer.npz"), framebuffer=out["fb_bmp"], bmp=out["bmp"],
                        hdr=out["hdr"])
    print("image_writer done")


def make_emssd():
    """emssd_ref.npz: steerable-sampler data files the reference itself wrote
    (EnvironmentMapSteerableSampler::SaveToDisk, run by its Init on a map without a cached file)
    for the 64x32 sky of the environment-map box: a uniform triangulation (minimum = maximum
    subdivision level 2) and an adaptive one (levels 1-3, approximation error 0.05), with the
    file names the reference chose and the map they were built from."""
    scene = S.cornell_env(16, 16, 64, 32)
    out = {"env_map": scene.env_map.astype(np.float32)}
    for key, params in (("uniform", ("5", "2", "2")), ("adaptive", ("0.05", "1", "3"))):
        with tempfile.TemporaryDirectory() as td:
            em_path = os.path.join(td, "em.bin")
            scene.write_env_map(em_path)
            text = scene.to_text(em_path=em_path, algorithm="pt", max_path_length=4)
            O.reference_render(text, renderers=1, iters=1, seed=1, em_sampler="steerable",
                               extra=("--em-params",) + params)
            files = [f for f in os.listdir(td) if f.endswith(".emssd")]
            assert len(files) == 1, files
            with open(os.path.join(td, files[0]), "rb") as f:
                out[key] = np.frombuffer(f.read(), np.uint8).copy()
            out[key + "_name"] = np.array(files[0])
    np.savez_compressed(os.path.join(HERE, "emssd_ref.npz"), **out)
    print("emssd_ref done", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    for extra, fn in (("image_writer", make_image_writer), ("emssd", make_emssd)):
        if extra in sys.argv[1:]:
            fn()
            sys.argv.remove(extra)
            if len(sys.argv) == 1:
                sys.exit(0)
    names = sys.argv[1:] or (list(CASES) + list(PRESET_CASES))
    for n in [x for x in names if x in PRESET_CASES]:
        make_preset(n)
    for n in [x for x in names if x not in PRESET_CASES]:
        make(n)
