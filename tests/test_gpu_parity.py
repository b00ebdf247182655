"""Parity of the CUDA path with the oracle and with the reference (GPU tests).

* path by path: the CUDA kernels and the C++ oracle draw the same Philox
  numbers, so each sample's radiance must agree up to float rounding (a few
  paths may take another branch after a rounding difference);
* against the reference: golden images rendered by the reference's own code
  (tests/golden) must agree per pixel, |z| <= 4 on >= 99.9% of pixel channels.
"""
import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import scene as S

from _util import load_golden, scene_from_golden, z_ok, zscores

pytestmark = pytest.mark.gpu

GOLDEN_CASES = ["cornell_area_32", "cornell_area_32_naive", "cornell_area_32_rr",
                "cornell_env_32_cdf", "cornell_env_32_cos",
                "cornell_area_32_dbs", "cornell_area_32_dlsa", "cornell_area_32_dlss", "cornell_area_32_dmis",
                "cornell_env_32_dmis_cdf", "cornell_env_32_dbs", "cornell_area_32_el", "cornell_area_32_nv",
                "cornell_area_32_sb4_iic16", "cornell_env_32_sb4_iic16", "cornell_area_32_sb3_lvl05_r2",
                "cornell_envarea_32_cdf", "cornell_envarea_32_dmis", "cornell_areabg_32",
                "cornell_mixed_32", "cornell_mixed_32_rr", "cornell_mixed_32_point", "cornell_mixed_32_naive",
                "cornell_mixed_32_dmis", "cornell_mixed_32_dlsa", "cornell_mixed_32_dlss", "cornell_mixed_32_dbs",
                "cornell_mixed_32_sb4_iic16", "cornell_envmixed_32_cdf",
                # the reference's own built-in scenes (-s ids), built here by pg3render_gb300.presets
                "preset_00", "preset_01", "preset_03", "preset_05", "preset_07", "preset_12", "preset_16",
                "preset_19", "preset_29", "preset_31", "preset_38", "preset_12_dmis",
                # the SRA layered material (one-hit algorithms, as in the reference)
                "preset_27_dmis", "preset_27_dlss", "cornell_mixedsra_32_dmis", "cornell_mixedsra_32_dbs"]
VISUALISERS = ("cornell_area_32_el", "cornell_area_32_nv")
# the reference's acronyms of its algorithm ids (src/config.hxx:147-170)
ALG_IDS = {"el": 0, "nv": 1, "dbs": 2, "dlsa": 3, "dlss": 4, "dmis": 5, "ptn": 6, "pt": 7}
SAMPLERS = {"cdf": P.renderer.EM_CDF, "cosine": P.renderer.EM_COSINE}

# Path-by-path tolerance: per sample and channel |gpu - oracle| <= 1e-3 * max(1, |oracle|)
# for at least 99% of the samples (the rest may have taken another branch).
REL_TOL = 1e-3
MIN_MATCH = 0.99


def _cfg(scene, maxpl, alg=P.renderer.kPathTracing, sampler=P.renderer.EM_CDF, **kw):
    return P.Config(scene=scene, algorithm=alg, max_path_length=maxpl, em_sampler=sampler, **kw)


def _oracle_samples(scene, text, spp, seed, sampler=0, rr=0):
    import oracle as O
    o = O.render(text, scene.camera.width, scene.camera.height, seed=seed, spp=spp, em_sampler=sampler,
                 rr_min_path_length=rr, per_sample=True)
    return o["samples"]


def _match_fraction(g, o):
    ok = np.abs(g - o) <= REL_TOL * np.maximum(1.0, np.abs(o))
    return float(ok.mean())


@pytest.mark.parametrize("alg", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("env", [False, True])
def test_one_hit_algorithms_path_by_path(alg, env, tmp_path):
    """Eye light, normal visualiser and the four direct-illumination estimators against the
    oracle, sample by sample (same Philox numbers), on the area-light and the map scene."""
    scene = S.cornell_env(24, 24, 64, 32) if env else S.cornell_box(24, 24)
    em = str(tmp_path / "em.bin")
    if env:
        scene.write_env_map(em)
    names = ["el", "nv", "dbs", "dlsa", "dlss", "dmis"]
    text = scene.to_text(em_path=em, algorithm=names[alg], max_path_length=8)
    seed = 31
    with P.GpuPathTracer(_cfg(scene, 8, alg, P.renderer.EM_CDF), seed=seed) as r:
        g = r.render_samples(alg, 0, 8)
    o = _oracle_samples(scene, text, 8, seed, 0)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac
    assert np.isfinite(g).all() and g.max() > 0


@pytest.mark.parametrize("split", [(4, 1.0, 1.0, 16.0, 0), (3, 0.5, 2.0, 0.0, 8), (1, 1.0, 1.0, 2.0, 8),
                                   (2, 1.0, 1.0, 0.0, 0)])
@pytest.mark.parametrize("env", [False, True])
def test_splitting_and_clipping_path_by_path(split, env, tmp_path):
    """The recursive estimator (splitting budget, level, light-to-BSDF ratio, indirect clipping;
    roulette when the max path length is 0) against the oracle, sample by sample."""
    budget, level, ratio, clip, maxpl = split
    scene = S.cornell_env(24, 24, 64, 32) if env else S.cornell_box(24, 24)
    em = str(tmp_path / "em.bin")
    if env:
        scene.write_env_map(em)
    text = scene.to_text(em_path=em, max_path_length=maxpl, splitting=(budget, level, ratio, clip))
    seed = 41
    cfg = _cfg(scene, maxpl, P.renderer.kPathTracing, P.renderer.EM_CDF, splitting_budget=budget,
               splitting_level=level, light_to_bsdf_ratio=ratio, indirect_illum_clipping=clip)
    with P.GpuPathTracer(cfg, seed=seed) as r:
        g = r.render_samples(P.renderer.kPathTracing, 0, 4)
        st = r.stats()
    o = _oracle_samples(scene, text, 4, seed, 0)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac
    assert st["paths"] == 24 * 24 * 4 and np.isfinite(g).all()


@pytest.mark.parametrize("case", ["area", "area_naive", "env_cdf", "env_cos", "envarea_cdf", "envarea_cos",
                                  "areabg", "areabg_naive"])
def test_path_by_path_vs_oracle(case, tmp_path):
    if case.startswith("areabg"):
        scene = S.cornell_box_bg(24, 24)
        maxpl, sampler = 8, 0
    elif case.startswith("area"):
        scene = S.cornell_box(24, 24)
        maxpl, sampler = 8, 0
    elif case.startswith("envarea"):
        scene = S.cornell_env_area(24, 24, 64, 32)
        maxpl, sampler = 12, (0 if case.endswith("cdf") else 1)
    else:
        scene = S.cornell_env(24, 24, 64, 32)
        maxpl, sampler = 12, (0 if case == "env_cdf" else 1)
    alg = P.renderer.kPathTracingNaive if case.endswith("naive") else P.renderer.kPathTracing
    em = str(tmp_path / "em.bin")
    if scene.env_map is not None:
        scene.write_env_map(em)
    text = scene.to_text(em_path=em, algorithm="ptn" if alg == 6 else "pt", max_path_length=maxpl)
    seed = 77
    with P.GpuPathTracer(_cfg(scene, maxpl, alg, sampler), seed=seed) as r:
        g = r.render_samples(alg, 0, 8)
    o = _oracle_samples(scene, text, 8, seed, sampler)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac
    # the sample means agree much tighter than the per-pixel noise
    assert np.allclose(g.mean(axis=(0, 1, 2)), o.mean(axis=(0, 1, 2)), rtol=2e-2)


# (algorithm, max path length, splitting, scene variant, pipeline)
MIXED_CASES = {
    "pt": ("pt", 8, None, "mixed", P.renderer.PIPELINE_WAVEFRONT),
    "pt_megakernel": ("pt", 8, None, "mixed", P.renderer.PIPELINE_MEGAKERNEL),
    "rr": ("pt", 0, None, "mixed", P.renderer.PIPELINE_WAVEFRONT),
    "point_only": ("pt", 8, None, "point", P.renderer.PIPELINE_WAVEFRONT),
    "naive": ("ptn", 8, None, "mixed", P.renderer.PIPELINE_AUTO),
    "dbs": ("dbs", 8, None, "mixed", P.renderer.PIPELINE_AUTO),
    "dlsa": ("dlsa", 8, None, "mixed", P.renderer.PIPELINE_AUTO),
    "dlss": ("dlss", 8, None, "mixed", P.renderer.PIPELINE_AUTO),
    "dmis": ("dmis", 8, None, "mixed", P.renderer.PIPELINE_AUTO),
    "sb4_iic16": ("pt", 0, (4, 1.0, 1.0, 16.0), "mixed", P.renderer.PIPELINE_AUTO),
    "env": ("pt", 12, None, "env", P.renderer.PIPELINE_WAVEFRONT),
    "env_steerable": ("pt", 12, None, "env", P.renderer.PIPELINE_WAVEFRONT),
}


@pytest.mark.parametrize("case", list(MIXED_CASES))
def test_mixed_materials_and_point_light_path_by_path(case, tmp_path):
    """Phong, smooth conductor and smooth dielectric materials and a point light, through every
    estimator and both pipelines, against the oracle sample by sample."""
    alg_name, maxpl, split, variant, pipeline = MIXED_CASES[case]
    if variant == "env":
        scene = S.cornell_env_mixed(24, 24, 64, 32)
    else:
        scene = S.cornell_mixed(24, 24, area=(variant == "mixed"))
    em = str(tmp_path / "em.bin")
    if scene.env_map is not None:
        scene.write_env_map(em)
    text = scene.to_text(em_path=em, algorithm=alg_name, max_path_length=maxpl, splitting=split)
    alg = ALG_IDS[alg_name]
    sampler = P.renderer.EM_STEERABLE if case == "env_steerable" else P.renderer.EM_CDF
    kw = {}
    if split is not None:
        kw = dict(splitting_budget=split[0], splitting_level=split[1], light_to_bsdf_ratio=split[2],
                  indirect_illum_clipping=split[3])
    seed = 53
    with P.GpuPathTracer(_cfg(scene, maxpl, alg, sampler, pipeline=pipeline, **kw), seed=seed) as r:
        g = r.render_samples(alg, 0, 8)
    if case == "env_steerable":
        # the oracle has no steerable sampler: the image means of the two samplers agree within
        # their standard errors
        o = _oracle_samples(scene, text, 256, seed, 0).reshape(-1, 3).astype(np.float64)
        with P.GpuPathTracer(_cfg(scene, maxpl, alg, sampler, pipeline=pipeline), seed=seed) as r:
            g = r.render_samples(alg, 0, 1024).reshape(-1, 3).astype(np.float64)
        assert np.isfinite(g).all()
        se = np.sqrt(g.var(axis=0) / len(g) + o.var(axis=0) / len(o))
        assert np.all(np.abs(g.mean(axis=0) - o.mean(axis=0)) <= 5 * se), (g.mean(axis=0), o.mean(axis=0), se)
        return
    o = _oracle_samples(scene, text, 8, seed, 0)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac
    assert np.isfinite(g).all() and g.max() > 0


def test_triangle_mesh_scene_through_the_lbvh_path_by_path(tmp_path):
    """The environment box with icosphere meshes (1288 triangles): the LBVH wavefront against the
    oracle's list loop, sample by sample."""
    scene = S.cornell_env_mesh(24, 24, 64, 32, level=3)
    em = str(tmp_path / "em.bin")
    scene.write_env_map(em)
    text = scene.to_text(em_path=em, max_path_length=12)
    seed = 83
    cfg = _cfg(scene, 12, P.renderer.kPathTracing, P.renderer.EM_CDF, traversal=P.renderer.TRAVERSAL_BVH)
    with P.GpuPathTracer(cfg, seed=seed) as r:
        g = r.render_samples(P.renderer.kPathTracing, 0, 4)
    o = _oracle_samples(scene, text, 4, seed, 0)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac


@pytest.mark.parametrize("alg", [2, 3, 4, 5])
def test_sra_layered_material_path_by_path(alg, tmp_path):
    """The SRA layered material (GGX coat over a Lambert base, and the reference's scene 27 with a
    conductor base) through the one-hit algorithms, against the oracle sample by sample."""
    from pg3render_gb300 import presets as PR
    names = ["el", "nv", "dbs", "dlsa", "dlss", "dmis"]
    for scene in (S.cornell_mixed(24, 24, sra=True), PR.reference_scene(27, 24, 24)):
        text = scene.to_text(algorithm=names[alg], max_path_length=8)
        seed = 71
        with P.GpuPathTracer(_cfg(scene, 8, alg), seed=seed) as r:
            g = r.render_samples(alg, 0, 8)
        o = _oracle_samples(scene, text, 8, seed, 0)
        frac = _match_fraction(g, o)
        assert frac >= MIN_MATCH, "%s: only %.4f of samples match the oracle" % (scene.name, frac)
        assert np.isfinite(g).all() and g.max() > 0


def test_sra_layered_material_is_refused_by_the_path_tracers():
    scene = S.cornell_mixed(16, 16, sra=True)
    with P.GpuPathTracer(_cfg(scene, 8, P.renderer.kDirectIllumMis)) as r:
        for alg in (P.renderer.kPathTracing, P.renderer.kPathTracingNaive):
            with pytest.raises(P.Pg3Error) as e:
                r.RunIteration(alg, 0, 1)
            assert "SRA" in str(e.value)
        r.RunIteration(P.renderer.kDirectIllumMis, 0, 2)
        assert r.iterations == 2


@pytest.mark.parametrize("sid", [1, 5, 12, 16, 29, 31, 36, 38])
def test_reference_scenes_path_by_path(sid, tmp_path):
    """The reference's built-in scenes (presets) through the wavefront pipeline, against the
    oracle sample by sample."""
    from pg3render_gb300 import presets as PR
    scene = PR.reference_scene(sid, 24, 24)
    text = scene.to_text(max_path_length=8)
    seed = 61
    with P.GpuPathTracer(_cfg(scene, 8), seed=seed) as r:
        g = r.render_samples(P.renderer.kPathTracing, 0, 8)
    o = _oracle_samples(scene, text, 8, seed, 0)
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, "only %.4f of samples match the oracle" % frac
    assert np.isfinite(g).all() and g.max() > 0


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_against_reference_golden(name):
    d, text, td = load_golden(name)
    scene = scene_from_golden(d)
    alg = ALG_IDS[str(d["algorithm"])]
    sp = d["splitting"] if "splitting" in d else (1, 1.0, 1.0, 0.0)
    cfg = _cfg(scene, int(d["max_path_length"]), alg, SAMPLERS[str(d["em_sampler"])], splitting_budget=int(sp[0]),
               splitting_level=float(sp[1]), light_to_bsdf_ratio=float(sp[2]), indirect_illum_clipping=float(sp[3]))
    # heavy-tailed estimators (naive, cosine sky sampling) need many samples; the benchmark scenes'
    # goldens hold 65536 samples per pixel of the reference's render, matched here
    spp = max(32768, int(d["spp"]))
    with P.GpuPathTracer(cfg, seed=2024) as r:
        r.RunIteration(alg, 0, spp)
        mean, var, n = r.framebuffer(with_variance=True)
        assert n == spp and r.WasUsed()
    z = zscores(mean, var / spp, d["mean"], d["var_mean"])
    # (deterministic pixels carry fp64 rounding in their variance: relative threshold)
    frac, zm, zs = z_ok(z, stochastic=(var / spp + d["var_mean"]) > 1e-10 * d["mean"] ** 2)
    assert frac >= 0.999, "%s: only %.4f of |z| <= 4 (mean z %.3f, std %.3f)" % (name, frac, zm, zs)
    if name not in VISUALISERS:   # (deterministic inside a surface: no z distribution there)
        assert abs(zm) < 0.25 and 0.7 < zs < 1.3, "%s: z distribution off (mean %.3f, std %.3f)" % (name, zm, zs)


def test_bvh_and_list_traversal_identical():
    # the list loop, the binary LBVH and the 4-wide BVH collapsed from it return the same hits
    scene = S.cornell_box(24, 24)
    outs = []
    for trav in (P.renderer.TRAVERSAL_LIST, P.renderer.TRAVERSAL_BVH, P.renderer.TRAVERSAL_BVH4):
        with P.GpuPathTracer(_cfg(scene, 8, traversal=trav), seed=5) as r:
            outs.append(r.render_samples(P.renderer.kPathTracing, 0, 4))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("level", [3, 5])
def test_wide_and_binary_bvh_identical_on_meshes(level):
    # icosphere meshes (1288 and 20488 triangles): every closest-hit and any-hit query through the
    # 4-wide BVH finds what the binary LBVH finds, so the samples agree bit for bit
    scene = S.cornell_env_mesh(32, 32, 64, 32, level=level)
    outs = []
    for trav in (P.renderer.TRAVERSAL_BVH, P.renderer.TRAVERSAL_BVH4):
        cfg = _cfg(scene, 12, P.renderer.kPathTracing, P.renderer.EM_STEERABLE, traversal=trav, rr_min_path_length=4)
        with P.GpuPathTracer(cfg, seed=9) as r:
            outs.append(r.render_samples(P.renderer.kPathTracing, 0, 8))
            r.synchronize()   # no traversal-stack or guard flag
    assert np.array_equal(outs[0], outs[1])


def test_iterations_accumulate_like_get_framebuffer():
    scene = S.cornell_box(16, 16)
    with P.GpuPathTracer(_cfg(scene, 8), seed=11) as r:
        assert not r.WasUsed()
        samples = r.render_samples(P.renderer.kPathTracing, 0, 6)
        r.RunIteration(P.renderer.kPathTracing, 0, 2)
        r.RunIteration(P.renderer.kPathTracing, 2, 4)
        mean = r.GetFramebuffer()
        assert r.iterations == 6
    assert np.allclose(mean, samples.astype(np.float64).mean(axis=0), rtol=1e-5, atol=1e-6)


def test_stats_counts():
    scene = S.cornell_box(16, 16)
    with P.GpuPathTracer(_cfg(scene, 8), seed=3) as r:
        r.RunIteration(P.renderer.kPathTracing, 0, 4)
        st = r.stats()
    assert st["paths"] == 16 * 16 * 4
    assert st["extension_rays"] >= st["paths"]
    ended = (st["terminated_by_background"] + st["terminated_by_blocker"] + st["terminated_by_max_limit"]
             + st["terminated_by_russian_roulette"])
    assert ended <= st["paths"] and ended > 0
    assert st["terminated_by_max_limit"] > 0   # a closed box keeps many paths to the limit


@pytest.mark.parametrize("maxpl,rr", [(8, 0), (12, 4), (0, 0)])
def test_path_length_histogram(maxpl, rr):
    # the reference's introspection data (src/renderer.hxx:80-118): every path ended by roulette,
    # the background, a blocker or the length limit counts once, in bin floor(log2(length + 1))
    scene = S.cornell_box(16, 16) if maxpl == 8 else S.cornell_env(16, 16, 64, 32)
    with P.GpuPathTracer(_cfg(scene, maxpl, rr_min_path_length=rr), seed=3) as r:
        r.RunIteration(P.renderer.kPathTracing, 0, 16)
        st = r.stats()
    hist = st["length_histogram"]
    ended = (st["terminated_by_background"] + st["terminated_by_blocker"] + st["terminated_by_max_limit"]
             + st["terminated_by_russian_roulette"])
    assert sum(hist) == ended > 0
    # (a camera ray that leaves to the background is a path of length 0, src/path_tracer.hxx:428)
    assert 0 <= st["min_path_length"] <= st["max_path_length"]
    nz = [b for b, c in enumerate(hist) if c]
    assert 2 ** nz[0] - 1 <= st["min_path_length"] and st["max_path_length"] <= 2 ** (nz[-1] + 1) - 2
    if maxpl:
        assert st["max_path_length"] == maxpl                        # paths reach the limit
        assert hist[int(np.log2(maxpl + 1))] >= st["terminated_by_max_limit"]
    else:
        assert st["terminated_by_russian_roulette"] > 0 and st["max_path_length"] > 4
    # the megakernel pipeline leaves the histogram empty
    with P.GpuPathTracer(_cfg(scene, maxpl, rr_min_path_length=rr, pipeline=P.renderer.PIPELINE_MEGAKERNEL),
                         seed=3) as r:
        r.RunIteration(P.renderer.kPathTracing, 0, 2)
        assert sum(r.stats()["length_histogram"]) == 0


def test_chunked_launches_match_single_launch():
    scene = S.cornell_box(16, 16)
    outs = []
    for cap in (0, 16 * 16):   # default chunking vs one sample pass per launch
        with P.GpuPathTracer(_cfg(scene, 8, max_paths_in_flight=cap), seed=9) as r:
            outs.append(r.render_samples(P.renderer.kPathTracing, 3, 5))
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("case", ["c1_area_256_16spp", "c2_env_512_2spp_cdf"])
def test_full_size_path_by_path(case, tmp_path):
    """The benchmark scenes at their full resolution, every path compared with the oracle:
    the area-light box at 256x256 x 16 spp, max path length 8 (exactly the C1 workload,
    1,048,576 paths), and the environment-map box at 512x512 (2 spp, max length 12, roulette
    after 3 bounces; the CDF sampler, since the oracle restates the reference's samplers)."""
    if case.startswith("c1"):
        scene, spp, maxpl, rr, sampler, seed = S.cornell_box(256, 256), 16, 8, 0, P.renderer.EM_CDF, 21
        text = scene.to_text(max_path_length=maxpl)
    else:
        scene, spp, maxpl, rr, sampler, seed = S.cornell_env(512, 512, 1024, 512), 2, 12, 4, P.renderer.EM_CDF, 22
        em = str(tmp_path / "em.bin")
        scene.write_env_map(em)
        text = scene.to_text(em_path=em, max_path_length=maxpl)
    with P.GpuPathTracer(_cfg(scene, maxpl, sampler=sampler, rr_min_path_length=rr, base_seed=seed)) as r:
        g = r.render_samples(P.renderer.kPathTracing, 0, spp)
    o = _oracle_samples(scene, text, spp, seed, sampler=0, rr=rr)
    assert g.shape == o.shape
    frac = _match_fraction(g, o)
    assert frac >= MIN_MATCH, frac
    # and the image means agree to the statistical error of the sample count
    gm, om = g.mean(axis=(0, 1, 2)), o.mean(axis=(0, 1, 2))
    err = o.reshape(-1, 3).std(axis=0) / np.sqrt(o.shape[0] * o.shape[1] * o.shape[2])
    assert np.all(np.abs(gm - om) <= 4 * err + 1e-6), (gm, om, err)
