"""The oracle pinned against the reference (CPU tests).

* Philox4x32-10 reproduces the published Random123 known-answer vectors;
* the oracle's renders agree with the reference renderer's own golden images
  (tests/golden, made by tests/golden/make_golden.py with the reference code):
  |z| <= 4 on >= 99.9% of pixel channels, z mean ~ 0, z std ~ 1;
* the reference's tent-filter integral known answers (src/filter.hxx:123-170)
  hold for the oracle's environment-map CDF weights;
* CDF tables are monotone and normalised.
"""
import os

import numpy as np
import pytest

import oracle as O
from _util import load_golden, z_ok, zscores

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
# the visualisers are deterministic inside a surface (zero variance): only the fraction of
# |z| <= 4 is a meaningful statistic for them
VISUALISERS = ("cornell_area_32_el", "cornell_area_32_nv")


def test_philox_known_answers():
    # Random123 kat_vectors, philox4x32 10 rounds
    assert list(O.philox([0, 0, 0, 0], [0, 0])) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    ff = 0xffffffff
    assert list(O.philox([ff, ff, ff, ff], [ff, ff])) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert list(O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0])) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_reference_golden(name):
    d, text, td = load_golden(name)
    sampler = {"cdf": O.EM_CDF, "cosine": O.EM_COSINE}[str(d["em_sampler"])]
    # BSDF-only sampling of a small light (naive path tracing, dbs), and cosine sampling of a
    # sky with 1e4 suns, are heavy-tailed: their sample variances need more samples before
    # the z-test is calibrated
    spp = {"cornell_area_32_naive": 8192, "cornell_env_32_cos": 16384, "cornell_area_32_dbs": 8192,
           "cornell_env_32_dbs": 8192, "cornell_mixed_32_naive": 8192, "cornell_mixed_32_dbs": 8192,
           # glossy Phong lobes lit by a point light, caustics through smooth glass: heavy tails
           "cornell_mixed_32": 8192, "cornell_mixed_32_rr": 8192, "cornell_mixed_32_point": 8192,
           "cornell_envmixed_32_cdf": 8192,
           "preset_00": 8192, "preset_03": 8192, "preset_07": 8192, "preset_29": 8192, "preset_01": 32768,
           "preset_05": 32768, "preset_16": 32768, "preset_19": 32768, "preset_31": 32768,
           "preset_38": 32768, "preset_27_dmis": 8192, "preset_27_dlss": 8192, "cornell_mixedsra_32_dmis": 8192,
           "cornell_mixedsra_32_dbs": 8192,
           # the benchmark scenes: the oracle's 64k-spp render against the reference's 64k-spp golden
           # (at 1-8k spp the heavy tails skew the z distribution against so tight a golden)
           "cornell_area_32": 65536, "cornell_env_32_cdf": 65536}.get(name, 1024)
    o = O.render(text, 32, 32, seed=99, spp=spp, em_sampler=sampler)
    m = o["sum"] / spp
    v = np.maximum(o["sumsq"] / spp - m * m, 0.0) / spp
    frac, zm, zs = z_ok(zscores(m, v, d["mean"], d["var_mean"]), stochastic=(v + d["var_mean"]) > 1e-10 * m * m)
    assert frac >= 0.999, "%s: %.4f of |z| <= 4" % (name, frac)
    if name not in VISUALISERS:
        assert abs(zm) < 0.25 and 0.7 < zs < 1.3, "%s: z mean %.3f std %.3f" % (name, zm, zs)


def test_oracle_deterministic_and_sample_indexed():
    d, text, td = load_golden("cornell_area_32")
    a = O.render(text, 32, 32, seed=5, sample0=0, spp=4, per_sample=True)["samples"]
    b = O.render(text, 32, 32, seed=5, sample0=2, spp=2, per_sample=True)["samples"]
    assert np.array_equal(a[2:], b)                         # sample s is the same path whatever the batch
    c = O.render(text, 32, 32, seed=6, sample0=0, spp=4, per_sample=True)["samples"]
    assert not np.array_equal(a, c)                         # the seed keys the streams


def test_em_cdf_tables(tmp_path):
    from pg3render_gb300 import scene as S
    em = S.synthetic_sky(64, 32, seed=3)
    p = str(tmp_path / "em.bin")
    S.write_env_map(p, em)
    marg, cond = O.em_cdf(p, 64, 32)
    assert marg[0] == 0 and abs(marg[-1] - 1) < 1e-6 and np.all(np.diff(marg) >= 0)
    assert np.all(cond[:, 0] == 0) and np.allclose(cond[:, -1], 1, atol=1e-6) and np.all(np.diff(cond, axis=1) >= 0)
    # constant map: the tent-filter integral of a constant c is c (src/filter.hxx:123-170 KAT "1"),
    # so every conditional is uniform and the marginal follows sin(theta_mid)
    S.write_env_map(p, np.ones((32, 64, 3), np.float32))
    marg, cond = O.em_cdf(p, 64, 32)
    assert np.allclose(cond, np.linspace(0, 1, 65)[None, :], atol=1e-6)
    s = np.sin(np.pi * (np.arange(32) + 0.5) / 32)
    assert np.allclose(np.diff(marg), s / s.sum(), atol=1e-6)


def test_camera_matches_reference_mapping():
    # The oracle (and the kernels) send raster (x, y) along
    # forward + right*ndc_x*tan(hfov/2) - up*ndc_y*tan(vfov/2), which is what the reference's
    # 4x4 raster-to-world matrix does (src/camera.hxx:13-59): centre -> forward, left/right
    # edges at +-hfov/2, top row towards +up.
    from pg3render_gb300 import scene as S
    s = S.cornell_box(64, 48)
    text = s.to_text()
    d = O.camera_dirs(text, [[32, 24], [0, 24], [64, 24], [32, 0]])
    assert np.allclose(d[0], [0, 1, 0], atol=1e-6)
    half = np.degrees(np.arctan2(d[2][0], d[2][1]))
    assert abs(half - 22.5) < 1e-4 and abs(np.degrees(np.arctan2(-d[1][0], d[1][1])) - 22.5) < 1e-4
    vhalf = np.degrees(np.arctan2(d[3][2], d[3][1]))
    assert abs(np.tan(np.radians(vhalf)) - np.tan(np.radians(22.5)) * 48 / 64) < 1e-6


@pytest.mark.skipif(O.reference_binary("cdf") is None, reason="reference harness not built")
def test_reference_harness_runs_and_is_seeded():
    d, text, td = load_golden("cornell_area_32")
    a = O.reference_render(text, renderers=2, iters=1, seed=3)
    b = O.reference_render(text, renderers=2, iters=1, seed=3)
    assert np.array_equal(a["mean"], b["mean"]) and a["mean"].mean() > 0


def test_em_pixel_probabilities_match_cdf_tables(tmp_path):
    # the numpy restatement the GPU chi-square test uses equals the oracle's CDF tables
    from pg3render_gb300 import scene as S
    from _util import em_pixel_probs
    em = S.synthetic_sky(64, 32, seed=5)
    p = str(tmp_path / "em.bin")
    S.write_env_map(p, em)
    marg, cond = O.em_cdf(p, 64, 32)
    probs = np.diff(marg)[:, None] * np.diff(cond, axis=1)
    # float32 running sums: a few ulp of 1.0 in each CDF entry
    assert np.allclose(probs, em_pixel_probs(em), rtol=1e-3, atol=2e-7)
