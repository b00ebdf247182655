"""Sampler checks on the GPU (the sampler parity bars: pdf consistency and goodness of fit):

* every sampler's returned pdf equals the pdf its evaluation path computes for
  the same direction to 1e-5 relative (median 1e-6), and
* the sampled directions pass a chi-square goodness-of-fit test against that
  pdf, integrated per equal-area bin (low-expectation bins pooled).

Samplers: Lambert, GGX conductor, GGX dielectric and Phong BSDFs; the area light; the
environment map's cosine, CDF and (corrected) steerable samplers.
"""
import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import scene as S

from _util import chi2_test, dirs_to_pixels, em_pixel_probs, expected_counts, histogram_dirs

pytestmark = pytest.mark.gpu
R = P.renderer
N_CHI = 1 << 21
ALPHA = 1e-4     # significance of one chi-square test


def _bsdf_scene():
    s = S.Scene(S.Camera((0, -3, 0), (0, 1, 0), (0, 0, 1), 8, 8), name="bsdf_probe")
    mats = [S.Material(S.MAT_LAMBERT, (0.5, 0.6, 0.7)),
            S.Material(S.MAT_GGX_CONDUCTOR, alpha=0.3, ior=S.COPPER_IOR, ior_outer=S.AIR_IOR, absorb=S.COPPER_ABSORB),
            S.Material(S.MAT_GGX_CONDUCTOR, alpha=0.1, ior=S.COPPER_IOR, ior_outer=S.AIR_IOR, absorb=S.COPPER_ABSORB),
            S.Material(S.MAT_GGX_DIELECTRIC, alpha=0.3, ior=1.5, ior_outer=1.0),
            S.Material(S.MAT_GGX_DIELECTRIC, alpha=0.5, ior=1.5, ior_outer=1.0),
            # Phong: a diffuse + glossy mixture and a glossy-dominant lobe (component choice by
            # the luminance estimates, power-cosine lobe around the mirror direction)
            S.phong((0.6, 0.5, 0.4), (0.5, 0.5, 0.5), 20),
            S.phong((0.05, 0.05, 0.05), (0.8, 0.8, 0.8), 60)]
    for m in mats:
        s.add_material(m)
    s.add_triangle((-1, 0, -1), (1, 0, -1), (0, 0, 1), 0)
    s.background_const = (1.0, 1.0, 1.0)
    return s


def _env_scene(sampler, weights=R.STEER_WEIGHTS_POINT, adaptive=None):
    """adaptive: (minimum level, maximum level, maximum approximation error) of an adaptive
    steerable triangulation (leaves at several levels), None for one uniform level."""
    s = S.cornell_env(8, 8, 256, 128, em_seed=11)
    kw = {}
    if adaptive:
        kw = dict(steer_subdiv_level=adaptive[0], steer_max_subdiv_level=adaptive[1],
                  steer_max_approx_error=adaptive[2])
    return P.Config(scene=s, max_path_length=12, em_sampler=sampler, steer_weights=weights, **kw)


def _rel(a, b):
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


def _wol(theta_deg, below=False):
    t = np.radians(theta_deg)
    w = np.array([np.sin(t), 0.0, np.cos(t)], np.float32)
    return -w if below else w


BSDF_CASES = [(0, 40, False), (1, 45, False), (2, 30, False), (3, 50, False), (3, 35, True), (4, 60, False),
              (5, 30, False), (6, 55, False)]


@pytest.mark.parametrize("mat,theta,below", BSDF_CASES)
def test_bsdf_pdf_consistency(mat, theta, below):
    with P.GpuPathTracer(P.Config(scene=_bsdf_scene(), max_path_length=4)) as r:
        n = 1 << 18
        wol = np.tile(_wol(theta, below), (n, 1))
        o = r.probe_bsdf(mat, wol, seed=3)
    valid = (o["pdf_eval"] > 0) & np.isfinite(o["pdf_sampled"]) & (o["att_sampled"].max(axis=1) > 0)
    assert valid.mean() > 0.5
    rel = _rel(o["pdf_sampled"][valid], o["pdf_eval"][valid])
    # The evaluation recomputes the half vector from the two directions; float rounding of the
    # sampled direction, amplified by steep lobes (alpha 0.1) and refraction from inside,
    # reaches 4e-5 in the last 0.1% of samples.
    assert np.median(rel) <= 1e-6 and np.quantile(rel, 0.99) <= 1e-5 and np.quantile(rel, 0.999) <= 1e-4, \
        (np.median(rel), np.quantile(rel, 0.99), np.quantile(rel, 0.999))
    ra = _rel(o["att_sampled"][valid], o["att_eval"][valid])
    assert np.quantile(ra, 0.99) <= 1e-5 and np.quantile(ra, 0.999) <= 1e-4


@pytest.mark.parametrize("mat,theta,below", BSDF_CASES)
def test_bsdf_chi_square(mat, theta, below):
    # Directions the sampler produces with zero BSDF value (reflections below the horizon,
    # refractions to the wrong side) carry no weight and no evaluated pdf describes them:
    # the test histograms the valid samples and integrates the evaluated pdf where the
    # evaluated BSDF is non-zero (24x24 midpoint rule per bin: the refraction
    # Jacobian has a sharp ridge).
    nz, nphi = 40, 80
    with P.GpuPathTracer(P.Config(scene=_bsdf_scene(), max_path_length=4)) as r:
        w = _wol(theta, below)
        o = r.probe_bsdf(mat, np.tile(w, (N_CHI, 1)), seed=5)
        valid = o["att_sampled"].max(axis=1) > 0
        obs = histogram_dirs(o["wil"][valid], nz, nphi)

        def masked_pdf(d):
            pdf, att = r.probe_bsdf_pdf(mat, np.tile(w, (len(d), 1)), d, with_att=True)
            return pdf * (att > 0)
        exp = expected_counts(masked_pdf, N_CHI, nz, nphi, k=24)
    p, chi2, dof = chi2_test(obs, exp)
    assert abs(exp.sum() / N_CHI - valid.mean()) < 0.003, (exp.sum() / N_CHI, valid.mean())
    assert p > ALPHA, (p, chi2, dof)


def test_reference_vndf_fit_is_approximate():
    # The reference's visible-normal routine (Heitz & d'Eon 2014 with a rational fit of the
    # slope CDF, src/microfacet.hxx:610-729) over-produces sideways-tilted microfacets; its
    # refractions fail the same chi-square test that the exact sampler (the default) passes.
    nz, nphi = 40, 80
    scene = _bsdf_scene()
    w = _wol(50)
    stats = {}
    for mode in (0, 1):   # exact, reference fit
        with P.GpuPathTracer(P.Config(scene=scene, max_path_length=4, ggx_sampler=mode)) as r:
            o = r.probe_bsdf(3, np.tile(w, (N_CHI, 1)), seed=21)
            valid = o["att_sampled"].max(axis=1) > 0
            obs = histogram_dirs(o["wil"][valid], nz, nphi)

            def masked_pdf(d):
                pdf, att = r.probe_bsdf_pdf(3, np.tile(w, (len(d), 1)), d, with_att=True)
                return pdf * (att > 0)
            exp = expected_counts(masked_pdf, N_CHI, nz, nphi, k=24)
        stats[mode] = chi2_test(obs, exp)
    assert stats[0][0] > ALPHA, stats[0]
    assert stats[1][1] / stats[1][2] > 1.2, stats[1]


PT, PJ = R.STEER_WEIGHTS_POINT, R.STEER_WEIGHTS_PROJECTED
# adaptive steerable triangulations: the reference's default build parameters (levels 4-9,
# error 5) and a deeper refinement with leaves on five levels
REF_DEFAULT, DEEP = (4, 9, 5.0), (2, 7, 0.5)
ENV_CASES = [(R.EM_COSINE, (0.0, 0.0, 1.0), PT, None), (R.EM_CDF, (0.0, 0.0, 1.0), PT, None),
             (R.EM_STEERABLE, (0.0, 0.0, 1.0), PT, None), (R.EM_STEERABLE, (0.35, -0.2, 0.915), PT, None),
             (R.EM_STEERABLE, (0.0, 0.0, 1.0), PJ, None), (R.EM_STEERABLE, (-0.6, 0.3, 0.742), PJ, None),
             (R.EM_STEERABLE, (0.0, 0.0, 1.0), PT, REF_DEFAULT), (R.EM_STEERABLE, (0.35, -0.2, 0.915), PT, DEEP),
             (R.EM_STEERABLE, (-0.6, 0.3, 0.742), PJ, REF_DEFAULT)]


@pytest.mark.parametrize("sampler,normal,weights,adaptive", ENV_CASES)
def test_env_sampler_pdf_consistency(sampler, normal, weights, adaptive):
    nrm = np.asarray(normal, np.float32)
    nrm /= np.linalg.norm(nrm)
    with P.GpuPathTracer(_env_scene(sampler, weights, adaptive)) as r:
        n = 1 << 18
        o = r.probe_light(0, np.zeros((n, 3)), np.tile(nrm, (n, 1)), seed=9)
    # CDF samples below the horizon carry zero radiance but a valid pdf; compare where upper
    up = o["dirs"] @ nrm > 1e-4
    v = up & (o["pdf_eval"] > 0)
    assert v.mean() > 0.4
    rel = _rel(o["pdf_sampled"][v], o["pdf_eval"][v])
    assert np.median(rel) <= 1e-6 and np.quantile(rel, 0.999) <= 1e-5, (np.median(rel), np.quantile(rel, 0.999))


@pytest.mark.parametrize("sampler,normal,weights,adaptive", ENV_CASES)
def test_env_sampler_chi_square(sampler, normal, weights, adaptive):
    nrm = np.asarray(normal, np.float32)
    nrm /= np.linalg.norm(nrm)
    with P.GpuPathTracer(_env_scene(sampler, weights, adaptive)) as r:
        o = r.probe_light(0, np.zeros((N_CHI, 3)), np.tile(nrm, (N_CHI, 1)), seed=13)
        if sampler == R.EM_CDF:
            # The CDF sampler's pdf is exact per map pixel only (uniform in (u, v) inside a pixel,
            # reported with sin(theta_mid): src/em_simple_spherical_sampler.hxx:52-66), so its
            # directions are tested per map pixel against the pixel probabilities.
            em = r.config.scene.env_map
            H, W, _ = em.shape
            iy, ix = dirs_to_pixels(o["dirs"], W, H)
            obs = np.zeros((H, W))
            np.add.at(obs, (iy, ix), 1)
            exp = em_pixel_probs(em) * N_CHI
        else:
            nz, nphi = 64, 128
            obs = histogram_dirs(o["dirs"], nz, nphi)
            pdf_fn = lambda d: r.probe_light_pdf(0, np.zeros((len(d), 3)), np.tile(nrm, (len(d), 1)), d)  # noqa
            exp = expected_counts(lambda d: pdf_fn(d) * (d @ nrm >= 0), N_CHI, nz, nphi, k=6)
            assert abs(exp.sum() / N_CHI - 1.0) < 0.01, exp.sum() / N_CHI
    p, chi2, dof = chi2_test(obs, exp)
    assert p > ALPHA, (p, chi2, dof)


def test_area_light_pdf_consistency():
    s = S.cornell_box(8, 8)
    with P.GpuPathTracer(P.Config(scene=s, max_path_length=8)) as r:
        n = 1 << 16
        rng = np.random.default_rng(0)
        pts = np.stack([rng.uniform(-0.9, 0.9, n), rng.uniform(-0.9, 0.9, n), np.full(n, -0.99)], 1)
        nrm = np.tile([0.0, 0.0, 1.0], (n, 1))
        for light in (0, 1):
            o = r.probe_light(light, pts, nrm, seed=light)
            v = o["pdf_eval"] > 0
            assert v.mean() > 0.99
            rel = _rel(o["pdf_sampled"][v], o["pdf_eval"][v])
            assert np.quantile(rel, 0.999) <= 1e-5, np.quantile(rel, 0.999)


@pytest.mark.parametrize("pipeline,weights", [(R.PIPELINE_WAVEFRONT, PT), (R.PIPELINE_MEGAKERNEL, PT),
                                              (R.PIPELINE_WAVEFRONT, PJ)])
def test_steerable_render_converges_to_reference(pipeline, weights):
    # the reference's own steerable sampler is not pdf-consistent; its unbiased CDF-sampler
    # render of the same scene is the image the corrected steerable sampler must reach, with
    # either vertex weighting
    from _util import load_golden, scene_from_golden, z_ok, zscores
    d, text, td = load_golden("cornell_env_32_cdf")
    scene = scene_from_golden(d)
    cfg = P.Config(scene=scene, max_path_length=12, em_sampler=R.EM_STEERABLE, pipeline=pipeline,
                   steer_weights=weights)
    spp = 65536   # as many samples as the reference's golden
    with P.GpuPathTracer(cfg, seed=123) as r:
        r.RunIteration(R.kPathTracing, 0, spp)
        mean, var, n = r.framebuffer(with_variance=True)
    frac, zm, zs = z_ok(zscores(mean, var / spp, d["mean"], d["var_mean"]))
    assert frac >= 0.999 and abs(zm) < 0.25 and 0.7 < zs < 1.3, (frac, zm, zs)


def test_projected_weights_are_reproducible(tmp_path):
    # the projection sums texel contributions in fixed point: the same scene and seed give the
    # same vertex weights and the same image, bit for bit, whatever the order of the atomics
    cfg = _env_scene(R.EM_STEERABLE, PJ)
    imgs, files = [], []
    for k in range(2):
        with P.GpuPathTracer(cfg, seed=3) as r:
            r.RunIteration(R.kPathTracing, 0, 16)
            imgs.append(r.framebuffer()[0])
            f = str(tmp_path / ("w%d.emssd" % k))
            r.save_steerable(f)
            files.append(open(f, "rb").read())
    assert np.array_equal(imgs[0], imgs[1])
    assert files[0] == files[1]
    # and the projection is not the point sample (the sky's suns lie between vertices)
    with P.GpuPathTracer(_env_scene(R.EM_STEERABLE, PT), seed=3) as r:
        f = str(tmp_path / "point.emssd")
        r.save_steerable(f)
        assert open(f, "rb").read() != files[0]
