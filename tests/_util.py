"""Shared helpers of the tests: golden fixtures, z-tests, oracle scenes."""
import os
import re
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
EM_TOKEN = "@EM@"


def load_golden(name):
    """Returns (fixture dict, scene text with a real EM path, tempdir to keep alive)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    td = tempfile.TemporaryDirectory()
    text = str(d["scene_text"])
    if d["env_map"].size:
        from pg3render_gb300.scene import write_env_map
        p = os.path.join(td.name, "em.bin")
        write_env_map(p, d["env_map"])
        text = text.replace(EM_TOKEN, p)
    return d, text, td


def zscores(mean_a, var_a, mean_b, var_b):
    return (mean_a - mean_b) / np.sqrt(var_a + var_b + 1e-300)


def z_ok(z, frac_limit=0.999, zmax=4.0, stochastic=None):
    """Fraction of |z| <= zmax at least frac_limit (the image parity bar), plus the mean and
    standard deviation of z (systematic bias would shift the mean). stochastic (optional mask):
    the entries with sampling variance; deterministic pixels (a constant background seen
    directly, an emitter) have z = 0 and are left out of the two moments."""
    z = np.asarray(z).ravel()
    keep = np.isfinite(z)
    frac = float(np.mean(np.abs(z[keep]) <= zmax))
    if stochastic is not None:
        keep &= np.asarray(stochastic).ravel()
    zz = z[keep]
    return frac, float(np.mean(zz)), float(np.std(zz))


def scene_from_golden(d):
    """Rebuilds the Scene object a fixture was made from (same builder as make_golden)."""
    from pg3render_gb300 import scene as S
    text = str(d["scene_text"])
    name = text.splitlines()[0][2:].strip()
    if name.startswith("cornell_mixed_area_point_sra_"):
        s = S.cornell_mixed(32, 32, sra=True)
    elif name.startswith("reference_scene_"):
        from pg3render_gb300 import presets as PR
        s = PR.reference_scene(int(name.split("_")[2]), 32, 32)
    elif name.startswith("cornell_mixed_area_point_"):
        s = S.cornell_mixed(32, 32)
    elif name.startswith("cornell_mixed_point_"):
        s = S.cornell_mixed(32, 32, area=False)
    elif name.startswith("cornell_envmixed_"):
        s = S.cornell_env_mixed(32, 32, 64, 32)
    elif name.startswith("cornell_area_"):
        s = S.cornell_box(32, 32)
    elif name.startswith("cornell_areabg_"):
        s = S.cornell_box_bg(32, 32)
    elif name.startswith("cornell_envarea_"):
        s = S.cornell_env_area(32, 32, 64, 32)
    elif re.match(r"cornell_env_\d+x\d+_em\d+x\d+$", name):
        w, h, ew, eh = map(int, re.findall(r"\d+", name))
        s = S.cornell_env(w, h, ew, eh)
    else:
        s = S.cornell_env(32, 32, 64, 32)
    if s.env_map is not None:
        s.env_map = d["env_map"]
    return s


# ----------------------------------------------------------------------------- chi-square
def sphere_bins(nz, nphi):
    """Equal-area bins over the sphere: uniform in z = cos(theta) and phi."""
    return np.linspace(-1.0, 1.0, nz + 1), np.linspace(-np.pi, np.pi, nphi + 1)


def histogram_dirs(d, nz, nphi):
    ze, pe = sphere_bins(nz, nphi)
    z = np.clip(d[:, 2], -1.0, 1.0)
    phi = np.arctan2(d[:, 1], d[:, 0])
    h, _, _ = np.histogram2d(z, phi, bins=[ze, pe])
    return h


def expected_counts(pdf_fn, n, nz, nphi, k=6):
    """N * integral of pdf over each bin by a k x k midpoint rule (pdf_fn: dirs[m,3] -> pdf[m])."""
    ze, pe = sphere_bins(nz, nphi)
    dz, dp = 2.0 / nz, 2 * np.pi / nphi
    sz = (np.arange(nz * k) + 0.5) * (dz / k) - 1.0
    sp = (np.arange(nphi * k) + 0.5) * (dp / k) - np.pi
    Z, PH = np.meshgrid(sz, sp, indexing="ij")
    r = np.sqrt(np.maximum(0.0, 1.0 - Z * Z))
    dirs = np.stack([r * np.cos(PH), r * np.sin(PH), Z], -1).reshape(-1, 3).astype(np.float32)
    pdf = pdf_fn(dirs).astype(np.float64).reshape(nz * k, nphi * k)
    cell = (dz / k) * (dp / k)
    return n * pdf.reshape(nz, k, nphi, k).sum(axis=(1, 3)) * cell


def chi2_test(observed, expected, min_expected=5.0):
    """Pearson chi-square with low-expectation bins pooled; returns (p_value, chi2, dof)."""
    from scipy import stats
    o = observed.ravel().astype(np.float64)
    e = expected.ravel().astype(np.float64)
    keep = e >= min_expected
    o_pool, e_pool = o[~keep].sum(), e[~keep].sum()
    oo, ee = list(o[keep]), list(e[keep])
    if e_pool >= min_expected:
        oo.append(o_pool)
        ee.append(e_pool)
    oo, ee = np.array(oo), np.array(ee)
    ee *= oo.sum() / ee.sum()      # compare shapes (quadrature normalisation error removed)
    chi2 = float(((oo - ee) ** 2 / ee).sum())
    dof = len(oo) - 1
    return float(stats.chi2.sf(chi2, dof)), chi2, dof


def em_pixel_probs(em):
    """Per-pixel probability of the reference's CDF environment sampler: tent-filtered pixel
    luminance x sin(theta_mid), normalised (src/em_simple_spherical_sampler.hxx:117-152,
    src/em_image.hxx:152-183 with the wrap rules of :269-302), restated in numpy."""
    em = np.asarray(em, np.float64)
    H, W, _ = em.shape
    lum = 0.212671 * em[..., 0] + 0.715160 * em[..., 1] + 0.072169 * em[..., 2]

    def at(dx, dy):
        ys = np.arange(H)[:, None] + dy
        xs = np.arange(W)[None, :] + dx + np.where((ys < 0) | (ys >= H), W // 2, 0)
        ys = np.clip(ys, 0, H - 1)
        return lum[np.broadcast_to(ys, (H, W)), np.mod(xs, W)]

    tent = sum(at(dx, dy) * (2 / 3 if dx == 0 and dy == 0 else 1 / 24) for dx in (-1, 0, 1) for dy in (-1, 0, 1))
    f = tent * np.sin(np.pi * (np.arange(H) + 0.5) / H)[:, None]
    return f / f.sum()


def dirs_to_pixels(d, W, H):
    """Lat-long pixel of each direction (src/geom.hxx:77-95)."""
    phi = -np.arctan2(d[:, 1], d[:, 0])
    th = np.arccos(np.clip(d[:, 2], -1, 1))
    u = np.clip(0.5 + phi / (2 * np.pi), 0, 1)
    v = np.clip(th / np.pi, 0, 1)
    return np.minimum((v * H).astype(int), H - 1), np.minimum((u * W).astype(int), W - 1)
