"""Shared helpers of the tests: golden fixtures, z-tests, oracle scenes."""
import os
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


def z_ok(z, frac_limit=0.999, zmax=4.0):
    """Fraction of |z| <= zmax at least frac_limit (the spec gate), plus a
    sanity bound on the mean z (systematic bias would shift it)."""
    z = np.asarray(z).ravel()
    z = z[np.isfinite(z)]
    frac = float(np.mean(np.abs(z) <= zmax))
    return frac, float(np.mean(z)), float(np.std(z))


def scene_from_golden(d):
    """Rebuilds the Scene object a fixture was made from (same builder as make_golden)."""
    from pg3render_gb300 import scene as S
    text = str(d["scene_text"])
    name = text.splitlines()[0][2:].strip()
    if name.startswith("cornell_area_"):
        s = S.cornell_box(32, 32)
    else:
        s = S.cornell_env(32, 32, 64, 32)
    if s.env_map is not None:
        s.env_map = d["env_map"]
    return s
