"""Python access to the oracle (test infrastructure only).

* :func:`render` runs the C++ restatement ``pt_oracle.cpp`` (same Philox
  streams as the CUDA path) and returns per-pixel sums / sums of squares /
  optionally every sample.
* :func:`reference_render` runs the reference renderer's own code through
  ``oracle/_ref/pg3ref_*`` (K independent renderers, seeds base+i) and returns
  the mean image and the variance of one renderer's mean.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module.
"""
import ctypes
import json
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_lib = None

EM_CDF, EM_COSINE = 0, 1


def lib():
    global _lib
    if _lib is None:
        import build as _b  # noqa: E402  (oracle/build.py)
        path = _b.build_oracle()
        L = ctypes.CDLL(path)
        L.pg3o_render.restype = ctypes.c_int
        L.pg3o_render.argtypes = [ctypes.c_char_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32,
                                  ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_char_p, ctypes.c_int]
        L.pg3o_philox.argtypes = [ctypes.c_void_p] * 3
        L.pg3o_camera_dirs.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.pg3o_em_cdf.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def render(scene_text, width, height, seed=1234, sample0=0, spp=1, em_sampler=EM_CDF,
           rr_min_path_length=0, threads=0, per_sample=False, ggx_exact=True):
    """Returns dict(sum=[H,W,3] f64, sumsq=[H,W,3] f64, samples=[spp,H,W,3] f32 or None).
    ggx_exact selects the exact visible-normal sampler (False: the reference's fitted routine)."""
    lib().pg3o_set_ggx_exact(1 if ggx_exact else 0)
    npix = width * height
    s = np.zeros((npix, 3), np.float64)
    s2 = np.zeros((npix, 3), np.float64)
    ps = np.zeros((spp, npix, 3), np.float32) if per_sample else None
    err = ctypes.create_string_buffer(512)
    rc = lib().pg3o_render(scene_text.encode(), seed, sample0, spp, em_sampler, rr_min_path_length,
                           threads, _ptr(s), _ptr(s2), _ptr(ps), err, 512)
    if rc != 0:
        raise RuntimeError("oracle: " + err.value.decode())
    out = dict(sum=s.reshape(height, width, 3), sumsq=s2.reshape(height, width, 3), spp=spp)
    if per_sample:
        out["samples"] = ps.reshape(spp, height, width, 3)
    return out


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().pg3o_philox(_ptr(c), _ptr(k), _ptr(o))
    return o


def camera_dirs(scene_text, raster_xy):
    xy = np.ascontiguousarray(raster_xy, np.float32)
    out = np.zeros((len(xy), 3), np.float32)
    if lib().pg3o_camera_dirs(scene_text.encode(), _ptr(xy), len(xy), _ptr(out)) != 0:
        raise RuntimeError("oracle camera")
    return out


def em_cdf(em_path, width, height):
    marg = np.zeros(height + 1, np.float32)
    cond = np.zeros((height, width + 1), np.float32)
    if lib().pg3o_em_cdf(em_path.encode(), _ptr(marg), _ptr(cond)) != 0:
        raise RuntimeError("oracle em cdf")
    return marg, cond


# ---------------------------------------------------------------- reference harness
def reference_binary(em_sampler="cdf"):
    path = os.path.join(REF_DIR, "pg3ref_" + {"cdf": "cdf", "cosine": "cos", "steerable": "steer"}[em_sampler])
    return path if os.path.exists(path) else None


def reference_render(scene_text, renderers=8, iters=1, threads=0, seed=1234, em_sampler="cdf",
                     time_only=False, extra=()):
    """Runs the reference's own PathTracer. Returns dict(mean, var_of_renderer_mean, K, N, timing)."""
    exe = reference_binary(em_sampler)
    if exe is None:
        raise FileNotFoundError("reference harness not built (oracle/build_ref.py)")
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "scene.txt")
        op = os.path.join(td, "out.bin")
        with open(sp, "w") as f:
            f.write(scene_text)
        cmd = [exe, sp, op, "--renderers", str(renderers), "--iters", str(iters), "--seed", str(seed)]
        if threads:
            cmd += ["--threads", str(threads)]
        if time_only:
            cmd += ["--time"]
        cmd += list(extra)
        res = subprocess.run(cmd, check=True, capture_output=True, text=True)
        timing = json.loads(res.stdout.strip().splitlines()[-1])
        if time_only:
            return dict(timing=timing)
        with open(op, "rb") as f:
            W, H, K, N = np.frombuffer(f.read(16), np.uint32)
            mean = np.frombuffer(f.read(int(W * H * 3) * 8), np.float64).reshape(H, W, 3)
            var = np.frombuffer(f.read(int(W * H * 3) * 8), np.float64).reshape(H, W, 3)
    return dict(mean=mean.copy(), var_of_renderer_mean=var.copy(), K=int(K), N=int(N), timing=timing)
