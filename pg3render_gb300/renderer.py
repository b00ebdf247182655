"""Host-side mirror of the reference's renderer interface over the C ABI.

``Config`` carries the options of the reference's ``Config`` that the path
tracer reads (src/config.hxx:1100-1137); ``GpuPathTracer`` behaves like a
``PathTracer`` (src/path_tracer.hxx:5-41) deriving from ``AbstractRenderer``
(src/renderer.hxx:232-278): ``RunIteration`` renders one (or ``spp``)
iterations, ``GetFramebuffer`` returns the accumulated image divided by the
iteration count, ``WasUsed`` tells whether any iteration ran. Errors the
reference reports with PG3_FATAL_ERROR raise :class:`Pg3Error` here.
"""
import ctypes
import dataclasses
import os

import numpy as np

from . import _lib
from ._lib import (ALG_PATH_TRACING, ALG_PATH_TRACING_NAIVE, EM_CDF, EM_COSINE, EM_STEERABLE,  # noqa: F401
                   PIPELINE_AUTO, PIPELINE_MEGAKERNEL, PIPELINE_WAVEFRONT, STEER_WEIGHTS_POINT,
                   STEER_WEIGHTS_PROJECTED, TRAVERSAL_AUTO, TRAVERSAL_BVH, TRAVERSAL_BVH4, TRAVERSAL_LIST,
                   Pg3Error)

def steerable_file_name(em_path, level, max_approx_error=5.0, bilinear=True):
    """The path under which the reference caches the steerable sampler of the map at em_path
    (EnvironmentMapSteerableSampler::GenerateSaveFilePath, src/em_steerable_sampler.hxx:1596-1646)
    for a uniform triangulation: minimum = maximum subdivision level, its default debugging
    parameters (50 samples per dimension, span 1.1, oversampling 0.7) and 6 children per node."""
    return "%s.%s_e%.2f_sll%d_slu%d_tms%d_ts%.2f_os%.2f_mc%d.v2.1.emssd" % (
        em_path, "bi" if bilinear else "nn", max_approx_error, level, level, 50, 1.1, 0.7, 6)


def write_image(mean_rgb, path, gamma=2.2):
    """Writes an (H, W, 3) mean image as ``.hdr`` or a gamma-encoded 24-bit BMP (no GPU needed)."""
    a = np.ascontiguousarray(mean_rgb, np.float64)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("mean_rgb must be (height, width, 3)")
    L = _lib.load()
    _lib.check(L.pg3gpu_write_image(a.ctypes.data_as(ctypes.c_void_p), a.shape[1], a.shape[0], os.fsencode(path),
                                    gamma), None)


# Algorithm enum of src/config.hxx:23-34
kEyeLight, kNormalVisualiser, kDirectIllumBsdfSampling, kDirectIllumLightSamplingAll, \
    kDirectIllumLightSamplingSingle, kDirectIllumMis, kPathTracingNaive, kPathTracing = range(8)


@dataclasses.dataclass
class Config:
    scene: object = None                 # pg3render_gb300.scene.Scene
    algorithm: int = kPathTracing        # mAlgorithm
    iterations: int = 1                  # mIterations
    base_seed: int = 1234                # mBaseSeed
    min_path_length: int = 1             # mMinPathLength
    max_path_length: int = 0             # mMaxPathLength (0: Russian roulette)
    indirect_illum_clipping: float = 0.0  # mIndirectIllumClipping (the reference CLI's default is 16)
    splitting_budget: int = 1            # mSplittingBudget (the reference CLI's default is 4)
    splitting_level: float = 1.0         # mDbgSplittingLevel
    light_to_bsdf_ratio: float = 1.0     # mDbgSplittingLightToBrdfSmplRatio
    em_sampler: int = EM_CDF             # compile-time PG3_USE_ENVMAP_* in the reference
    rr_min_path_length: int = 0          # extension: roulette from this length on with a max length set
    traversal: int = TRAVERSAL_AUTO
    pipeline: int = PIPELINE_AUTO
    steer_subdiv_level: int = 3
    max_paths_in_flight: int = 0
    ggx_sampler: int = 0                 # GGX_VNDF_EXACT; GGX_VNDF_REFERENCE_FIT = the reference's routine
    steer_weights: int = 1               # STEER_WEIGHTS_PROJECTED; STEER_WEIGHTS_POINT = the reference's build
    steer_max_subdiv_level: int = 0      # > steer_subdiv_level: adaptive triangulation between the levels
    steer_max_approx_error: float = 5.0  # adaptive triangulation: the reference's maximum approximation error

    def options(self, seed=None):
        o = _lib.Options()
        _lib.load().pg3gpu_default_options(ctypes.byref(o))
        o.algorithm = self.algorithm
        o.min_path_length = self.min_path_length
        o.max_path_length = self.max_path_length
        o.rr_min_path_length = self.rr_min_path_length
        o.indirect_clipping = self.indirect_illum_clipping
        o.splitting_budget = self.splitting_budget
        o.splitting_level = self.splitting_level
        o.light_to_bsdf_ratio = self.light_to_bsdf_ratio
        o.em_sampler = self.em_sampler
        o.traversal = self.traversal
        o.pipeline = self.pipeline
        o.steer_subdiv_level = self.steer_subdiv_level
        o.seed = self.base_seed if seed is None else seed
        o.max_paths_in_flight = self.max_paths_in_flight
        o.ggx_sampler = self.ggx_sampler
        o.steer_weights = self.steer_weights
        o.steer_max_subdiv_level = self.steer_max_subdiv_level
        o.steer_max_approx_error = self.steer_max_approx_error
        return o


class GpuPathTracer:
    """One GPU renderer context (the reference creates one renderer per thread;
    here one context renders whole iterations on the device)."""

    def __init__(self, config: Config, seed=None, device=0, stream=None):
        self.config = config
        self._L = _lib.load()
        self._desc = _lib.scene_desc(config.scene)
        self._opts = config.options(seed)
        h = ctypes.c_void_p()
        _lib.check(self._L.pg3gpu_create(ctypes.byref(self._desc), ctypes.byref(self._opts), device, ctypes.byref(h)))
        self._ctx = h
        self.width = config.scene.camera.width
        self.height = config.scene.camera.height
        if stream is not None:
            self.set_stream(stream)

    # -- reference-named entry points ------------------------------------------------
    def RunIteration(self, algorithm, iteration, spp=1):   # noqa: N802
        _lib.check(self._L.pg3gpu_run_iteration(self._ctx, algorithm, iteration, spp), self._ctx)

    def GetFramebuffer(self):   # noqa: N802
        return self.framebuffer()[0]

    def WasUsed(self):   # noqa: N802
        return self.iterations > 0

    # -- pythonic helpers --------------------------------------------------------------
    run_iteration = RunIteration

    @property
    def iterations(self):
        return int(self._L.pg3gpu_iterations(self._ctx))

    def set_stream(self, stream):
        ptr = stream if isinstance(stream, int) else getattr(stream, "cuda_stream", stream)
        _lib.check(self._L.pg3gpu_set_stream(self._ctx, ctypes.c_void_p(ptr)), self._ctx)

    def synchronize(self):
        _lib.check(self._L.pg3gpu_synchronize(self._ctx), self._ctx)

    def framebuffer(self, with_variance=False):
        n = self.width * self.height * 3
        mean = np.zeros(n, np.float64)
        var = np.zeros(n, np.float64) if with_variance else None
        it = ctypes.c_uint64()
        _lib.check(self._L.pg3gpu_read_framebuffer(
            self._ctx, mean.ctypes.data_as(ctypes.c_void_p),
            var.ctypes.data_as(ctypes.c_void_p) if var is not None else None, ctypes.byref(it)), self._ctx)
        shape = (self.height, self.width, 3)
        return mean.reshape(shape), (var.reshape(shape) if var is not None else None), int(it.value)

    def clear(self):
        _lib.check(self._L.pg3gpu_clear_framebuffer(self._ctx), self._ctx)

    def save_image(self, path, gamma=2.2):
        """The mean image as ``.hdr`` (Radiance RGBE) or, for any other extension, a 24-bit BMP
        with 1/gamma applied (the reference's main program writes gamma 2.2)."""
        _lib.check(self._L.pg3gpu_save_image(self._ctx, os.fsencode(path), gamma), self._ctx)

    def save_steerable(self, path, max_approx_error=5.0):
        """Writes the steerable sampler's triangulation, vertex weights and tree as a ``.emssd``
        file of format 2.1, the reference's sampler cache (see :func:`steerable_file_name`)."""
        _lib.check(self._L.pg3gpu_save_steerable(self._ctx, os.fsencode(path), max_approx_error), self._ctx)

    def load_steerable(self, path):
        """Replaces the steerable sampler's vertex weights with those of a ``.emssd`` file of the
        context's uniform subdivision level (written by the reference or by save_steerable)."""
        _lib.check(self._L.pg3gpu_load_steerable(self._ctx, os.fsencode(path)), self._ctx)

    def render_samples(self, algorithm, iteration, spp):
        out = np.zeros((spp, self.height, self.width, 3), np.float32)
        _lib.check(self._L.pg3gpu_render_samples(self._ctx, algorithm, iteration, spp,
                                                  out.ctypes.data_as(ctypes.c_void_p)), self._ctx)
        return out

    def stats(self):
        s = _lib.Stats()
        _lib.check(self._L.pg3gpu_get_stats(self._ctx, ctypes.byref(s)), self._ctx)
        out = {f: getattr(s, f) for f, _ in _lib.Stats._fields_}
        out["length_histogram"] = list(s.length_histogram)
        return out

    def reset_stats(self):
        _lib.check(self._L.pg3gpu_reset_stats(self._ctx), self._ctx)

    # -- sampler probes (tests) --------------------------------------------------------
    def probe_bsdf(self, material, wol, seed=0):
        wol = np.ascontiguousarray(wol, np.float32)
        n = len(wol)
        wil, ps, pe = np.zeros((n, 3), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
        a_s, a_e = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
        _lib.check(self._L.pg3gpu_probe_bsdf(self._ctx, material, n, p(wol), seed, p(wil), p(ps), p(pe), p(a_s),
                                             p(a_e)), self._ctx)
        return dict(wil=wil, pdf_sampled=ps, pdf_eval=pe, att_sampled=a_s, att_eval=a_e)

    def probe_bsdf_pdf(self, material, wol, wil, with_att=False):
        wol = np.ascontiguousarray(wol, np.float32)
        wil = np.ascontiguousarray(wil, np.float32)
        out = np.zeros(len(wol), np.float32)
        att = np.zeros(len(wol), np.float32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
        _lib.check(self._L.pg3gpu_probe_bsdf_pdf(self._ctx, material, len(wol), p(wol), p(wil), p(out), p(att)),
                   self._ctx)
        return (out, att) if with_att else out

    def probe_light(self, light, points, normals, seed=0):
        pts = np.ascontiguousarray(points, np.float32)
        nrm = np.ascontiguousarray(normals, np.float32)
        n = len(pts)
        d, ps, pe, rc = np.zeros((n, 3), np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32), \
            np.zeros((n, 3), np.float32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
        _lib.check(self._L.pg3gpu_probe_light(self._ctx, light, n, p(pts), p(nrm), seed, p(d), p(ps), p(pe), p(rc)),
                   self._ctx)
        return dict(dirs=d, pdf_sampled=ps, pdf_eval=pe, radiance_cos=rc)

    def probe_light_pdf(self, light, points, normals, dirs):
        pts = np.ascontiguousarray(points, np.float32)
        nrm = np.ascontiguousarray(normals, np.float32)
        dd = np.ascontiguousarray(dirs, np.float32)
        out = np.zeros(len(pts), np.float32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
        _lib.check(self._L.pg3gpu_probe_light_pdf(self._ctx, light, len(pts), p(pts), p(nrm), p(dd), p(out)),
                   self._ctx)
        return out

    def export_bvh(self):
        """(codes, ids, nodes[n-1, 16] float32) of the device LBVH."""
        n = ctypes.c_uint32()
        _lib.check(self._L.pg3gpu_export_bvh(self._ctx, ctypes.byref(n), None, None, None), self._ctx)
        n = n.value
        codes, ids = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        nodes = np.zeros((max(n - 1, 0), 16), np.float32)
        p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
        if n >= 2:
            _lib.check(self._L.pg3gpu_export_bvh(self._ctx, ctypes.byref(ctypes.c_uint32()), p(codes), p(ids),
                                                 p(nodes)), self._ctx)
        return codes, ids, nodes

    def device_framebuffer(self):
        a, b = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(self._L.pg3gpu_device_framebuffer(self._ctx, ctypes.byref(a), ctypes.byref(b)), self._ctx)
        return a.value, b.value

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.pg3gpu_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class GpuBatch:
    """Many scene instances rendered by one persistent wavefront (pg3gpu_batch_* of the C ABI).

    ``configs`` are Config objects (one scene each; ``seeds`` optionally overrides their seeds)
    and ``spp`` the samples per pixel of each instance per run. No counterpart in the reference.
    """

    def __init__(self, configs, spp, seeds=None, device=0):
        n = len(configs)
        self._L = _lib.load()
        self._descs = [_lib.scene_desc(c.scene) for c in configs]
        descs = (_lib.SceneDesc * n)(*self._descs)
        opts = (_lib.Options * n)(*[c.options(None if seeds is None else seeds[i]) for i, c in enumerate(configs)])
        self._keep = (descs, opts)
        spps = (ctypes.c_uint32 * n)(*[int(x) for x in spp])
        h = ctypes.c_void_p()
        st = self._L.pg3gpu_batch_create(descs, opts, spps, n, device, ctypes.byref(h))
        if st:
            raise Pg3Error(st, self._L.pg3gpu_batch_last_error(None).decode(errors="replace"))
        self._b = h
        self.sizes = [(c.scene.camera.height, c.scene.camera.width) for c in configs]
        self.spp = list(spp)

    def _check(self, st):
        if st:
            raise Pg3Error(st, self._L.pg3gpu_batch_last_error(self._b).decode(errors="replace"))

    def run(self):
        self._check(self._L.pg3gpu_batch_run(self._b))

    def synchronize(self):
        self._check(self._L.pg3gpu_batch_synchronize(self._b))

    def clear(self):
        self._check(self._L.pg3gpu_batch_clear(self._b))

    def save_image(self, i, path, gamma=2.2):
        self._check(self._L.pg3gpu_batch_save_image(self._b, i, os.fsencode(path), gamma))

    def framebuffer(self, i, with_variance=False):
        h, w = self.sizes[i]
        mean = np.zeros(h * w * 3, np.float64)
        var = np.zeros(h * w * 3, np.float64) if with_variance else None
        it = ctypes.c_uint64()
        self._check(self._L.pg3gpu_batch_read_framebuffer(
            self._b, i, mean.ctypes.data_as(ctypes.c_void_p),
            var.ctypes.data_as(ctypes.c_void_p) if var is not None else None, ctypes.byref(it)))
        return mean.reshape(h, w, 3), (var.reshape(h, w, 3) if var is not None else None), int(it.value)

    def tuning(self):
        t = _lib.BatchTuning()
        self._check(self._L.pg3gpu_batch_get_tuning(self._b, ctypes.byref(t)))
        return dict(capacity=t.capacity, block_size=t.block_size, blocks_per_sm=t.blocks_per_sm,
                    regen_threshold=t.regen_threshold, use_graph=t.use_graph)

    def set_tuning(self, capacity=0, block_size=0, blocks_per_sm=0, regen_threshold=0.0, use_graph=1):
        t = _lib.BatchTuning(capacity, block_size, blocks_per_sm, regen_threshold, use_graph)
        self._check(self._L.pg3gpu_batch_set_tuning(self._b, ctypes.byref(t)))

    def autotune(self, max_trials=16):
        t = _lib.BatchTuning()
        self._check(self._L.pg3gpu_batch_autotune(self._b, max_trials, ctypes.byref(t)))
        return self.tuning()

    def stats(self):
        s = _lib.Stats()
        self._check(self._L.pg3gpu_batch_get_stats(self._b, ctypes.byref(s)))
        out = {f: getattr(s, f) for f, _ in _lib.Stats._fields_}
        out["length_histogram"] = list(s.length_histogram)
        return out

    def set_stream(self, stream):
        ptr = stream if isinstance(stream, int) else getattr(stream, "cuda_stream", stream)
        self._check(self._L.pg3gpu_batch_set_stream(self._b, ctypes.c_void_p(ptr)))

    def close(self):
        if getattr(self, "_b", None):
            self._L.pg3gpu_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def render(config: Config, spp=None, seed=None, device=0):
    """Convenience: renders config.iterations (or spp) samples and returns the mean image."""
    with GpuPathTracer(config, seed=seed, device=device) as r:
        r.RunIteration(config.algorithm, 0, spp or config.iterations)
        return r.GetFramebuffer()
