"""ctypes binding of the C ABI declared in include/pg3gpu.h.

The shared library is built in-tree (``pg3render_gb300/_build/libpg3gpu.so``);
loading fails loudly when it is missing -- there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpg3gpu.so")

# status codes / enums (include/pg3gpu.h)
OK, ERR_INVALID_ARGUMENT, ERR_UNSUPPORTED, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_DEVICE_LIMIT = range(6)
ALG_PATH_TRACING_NAIVE, ALG_PATH_TRACING = 6, 7
MAT_LAMBERT, MAT_GGX_CONDUCTOR, MAT_GGX_DIELECTRIC = 0, 1, 2
BG_NONE, BG_CONSTANT, BG_ENVMAP = 0, 1, 2
EM_CDF, EM_COSINE, EM_STEERABLE = 0, 1, 2
TRAVERSAL_AUTO, TRAVERSAL_LIST, TRAVERSAL_BVH, TRAVERSAL_BVH4 = 0, 1, 2, 3
PIPELINE_AUTO, PIPELINE_MEGAKERNEL, PIPELINE_WAVEFRONT = 0, 1, 2
GGX_VNDF_EXACT, GGX_VNDF_REFERENCE_FIT = 0, 1
STEER_WEIGHTS_POINT, STEER_WEIGHTS_PROJECTED = 0, 1

c_float3 = ctypes.c_float * 3


class Camera(ctypes.Structure):
    _fields_ = [("position", c_float3), ("forward", c_float3), ("up", c_float3),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("hfov_deg", ctypes.c_float)]


class Material(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("albedo", c_float3), ("alpha", ctypes.c_float),
                ("ior", ctypes.c_float), ("ior_outer", ctypes.c_float), ("absorb", ctypes.c_float),
                ("glossy", c_float3), ("phong_exponent", ctypes.c_float),
                ("inner_kind", ctypes.c_int32), ("inner_alpha", ctypes.c_float), ("inner_ior", ctypes.c_float),
                ("inner_ior_outer", ctypes.c_float), ("medium_attenuation", c_float3),
                ("medium_thickness", ctypes.c_float)]


class Triangle(ctypes.Structure):
    _fields_ = [("p", ctypes.c_float * 9), ("material", ctypes.c_int32)]


class Sphere(ctypes.Structure):
    _fields_ = [("center", c_float3), ("radius", ctypes.c_float), ("material", ctypes.c_int32)]


class AreaLight(ctypes.Structure):
    _fields_ = [("triangle", ctypes.c_uint32), ("radiance", c_float3)]


class PointLight(ctypes.Structure):
    _fields_ = [("position", c_float3), ("power", c_float3)]


class SceneDesc(ctypes.Structure):
    _fields_ = [("camera", Camera),
                ("materials", ctypes.POINTER(Material)), ("num_materials", ctypes.c_uint32),
                ("triangles", ctypes.POINTER(Triangle)), ("num_triangles", ctypes.c_uint32),
                ("spheres", ctypes.POINTER(Sphere)), ("num_spheres", ctypes.c_uint32),
                ("area_lights", ctypes.POINTER(AreaLight)), ("num_area_lights", ctypes.c_uint32),
                ("background", ctypes.c_int32), ("background_radiance", c_float3),
                ("env_map", ctypes.POINTER(ctypes.c_float)),
                ("env_width", ctypes.c_uint32), ("env_height", ctypes.c_uint32),
                ("point_lights", ctypes.POINTER(PointLight)), ("num_point_lights", ctypes.c_uint32)]


class Options(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int32), ("min_path_length", ctypes.c_uint32),
                ("max_path_length", ctypes.c_uint32), ("rr_min_path_length", ctypes.c_uint32),
                ("indirect_clipping", ctypes.c_float), ("splitting_budget", ctypes.c_uint32),
                ("em_sampler", ctypes.c_int32), ("traversal", ctypes.c_int32), ("pipeline", ctypes.c_int32),
                ("steer_subdiv_level", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("max_paths_in_flight", ctypes.c_uint32), ("ggx_sampler", ctypes.c_int32),
                ("splitting_level", ctypes.c_float), ("light_to_bsdf_ratio", ctypes.c_float),
                ("steer_weights", ctypes.c_int32), ("steer_max_subdiv_level", ctypes.c_uint32),
                ("steer_max_approx_error", ctypes.c_float), ("reserved", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("paths", ctypes.c_uint64), ("extension_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("terminated_by_russian_roulette", ctypes.c_uint64),
                ("terminated_by_background", ctypes.c_uint64), ("terminated_by_blocker", ctypes.c_uint64),
                ("terminated_by_max_limit", ctypes.c_uint64), ("terminated_by_safety_limit", ctypes.c_uint64),
                ("last_iteration_ms", ctypes.c_double), ("path_kernel_ms", ctypes.c_double),
                ("path_kernel_launches", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("length_histogram", ctypes.c_uint64 * 16), ("min_path_length", ctypes.c_uint32),
                ("max_path_length", ctypes.c_uint32)]


class BatchTuning(ctypes.Structure):
    _fields_ = [("capacity", ctypes.c_uint32), ("block_size", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("regen_threshold", ctypes.c_float), ("use_graph", ctypes.c_int32), ("reserved", ctypes.c_uint32 * 3)]


BATCH_MAX_INSTANCES = 128

# every exported symbol, with its ctypes signature (checked against include/pg3gpu.h by the tests)
SIGNATURES = {
    "pg3gpu_default_options": (None, [ctypes.POINTER(Options)]),
    "pg3gpu_create": (ctypes.c_int, [ctypes.POINTER(SceneDesc), ctypes.POINTER(Options), ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_void_p)]),
    "pg3gpu_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_run_iteration": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32]),
    "pg3gpu_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_read_framebuffer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.POINTER(ctypes.c_uint64)]),
    "pg3gpu_clear_framebuffer": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_write_image": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_char_p,
                                          ctypes.c_float]),
    "pg3gpu_save_image": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_float]),
    "pg3gpu_save_steerable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_float]),
    "pg3gpu_load_steerable": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p]),
    "pg3gpu_iterations": (ctypes.c_uint64, [ctypes.c_void_p]),
    "pg3gpu_render_samples": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.c_void_p]),
    "pg3gpu_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "pg3gpu_reset_stats": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_device_framebuffer": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p),
                                                 ctypes.POINTER(ctypes.c_void_p)]),
    "pg3gpu_probe_bsdf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_void_p,
                                         ctypes.c_uint32] + [ctypes.c_void_p] * 5),
    "pg3gpu_probe_bsdf_pdf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32] + [ctypes.c_void_p] * 4),
    "pg3gpu_probe_light": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_uint32] + [ctypes.c_void_p] * 4),
    "pg3gpu_probe_light_pdf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32] + [ctypes.c_void_p] * 4),
    "pg3gpu_export_bvh": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)] + [ctypes.c_void_p] * 3),
    "pg3gpu_steer_triangulate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                ctypes.c_uint32, ctypes.c_float, ctypes.POINTER(ctypes.c_uint32),
                                                ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]),
    "pg3gpu_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_diff_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]),
    "pg3gpu_diff_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_set_sample_offset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_batch_create": (ctypes.c_int, [ctypes.POINTER(SceneDesc), ctypes.POINTER(Options),
                                           ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_void_p)]),
    "pg3gpu_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_batch_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "pg3gpu_batch_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchTuning)]),
    "pg3gpu_batch_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchTuning)]),
    "pg3gpu_batch_run": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_batch_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_batch_read_framebuffer": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                                     ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    "pg3gpu_batch_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "pg3gpu_batch_save_image": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_float]),
    "pg3gpu_batch_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(BatchTuning)]),
    "pg3gpu_batch_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "pg3gpu_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "pg3gpu_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "pg3gpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "pg3gpu_version": (ctypes.c_char_p, []),
}

_lib = None


def load(path=None):
    """Loads libpg3gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("PG3GPU_LIBRARY") or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("pg3gpu: CUDA library not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class Pg3Error(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("pg3gpu status %d (%s): %s" % (status, load().pg3gpu_status_string(status).decode(), msg))
        self.status = status


def check(status, ctx=None):
    if status != OK:
        msg = load().pg3gpu_last_error(ctx).decode(errors="replace")
        raise Pg3Error(status, msg)


def scene_desc(scene):
    """Builds a SceneDesc (and keeps the backing arrays alive on the returned object)."""
    from . import scene as S
    d = SceneDesc()
    c = scene.camera
    d.camera = Camera(c_float3(*c.position), c_float3(*c.forward), c_float3(*c.up), c.width, c.height, c.hfov_deg)
    mats = (Material * max(1, len(scene.materials)))()
    for i, m in enumerate(scene.materials):
        mats[i] = Material(m.kind, c_float3(*m.albedo), m.alpha, m.ior, m.ior_outer, m.absorb,
                           c_float3(*m.glossy), m.phong_exponent, m.inner_kind, m.inner_alpha, m.inner_ior,
                           m.inner_ior_outer, c_float3(*m.medium_attenuation), m.medium_thickness)
    tris = (Triangle * max(1, len(scene.triangles)))()
    for i, (p0, p1, p2, mat) in enumerate(scene.triangles):
        tris[i] = Triangle((ctypes.c_float * 9)(*p0, *p1, *p2), mat)
    sphs = (Sphere * max(1, len(scene.spheres)))()
    for i, (cc, r, mat) in enumerate(scene.spheres):
        sphs[i] = Sphere(c_float3(*cc), r, mat)
    lights = (AreaLight * max(1, len(scene.area_lights)))()
    for i, (ti, rad) in enumerate(scene.area_lights):
        lights[i] = AreaLight(ti, c_float3(*rad))
    d.materials, d.num_materials = mats, len(scene.materials)
    d.triangles, d.num_triangles = tris, len(scene.triangles)
    d.spheres, d.num_spheres = sphs, len(scene.spheres)
    d.area_lights, d.num_area_lights = lights, len(scene.area_lights)
    points = (PointLight * max(1, len(scene.point_lights)))()
    for i, (pos, power) in enumerate(scene.point_lights):
        points[i] = PointLight(c_float3(*pos), c_float3(*power))
    d.point_lights, d.num_point_lights = points, len(scene.point_lights)
    keep = [mats, tris, sphs, lights, points]
    if scene.env_map is not None:
        em = np.ascontiguousarray(scene.env_map, dtype=np.float32)
        d.background = BG_ENVMAP
        d.env_map = em.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        d.env_height, d.env_width = em.shape[0], em.shape[1]
        keep.append(em)
    elif scene.background_const is not None:
        d.background = BG_CONSTANT
        d.background_radiance = c_float3(*scene.background_const)
    else:
        d.background = BG_NONE
    d._keep = keep
    return d
