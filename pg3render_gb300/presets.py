"""The reference's built-in scenes: the Cornell-box family of ``Scene::LoadCornellBox``
(src/scene.hxx:176-1000) selected by a box mask, and the 39 numbered configurations the
command line's ``-s`` option picks (``g_SceneConfigs``, src/config.hxx:36-115).

The geometry, materials and lights follow the reference's construction: the same vertices,
the same material table (ids 0-12), lights of the same power. Environment-map types that the
reference reads from OpenEXR light probes need the caller's texels (``env_map``, float32
[H, W, 3], row 0 at theta = 0): there is no EXR decoder here. Two cases differ:

* the SRA layered sphere material (``SPHERES_SRA_LAYERS``, configuration 27) renders with the
  one-hit algorithms only, as in the reference, whose path tracers stop on it;
* the vertical GGX-dielectric rectangle (configuration 29) samples lights from its front side
  only (the reference also from its back side); the estimate keeps its expectation, only its
  noise differs.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np

from . import scene as S

# BoxMask flags (src/scene.hxx:117-151)
LIGHT_CEILING = 0x00000001
LIGHT_BOX = 0x00000002
LIGHT_POINT = 0x00000004
LIGHT_ENV = 0x00000008
SPHERES_2 = 0x00000010
SPHERE_1 = 0x00000020
VERTICAL_RECTANGLE = 0x00000040
DIAGONAL_RECTANGLES = 0x00000080
WALLS = 0x00000100
FLOOR = 0x00000200
LAYERED_SPHERE = 0x10000000
SPHERES_PHONG_DIFFUSE = 0x00001000
SPHERES_PHONG_GLOSSY = 0x00002000
WALLS_PHONG_DIFFUSE = 0x00004000
WALLS_PHONG_GLOSSY = 0x00008000
SPHERES_FRESNEL_CONDUCTOR = 0x00010000
SPHERES_FRESNEL_DIELECTRIC = 0x00020000
SPHERES_GGX_CONDUCTOR = 0x00040000
SPHERES_GGX_DIELECTRIC = 0x00080000
SPHERES_SRA_LAYERS = 0x00100000
VERT_RECT_FRESNEL_DIELECTRIC = 0x00200000
VERT_RECT_GGX_DIELECTRIC = 0x00400000
DEFAULT = LIGHT_CEILING | WALLS | SPHERES_2 | SPHERES_PHONG_DIFFUSE | WALLS_PHONG_DIFFUSE

# Environment-map types (src/scene.hxx:154-174): the constant ones are built in, the others
# are the reference's EXR light probes and need env_map
EM_CONST_BLUISH = 0
EM_CONST_SRGB_WHITE = 1
EM_IMG_CONST_WHITE_8x4 = 2
EM_IMG_CONST_WHITE_1024x512 = 3
EM_IMG_DEBUG_SINGLE_PIXEL = 4
EM_IMG_PISA = 5
EM_IMG_GLACIER = 6
EM_IMG_DOGE2 = 7
EM_IMG_PLAYA_SUNRISE = 8
EM_IMG_ENNIS = 9
EM_IMG_SATELLITE = 10
EM_IMG_PEACE_GARDENS_DUSK = 11
EM_IMG_SYNTH_THREE_POINT = 12

_FULL_BOX = WALLS | FLOOR | SPHERES_2
_2SPHERES_ON_FLOOR = FLOOR | SPHERES_2
_BOX_1SPHERE = WALLS | FLOOR | SPHERE_1
_1SPHERE = SPHERE_1
_RECTANGLES = VERTICAL_RECTANGLE | DIAGONAL_RECTANGLES
_DIFFUSE = WALLS_PHONG_DIFFUSE | SPHERES_PHONG_DIFFUSE
_GLOSSY = WALLS_PHONG_GLOSSY | SPHERES_PHONG_GLOSSY

# g_SceneConfigs (src/config.hxx:45-115): the -s scene ids 0-38
SCENE_CONFIGS = [
    LIGHT_POINT | _FULL_BOX | _DIFFUSE,                                                  # 0
    LIGHT_POINT | _FULL_BOX | _DIFFUSE | _GLOSSY,                                        # 1
    LIGHT_CEILING | _FULL_BOX | _DIFFUSE,                                                # 2
    LIGHT_CEILING | _FULL_BOX | _DIFFUSE | _GLOSSY,                                      # 3
    LIGHT_BOX | _FULL_BOX | _DIFFUSE,                                                    # 4
    LIGHT_BOX | _FULL_BOX | _DIFFUSE | _GLOSSY,                                          # 5
    LIGHT_ENV | _FULL_BOX | _DIFFUSE,                                                    # 6
    LIGHT_ENV | _FULL_BOX | _DIFFUSE | _GLOSSY,                                          # 7
    LIGHT_ENV | _2SPHERES_ON_FLOOR | _DIFFUSE,                                           # 8
    LIGHT_ENV | _2SPHERES_ON_FLOOR | _DIFFUSE | _GLOSSY,                                 # 9
    LIGHT_BOX | LIGHT_ENV | _FULL_BOX | _DIFFUSE,                                        # 10
    LIGHT_POINT | LIGHT_BOX | _FULL_BOX | _DIFFUSE,                                      # 11
    LIGHT_POINT | LIGHT_BOX | LIGHT_ENV | _FULL_BOX | _DIFFUSE,                          # 12
    LIGHT_POINT | LIGHT_BOX | LIGHT_ENV | _2SPHERES_ON_FLOOR | _DIFFUSE,                 # 13
    LIGHT_POINT | LIGHT_BOX | LIGHT_ENV | _2SPHERES_ON_FLOOR | _DIFFUSE | _GLOSSY,       # 14
    LIGHT_POINT | LIGHT_BOX | LIGHT_ENV | _FULL_BOX | _DIFFUSE | _GLOSSY,                # 15
    LIGHT_POINT | _FULL_BOX | SPHERES_FRESNEL_CONDUCTOR | WALLS_PHONG_DIFFUSE,            # 16
    LIGHT_BOX | _FULL_BOX | SPHERES_FRESNEL_CONDUCTOR | WALLS_PHONG_DIFFUSE,              # 17
    LIGHT_CEILING | _FULL_BOX | SPHERES_FRESNEL_CONDUCTOR | WALLS_PHONG_DIFFUSE,          # 18
    LIGHT_BOX | _FULL_BOX | SPHERES_FRESNEL_CONDUCTOR | WALLS_PHONG_DIFFUSE | WALLS_PHONG_GLOSSY,  # 19
    LIGHT_ENV | _1SPHERE | SPHERES_PHONG_DIFFUSE,                                        # 20
    LIGHT_ENV | _1SPHERE | SPHERES_PHONG_GLOSSY,                                         # 21
    LIGHT_ENV | _1SPHERE | SPHERES_PHONG_DIFFUSE | SPHERES_PHONG_GLOSSY,                  # 22
    LIGHT_ENV | _1SPHERE | SPHERES_FRESNEL_CONDUCTOR,                                    # 23
    LIGHT_ENV | _1SPHERE | SPHERES_FRESNEL_DIELECTRIC,                                   # 24
    LIGHT_ENV | _1SPHERE | SPHERES_GGX_CONDUCTOR,                                        # 25
    LIGHT_ENV | _1SPHERE | SPHERES_GGX_DIELECTRIC,                                       # 26
    LIGHT_ENV | _1SPHERE | SPHERES_SRA_LAYERS,                                           # 27
    LIGHT_ENV | _RECTANGLES | VERT_RECT_FRESNEL_DIELECTRIC,                              # 28
    LIGHT_ENV | _RECTANGLES | VERT_RECT_GGX_DIELECTRIC,                                  # 29
    LIGHT_BOX | _BOX_1SPHERE | SPHERES_FRESNEL_CONDUCTOR | WALLS_PHONG_DIFFUSE,           # 30
    LIGHT_BOX | _BOX_1SPHERE | SPHERES_FRESNEL_DIELECTRIC | WALLS_PHONG_DIFFUSE,          # 31
    LIGHT_BOX | _BOX_1SPHERE | SPHERES_GGX_CONDUCTOR | WALLS_PHONG_DIFFUSE,               # 32
    LIGHT_BOX | _BOX_1SPHERE | SPHERES_GGX_DIELECTRIC | WALLS_PHONG_DIFFUSE,              # 33
    LIGHT_CEILING | _BOX_1SPHERE | SPHERES_GGX_CONDUCTOR | WALLS_PHONG_DIFFUSE,           # 34
    LIGHT_CEILING | _BOX_1SPHERE | SPHERES_GGX_DIELECTRIC | WALLS_PHONG_DIFFUSE,          # 35
    LIGHT_POINT | _BOX_1SPHERE | SPHERES_GGX_DIELECTRIC | WALLS_PHONG_DIFFUSE,            # 36
    LIGHT_ENV | _BOX_1SPHERE | SPHERES_GGX_DIELECTRIC | WALLS_PHONG_DIFFUSE,              # 37
    LIGHT_ENV | LAYERED_SPHERE,                                                          # 38
]

# Cornell-box and light-box corners (src/scene.hxx:437-446, 724-733), float32 like the reference
_CB = np.array([(-1.27029, 1.30455, -1.28002), (1.28975, 1.30455, -1.28002), (1.28975, 1.30455, 1.28002),
                (-1.27029, 1.30455, 1.28002), (-1.27029, -1.25549, -1.28002), (1.28975, -1.25549, -1.28002),
                (1.28975, -1.25549, 1.28002), (-1.27029, -1.25549, 1.28002)], np.float32)
_LB = np.array([(-0.25, 0.25, 1.26002), (0.25, 0.25, 1.26002), (0.25, 0.25, 1.28002), (-0.25, 0.25, 1.28002),
                (-0.25, -0.25, 1.26002), (0.25, -0.25, 1.26002), (0.25, -0.25, 1.28002), (-0.25, -0.25, 1.28002)],
               np.float32)


def _f32(v):
    return np.asarray(v, np.float32)


def _t(v):
    return tuple(float(x) for x in _f32(v))


def _materials(mask: int):
    """The material table, ids 0-12 (src/scene.hxx:199-433)."""
    P, M = S.phong, S.Material
    m = [M(S.MAT_LAMBERT), M(S.MAT_LAMBERT)]   # 0, 1: the two light triangles, emit only
    walls = (bool(mask & WALLS_PHONG_DIFFUSE), bool(mask & WALLS_PHONG_GLOSSY))
    for d in [(0.803922, 0.803922, 0.803922), (0.156863, 0.803922, 0.172549), (0.803922, 0.152941, 0.152941),
              (0.803922, 0.803922, 0.803922)]:                       # 2 floor, 3 left, 4 right, 5 back
        m.append(P(d, (0.5, 0.5, 0.5), 90, *walls))
    sph = (bool(mask & SPHERES_PHONG_DIFFUSE), bool(mask & SPHERES_PHONG_GLOSSY))
    copper = dict(ior=S.COPPER_IOR, ior_outer=S.AIR_IOR, absorb=S.COPPER_ABSORB)
    if mask & SPHERES_FRESNEL_CONDUCTOR:                                      # 6, 7
        m.append(M(S.MAT_SMOOTH_CONDUCTOR, **copper))
        m.append(M(S.MAT_SMOOTH_CONDUCTOR, ior=S.SILVER_IOR, ior_outer=S.AIR_IOR, absorb=S.SILVER_ABSORB))
    elif mask & SPHERES_GGX_CONDUCTOR:
        m.append(M(S.MAT_GGX_CONDUCTOR, alpha=0.1, **copper))
        m.append(M(S.MAT_GGX_CONDUCTOR, alpha=0.1, **copper))
    else:
        m.append(P((0.803922, 0.803922, 0.152941), (0.7, 0.7, 0.7), 200, *sph))
        m.append(P((0.152941, 0.152941, 0.803922), (0.7, 0.7, 0.7), 600, *sph))
    if mask & SPHERES_FRESNEL_CONDUCTOR:                                      # 8 large sphere
        m.append(M(S.MAT_SMOOTH_CONDUCTOR, **copper))
    elif mask & SPHERES_FRESNEL_DIELECTRIC:
        m.append(M(S.MAT_SMOOTH_DIELECTRIC, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR))
    elif mask & SPHERES_GGX_CONDUCTOR:
        m.append(M(S.MAT_GGX_CONDUCTOR, alpha=0.01, **copper))
    elif mask & SPHERES_GGX_DIELECTRIC:
        m.append(M(S.MAT_GGX_DIELECTRIC, alpha=0.01, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR))
    elif mask & SPHERES_SRA_LAYERS:
        # outer GGX dielectric 0.010 glass in air, inner GGX conductor 0.200 silver under glass,
        # a yellow-to-dark-red medium 0.001 thick (the defaults of src/scene.hxx:325-371)
        m.append(M(S.MAT_SRA_LAYERED, alpha=0.01, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR, absorb=S.SILVER_ABSORB,
                   inner_kind=S.MAT_GGX_CONDUCTOR, inner_alpha=0.2, inner_ior=S.SILVER_IOR,
                   inner_ior_outer=S.GLASS_IOR, medium_attenuation=(0.05, 0.8, 4.0), medium_thickness=0.001))
    else:
        m.append(P((0.803922, 0.803922, 0.803922), (0.5, 0.5, 0.5), 90, *sph))
    if mask & VERT_RECT_FRESNEL_DIELECTRIC:                                   # 9 vertical rectangle
        m.append(M(S.MAT_SMOOTH_DIELECTRIC, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR))
    elif mask & VERT_RECT_GGX_DIELECTRIC:
        m.append(M(S.MAT_GGX_DIELECTRIC, alpha=0.1, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR))
    else:
        m.append(P((0.8, 0.8, 0.8), (0.0, 0.0, 0.0), 1, True, False))
    m.append(P((0.8, 0.8, 0.8), (0.0, 0.0, 0.0), 1, True, False))           # 10 diagonal rectangles
    m.append(M(S.MAT_GGX_DIELECTRIC, alpha=0.01, ior=S.GLASS_IOR, ior_outer=S.AIR_IOR))   # 11 layered outer
    m.append(M(S.MAT_GGX_CONDUCTOR, alpha=0.2, ior=S.SILVER_IOR, ior_outer=S.GLASS_IOR,   # 12 layered inner
               absorb=S.SILVER_ABSORB))
    return m


def cornell_box(mask: int = DEFAULT, width: int = 512, height: int = 512, env_type: int = EM_CONST_BLUISH,
                env_map: Optional[np.ndarray] = None) -> S.Scene:
    """Scene::LoadCornellBox(resolution, aux, mask, env_type) (src/scene.hxx:176-1000)."""
    cam = S.Camera((-0.0439815, -4.12529, 0.222539), (0.00688625, 0.998505, -0.0542161),
                   (3.73896e-4, 0.0542148, 0.998529), width, height, 45.0)
    sc = S.Scene(cam, name="reference_box_0x%08x_em%d" % (mask, env_type))
    sc.materials = _materials(mask)
    ceiling, box = bool(mask & LIGHT_CEILING), bool(mask & LIGHT_BOX)
    cb, lb = _CB, _LB
    tri = lambda a, b, c, m: sc.add_triangle(_t(a), _t(b), _t(c), m)   # noqa: E731
    if mask & FLOOR:
        tri(cb[0], cb[4], cb[5], 2)
        tri(cb[5], cb[1], cb[0], 2)
    light_tris = []
    if mask & WALLS:
        tri(cb[3], cb[7], cb[4], 3)
        tri(cb[4], cb[0], cb[3], 3)
        tri(cb[1], cb[5], cb[6], 4)
        tri(cb[6], cb[2], cb[1], 4)
        tri(cb[0], cb[1], cb[2], 5)
        tri(cb[2], cb[3], cb[0], 5)
        if ceiling and not box:
            light_tris = [tri(cb[2], cb[6], cb[7], 0), tri(cb[7], cb[3], cb[2], 1)]
        else:
            tri(cb[2], cb[6], cb[7], 2)
            tri(cb[7], cb[3], cb[2], 2)
    if mask & SPHERES_2:
        r = np.float32(0.5)
        lwc = (cb[0] + cb[4]) * np.float32(0.5) + _f32((0, 0, r))
        rwc = (cb[1] + cb[5]) * np.float32(0.5) + _f32((0, 0, r))
        w = rwc[0] - lwc[0]
        lbc = lwc + _f32((np.float32(2) * w / np.float32(7), 0, 0))
        rbc = rwc - _f32((np.float32(2) * w / np.float32(7), -w / np.float32(4), 0))
        sc.spheres.append((_t(lbc), float(r), 6))
        sc.spheres.append((_t(rbc), float(r), 7))
    if mask & SPHERE_1:
        r = np.float32(1.0)
        c = (cb[0] + cb[5]) * np.float32(0.5) + _f32((0, 0, r))
        sc.spheres.append((_t(c), float(r), 8))
    if mask & LAYERED_SPHERE:
        r = np.float32(1.3)
        c = (cb[0] + cb[5]) * np.float32(0.5) + _f32((0, 0, r))
        sc.spheres.append((_t(c), float(r), 11))
        sc.spheres.append((_t(c), float(r * (np.float32(1) - np.float32(0.01))), 12))
    if mask & DIAGONAL_RECTANGLES:
        front = (cb[4] + cb[5]) * np.float32(0.5)
        back = (cb[3] + cb[2]) * np.float32(0.5)
        hgt, wid = abs(cb[0][2] - cb[3][2]), abs(cb[0][0] - cb[1][0])
        hw, xo, zo = np.float32(0.15) * wid * np.float32(0.5), np.float32(0.6) * wid * np.float32(0.5), np.float32(0.1) * hgt
        for s in (-1, 1):
            q = [front + _f32((-hw + s * xo, 0, zo)), front + _f32((hw + s * xo, 0, zo)),
                 back + _f32((hw + s * xo, 0, zo)), back + _f32((-hw + s * xo, 0, zo))]
            tri(q[3], q[0], q[1], 10)
            tri(q[1], q[2], q[3], 10)
    if mask & VERTICAL_RECTANGLE:
        fc = (cb[0] + cb[5]) * np.float32(0.5)
        wid, hgt, dep = abs(cb[0][0] - cb[1][0]), abs(cb[0][2] - cb[3][2]), abs(cb[0][1] - cb[4][1])
        hw, rh = np.float32(8.0) * wid * np.float32(0.5), np.float32(0.7) * hgt
        yo, zo = np.float32(-1.0) * dep * np.float32(0.5), np.float32(0.1) * hgt
        q = [fc + _f32((-hw, yo, zo)), fc + _f32((hw, yo, zo)), fc + _f32((hw, yo, zo + rh)),
             fc + _f32((-hw, yo, zo + rh))]
        tri(q[3], q[0], q[1], 9)
        tri(q[1], q[2], q[3], 9)
    if box and not ceiling:
        tri(lb[0], lb[2], lb[1], 5)
        tri(lb[2], lb[0], lb[3], 5)
        tri(lb[3], lb[4], lb[7], 5)
        tri(lb[4], lb[3], lb[0], 5)
        tri(lb[1], lb[6], lb[5], 5)
        tri(lb[6], lb[1], lb[2], 5)
        tri(lb[4], lb[5], lb[6], 5)
        tri(lb[6], lb[7], lb[4], 5)
        light_tris = [tri(lb[0], lb[5], lb[4], 0), tri(lb[5], lb[0], lb[1], 1)]
    # lights: 25 W over the two light triangles (radiance = flux / (pi * area),
    # src/lights.hxx:107-112), a 50 W point light, the background last (src/scene.hxx:767-944)
    if (ceiling != box) and light_tris:
        for t in light_tris:
            p0, p1, p2 = (np.asarray(v, np.float32) for v in sc.triangles[t][:3])
            inv_area = np.float32(2.0) / np.float32(np.linalg.norm(np.cross(p1 - p0, p2 - p0)))
            L = float(np.float32(12.5) * (inv_area / np.float32(math.pi)))
            sc.area_lights.append((t, (L, L, L)))
    if mask & LIGHT_POINT:
        sc.point_lights.append(((0.0, -0.5, 1.0), (50.0, 50.0, 50.0)))
    if mask & LIGHT_ENV:
        if env_type == EM_CONST_BLUISH:
            sc.background_const = (135 / 255.0, 206 / 255.0, 250 / 255.0)
        elif env_type == EM_CONST_SRGB_WHITE:
            sc.background_const = (0.87, 0.87, 0.87)
        elif env_map is not None:
            sc.env_map = np.ascontiguousarray(env_map, np.float32)
        else:
            raise ValueError("environment-map type %d is an EXR light probe of the reference: pass its texels "
                             "as env_map" % env_type)
    return sc


def reference_scene(scene_id: int, width: int = 512, height: int = 512, env_type: int = EM_CONST_BLUISH,
                    env_map: Optional[np.ndarray] = None) -> S.Scene:
    """Scene number ``scene_id`` of the reference's -s option (src/config.hxx:45-115,
    src/pg3render.cxx via Config::LoadScene)."""
    if not 0 <= scene_id < len(SCENE_CONFIGS):
        raise ValueError("scene id must be in 0..%d" % (len(SCENE_CONFIGS) - 1))
    sc = cornell_box(SCENE_CONFIGS[scene_id], width, height, env_type, env_map)
    sc.name = "reference_scene_%d" % scene_id
    return sc
