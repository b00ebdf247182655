"""Scene descriptions for the path-tracing hot path.

A :class:`Scene` holds exactly what the reference's ``Scene`` exposes to its
renderers (src/scene.hxx:1276-1289): a camera, a material table, triangles and
spheres with material ids, area lights bound to emitting materials
(``mMaterial2Light``), and an optional background light (constant radiance or
a lat-long environment map).  It serialises to

* plain C structs for the C ABI (:mod:`pg3render_gb300._lib`), and
* the line-oriented text format read by the CPU oracle and the reference
  harness (``oracle/``).

The builders below construct the workloads the benchmarks use: the closed
Cornell box lit by a ceiling quad light, the same box opened at the top and lit
by a synthetic environment map, and seeded random variants of both.
"""
from __future__ import annotations

import dataclasses
import math
import os
import struct
from typing import List, Optional, Sequence, Tuple

import numpy as np

Vec3 = Tuple[float, float, float]

# Material kinds (values match include/pg3gpu.h PG3GPU_MAT_*).
MAT_LAMBERT = 0
MAT_GGX_CONDUCTOR = 1
MAT_GGX_DIELECTRIC = 2
MAT_PHONG = 3
MAT_SMOOTH_CONDUCTOR = 4
MAT_SMOOTH_DIELECTRIC = 5
MAT_SRA_LAYERED = 6

# Copper IOR and absorbance at ~590 nm, and the IOR of air, as the reference
# defines them (src/materials.hxx:22-27).
AIR_IOR = 1.000277
GLASS_IOR = 1.51
COPPER_IOR = 0.468
COPPER_ABSORB = 2.81
SILVER_IOR = 0.121
SILVER_ABSORB = 3.66
GOLD_IOR = 0.236
GOLD_ABSORB = 2.960089


@dataclasses.dataclass
class Material:
    kind: int
    albedo: Vec3 = (0.0, 0.0, 0.0)     # Lambert reflectance; Phong diffuse reflectance (as held)
    alpha: float = 0.1                 # GGX roughness (clamped to [0.001, 1] by the renderer)
    ior: float = 1.5                   # inner IOR
    ior_outer: float = 1.0             # outer IOR
    absorb: float = 0.0                # conductor k
    glossy: Vec3 = (0.0, 0.0, 0.0)     # Phong glossy reflectance
    phong_exponent: float = 1.0        # Phong lobe exponent
    # SRA layered: outer GGX dielectric (alpha, ior, ior_outer), inner Lambert (albedo) or GGX
    # conductor (inner_alpha, inner_ior, inner_ior_outer, absorb), medium between them
    inner_kind: int = 0
    inner_alpha: float = 0.1
    inner_ior: float = 1.0
    inner_ior_outer: float = 1.0
    medium_attenuation: Vec3 = (0.0, 0.0, 0.0)
    medium_thickness: float = 0.0


def phong(diffuse: Vec3, glossy: Vec3, exponent: float, use_diffuse: bool = True, use_glossy: bool = True) -> Material:
    """PhongMaterial(aDiffuseReflectance, aGlossyReflectance, aPhongExponent, aDiffuse, aGlossy)
    (src/materials.hxx:366-381): a disabled component is zero, and the diffuse part is halved
    when the glossy lobe is on."""
    d = tuple(float(x) for x in diffuse) if use_diffuse else (0.0, 0.0, 0.0)
    g = tuple(float(x) for x in glossy) if use_glossy else (0.0, 0.0, 0.0)
    if use_glossy:
        d = tuple(x / 2.0 for x in d)   # (equal to halving the float32 value: the ABI stores float32)
    return Material(MAT_PHONG, albedo=d, glossy=g, phong_exponent=float(exponent))


@dataclasses.dataclass
class Camera:
    position: Vec3
    forward: Vec3
    up: Vec3
    width: int
    height: int
    hfov_deg: float = 45.0


@dataclasses.dataclass
class Scene:
    camera: Camera
    materials: List[Material] = dataclasses.field(default_factory=list)
    # (p0, p1, p2, material)
    triangles: List[Tuple[Vec3, Vec3, Vec3, int]] = dataclasses.field(default_factory=list)
    # (center, radius, material)
    spheres: List[Tuple[Vec3, float, int]] = dataclasses.field(default_factory=list)
    # (triangle index, radiance rgb); the triangle's material is the light's emitter
    area_lights: List[Tuple[int, Vec3]] = dataclasses.field(default_factory=list)
    # (position, power rgb): point lights, light ids after the area lights
    point_lights: List[Tuple[Vec3, Vec3]] = dataclasses.field(default_factory=list)
    background_const: Optional[Vec3] = None
    env_map: Optional[np.ndarray] = None   # float32 [H, W, 3], row 0 = theta 0 (+z)
    name: str = "scene"

    # ------------------------------------------------------------------ build
    def add_material(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_triangle(self, p0, p1, p2, mat) -> int:
        self.triangles.append((tuple(map(float, p0)), tuple(map(float, p1)), tuple(map(float, p2)), int(mat)))
        return len(self.triangles) - 1

    def add_quad(self, a, b, c, d, mat, normal) -> Tuple[int, int]:
        """Two triangles (a,b,c) and (c,d,a), wound so that their geometric
        normal cross(p1-p0, p2-p0) points along ``normal``."""
        a, b, c, d = (np.asarray(v, dtype=np.float64) for v in (a, b, c, d))
        n = np.cross(b - a, c - a)
        if np.dot(n, np.asarray(normal, dtype=np.float64)) < 0:
            a, b, c, d = a, d, c, b
        return self.add_triangle(a, b, c, mat), self.add_triangle(c, d, a, mat)

    @property
    def num_lights(self) -> int:
        return len(self.area_lights) + len(self.point_lights) + (1 if self.has_background else 0)

    @property
    def has_background(self) -> bool:
        return self.background_const is not None or self.env_map is not None

    # -------------------------------------------------------------- text form
    def to_text(self, em_path: Optional[str] = None, algorithm: str = "pt",
                min_path_length: int = 1, max_path_length: int = 8, splitting=None) -> str:
        """splitting: optional (budget, level, light_to_bsdf_ratio, indirect_clipping)."""
        c = self.camera
        out = ["# %s" % self.name,
               "camera %r %r %r  %r %r %r  %r %r %r  %d %d %r" % (
                   *c.position, *c.forward, *c.up, c.width, c.height, c.hfov_deg)]
        for m in self.materials:
            if m.kind == MAT_LAMBERT:
                out.append("lambert %r %r %r" % tuple(m.albedo))
            elif m.kind == MAT_GGX_CONDUCTOR:
                out.append("ggx_conductor %r %r %r %r" % (m.alpha, m.ior, m.ior_outer, m.absorb))
            elif m.kind == MAT_GGX_DIELECTRIC:
                out.append("ggx_dielectric %r %r %r" % (m.alpha, m.ior, m.ior_outer))
            elif m.kind == MAT_PHONG:
                out.append("phong %r %r %r %r %r %r %r" % (*m.albedo, *m.glossy, m.phong_exponent))
            elif m.kind == MAT_SMOOTH_CONDUCTOR:
                out.append("smooth_conductor %r %r %r" % (m.ior, m.ior_outer, m.absorb))
            elif m.kind == MAT_SMOOTH_DIELECTRIC:
                out.append("smooth_dielectric %r %r" % (m.ior, m.ior_outer))
            elif m.kind == MAT_SRA_LAYERED:
                inner = ("lambert %r %r %r" % tuple(m.albedo) if m.inner_kind == MAT_LAMBERT else
                         "ggx_conductor %r %r %r %r" % (m.inner_alpha, m.inner_ior, m.inner_ior_outer, m.absorb))
                out.append("sra %r %r %r %s %r %r %r %r" % (m.alpha, m.ior, m.ior_outer, inner, *m.medium_attenuation,
                                                          m.medium_thickness))
            else:
                raise ValueError("unknown material kind %d" % m.kind)
        light_of = {ti: rad for ti, rad in self.area_lights}
        for i, (p0, p1, p2, mat) in enumerate(self.triangles):
            coords = "%r %r %r %r %r %r %r %r %r" % (*p0, *p1, *p2)
            if i in light_of:
                out.append("area_light %s %d %r %r %r" % (coords, mat, *light_of[i]))
            else:
                out.append("triangle %s %d" % (coords, mat))
        for (cc, r, mat) in self.spheres:
            out.append("sphere %r %r %r %r %d" % (*cc, r, mat))
        for (pos, power) in self.point_lights:
            out.append("point_light %r %r %r %r %r %r" % (*pos, *power))
        if self.env_map is not None:
            if em_path is None:
                raise ValueError("environment map scenes need em_path")
            out.append("background_em %s" % em_path)
        elif self.background_const is not None:
            out.append("background_const %r %r %r" % tuple(self.background_const))
        opts = "options %s %d %d" % (algorithm, min_path_length, max_path_length)
        if splitting is not None:
            opts += " %d %r %r %r" % (int(splitting[0]), float(splitting[1]), float(splitting[2]), float(splitting[3]))
        out.append(opts)
        return "\n".join(out) + "\n"

    def write_env_map(self, path: str) -> None:
        write_env_map(path, self.env_map)


def write_env_map(path: str, em: np.ndarray) -> None:
    """Raw lat-long format shared with the oracle: 'PG3F', uint32 W, H, 3,
    then float32 RGB rows from theta = 0 downwards."""
    em = np.ascontiguousarray(em, dtype=np.float32)
    h, w, ch = em.shape
    assert ch == 3
    with open(path, "wb") as f:
        f.write(b"PG3F" + struct.pack("<III", w, h, 3))
        f.write(em.tobytes())


def read_env_map(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        if f.read(4) != b"PG3F":
            raise ValueError("not an environment map file")
        w, h, ch = struct.unpack("<III", f.read(12))
        data = np.frombuffer(f.read(w * h * ch * 4), dtype=np.float32)
    return data.reshape(h, w, ch).copy()


# ---------------------------------------------------------------------------
# Synthetic environment map
# ---------------------------------------------------------------------------
def latlong_dirs(width: int, height: int) -> np.ndarray:
    """Unit directions of the pixel centres of a lat-long map, using the
    reference's mapping (src/geom.hxx:65-95): phi = -(u - 0.5) * 2pi,
    theta = v * pi, dir = (sin t cos p, sin t sin p, cos t)."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = -(u - 0.5) * 2.0 * math.pi
    theta = v * math.pi
    st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
    return np.stack([st * np.cos(phi)[None, :], st * np.sin(phi)[None, :],
                     np.broadcast_to(ct, (height, width))], axis=-1)


def synthetic_sky(width: int, height: int, seed: int = 7, n_lobes: int = 3,
                  peak_to_mean: float = 1.0e4, sigma_deg: Tuple[float, float] = (1.0, 3.0)) -> np.ndarray:
    """Seeded procedural sky: a zenith-to-horizon gradient, a dim ground and
    ``n_lobes`` Gaussian sun lobes of angular sigma in ``sigma_deg``, scaled so
    that the lobe peak is ``peak_to_mean`` times the mean of the sky without
    its lobes."""
    rng = np.random.default_rng(seed)
    d = latlong_dirs(width, height)
    cz = d[..., 2]
    zenith = np.array([0.25, 0.45, 0.95])
    horizon = np.array([0.85, 0.90, 1.00])
    ground = np.array([0.20, 0.17, 0.14])
    t = np.clip(cz, 0.0, 1.0)[..., None]
    sky = horizon * (1.0 - t) + zenith * t
    img = np.where(cz[..., None] > 0.0, sky, ground * (0.6 + 0.4 * np.clip(-cz, 0, 1))[..., None])
    img = img.astype(np.float64)
    lobes = np.zeros(img.shape[:2], dtype=np.float64)
    for _ in range(n_lobes):
        # lobe centres in the upper hemisphere, 10..70 degrees above the horizon
        elev = math.radians(rng.uniform(10.0, 70.0))
        az = rng.uniform(0.0, 2.0 * math.pi)
        c = np.array([math.cos(elev) * math.cos(az), math.cos(elev) * math.sin(az), math.sin(elev)])
        sig = math.radians(rng.uniform(*sigma_deg))
        ang = np.arccos(np.clip(d @ c, -1.0, 1.0))
        w = rng.uniform(0.5, 1.0)
        lobes += w * np.exp(-0.5 * (ang / sig) ** 2)
    # lobe peak = peak_to_mean x the mean radiance of the sky without its suns
    base_mean = img.mean()
    gain = peak_to_mean * base_mean / max(lobes.max(), 1e-12)
    sun = np.array([1.0, 0.95, 0.85])
    img = img + gain * lobes[..., None] * sun
    return img.astype(np.float32)


# ---------------------------------------------------------------------------
# Workload builders
# ---------------------------------------------------------------------------
WHITE = (0.76, 0.76, 0.76)
RED = (0.63, 0.065, 0.05)
GREEN = (0.14, 0.45, 0.09)


def _camera_for_box(width: int, height: int, hfov: float = 45.0) -> Camera:
    # pinhole on the axis of the open front face, framing the unit box
    dist = 1.0 / math.tan(math.radians(0.5 * hfov))
    return Camera((0.0, -1.0 - dist, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), width, height, hfov)


def _box(scene: Scene, white: Vec3 = WHITE, left: Vec3 = RED, right: Vec3 = GREEN,
         ceiling: bool = True) -> None:
    mw = scene.add_material(Material(MAT_LAMBERT, white))
    ml = scene.add_material(Material(MAT_LAMBERT, left))
    mr = scene.add_material(Material(MAT_LAMBERT, right))
    # box [-1,1]^3, open at y = -1 (camera side); normals point inwards
    scene.add_quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), mw, (0, 0, 1))      # floor
    if ceiling:
        scene.add_quad((-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1), mw, (0, 0, -1))     # ceiling
    scene.add_quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), mw, (0, -1, 0))         # back
    scene.add_quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), ml, (1, 0, 0))      # left
    scene.add_quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), mr, (-1, 0, 0))         # right


def _ceiling_light(scene: Scene, radiance: float = 25.0, half: float = 0.25, z: float = 0.99) -> None:
    # two emitting triangles, each with its own zero-reflectance material
    # (the reference binds lights to materials one-to-one, src/scene.hxx:784-797)
    m0 = scene.add_material(Material(MAT_LAMBERT, (0.0, 0.0, 0.0)))
    m1 = scene.add_material(Material(MAT_LAMBERT, (0.0, 0.0, 0.0)))
    a, b, c, d = (-half, -half, z), (half, -half, z), (half, half, z), (-half, half, z)
    n = np.cross(np.subtract(b, a), np.subtract(c, a))
    if n[2] > 0:   # emit downwards
        a, b, c, d = a, d, c, b
    t0 = scene.add_triangle(a, b, c, m0)
    t1 = scene.add_triangle(c, d, a, m1)
    scene.area_lights.append((t0, (radiance, radiance, radiance)))
    scene.area_lights.append((t1, (radiance, radiance, radiance)))


def cornell_box(width: int = 256, height: int = 256) -> Scene:
    """Closed box of 10 Lambert triangles (white floor, ceiling, back; red left,
    green right), a Lambert sphere and a GGX conductor sphere (alpha 0.1, copper
    n/k, grey Fresnel) of radius 0.35, and a 0.5x0.5 ceiling quad light of
    radiance 25; pinhole camera with a 45 degree horizontal field of view."""
    s = Scene(_camera_for_box(width, height), name="cornell_area_%dx%d" % (width, height))
    _box(s)
    m_diff = s.add_material(Material(MAT_LAMBERT, (0.70, 0.70, 0.70)))
    m_cond = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=0.1, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                     absorb=COPPER_ABSORB))
    s.spheres.append(((-0.45, 0.25, -0.65), 0.35, m_diff))
    s.spheres.append(((0.45, -0.25, -0.65), 0.35, m_cond))
    _ceiling_light(s)
    return s


def cornell_env(width: int = 512, height: int = 512, em_width: int = 1024, em_height: int = 512,
                em_seed: int = 7) -> Scene:
    """The same box with the ceiling removed, lit by a synthetic lat-long sky;
    spheres are a rough GGX dielectric (alpha 0.3, IOR 1.5) and a GGX
    conductor (alpha 0.05)."""
    s = Scene(_camera_for_box(width, height), name="cornell_env_%dx%d_em%dx%d" % (width, height, em_width, em_height))
    _box(s, ceiling=False)
    m_diel = s.add_material(Material(MAT_GGX_DIELECTRIC, alpha=0.3, ior=1.5, ior_outer=1.0))
    m_cond = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=0.05, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                     absorb=COPPER_ABSORB))
    s.spheres.append(((-0.45, 0.25, -0.65), 0.35, m_diel))
    s.spheres.append(((0.45, -0.25, -0.65), 0.35, m_cond))
    s.env_map = synthetic_sky(em_width, em_height, seed=em_seed)
    return s


def cornell_env_area(width: int = 512, height: int = 512, em_width: int = 1024, em_height: int = 512,
                     em_seed: int = 7) -> Scene:
    """cornell_env with the 0.5x0.5 light quad of radiance 25 under its open top: an environment
    map and area lights in one scene (light picking includes the background)."""
    s = cornell_env(width, height, em_width, em_height, em_seed)
    s.name = "cornell_envarea_%dx%d_em%dx%d" % (width, height, em_width, em_height)
    _ceiling_light(s)
    return s


def cornell_box_bg(width: int = 256, height: int = 256, background=(0.4, 0.5, 0.7)) -> Scene:
    """cornell_box with a constant background seen through the open front (area lights and a
    background light in one scene)."""
    s = cornell_box(width, height)
    s.name = "cornell_areabg_%dx%d" % (width, height)
    s.background_const = tuple(background)
    return s


def _mixed_materials_box(s: Scene, ceiling: bool) -> None:
    # Phong walls: the box's reflectances as the diffuse part (halved by the glossy lobe) and a
    # grey glossy lobe of 0.5, exponent 90, like the reference's glossy-walls box
    mw = s.add_material(phong(WHITE, (0.5, 0.5, 0.5), 90))
    ml = s.add_material(phong(RED, (0.5, 0.5, 0.5), 90))
    mr = s.add_material(phong(GREEN, (0.5, 0.5, 0.5), 90))
    s.add_quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), mw, (0, 0, 1))
    if ceiling:
        s.add_quad((-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1), mw, (0, 0, -1))
    s.add_quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), mw, (0, -1, 0))
    s.add_quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), ml, (1, 0, 0))
    s.add_quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), mr, (-1, 0, 0))
    m_phong = s.add_material(phong((0.803922, 0.803922, 0.152941), (0.7, 0.7, 0.7), 200))
    m_metal = s.add_material(Material(MAT_SMOOTH_CONDUCTOR, ior=COPPER_IOR, ior_outer=AIR_IOR, absorb=COPPER_ABSORB))
    m_glass = s.add_material(Material(MAT_SMOOTH_DIELECTRIC, ior=GLASS_IOR, ior_outer=AIR_IOR))
    s.spheres.append(((-0.45, 0.25, -0.65), 0.35, m_phong))
    s.spheres.append(((0.45, -0.25, -0.65), 0.35, m_metal))
    s.spheres.append(((-0.35, -0.5, -0.75), 0.25, m_glass))


def cornell_mixed(width: int = 256, height: int = 256, area: bool = True, point: bool = True,
                  sra: bool = False) -> Scene:
    """The closed box with the reference's other materials and a point light: Phong walls
    (diffuse + grey glossy 0.5, exponent 90), a Phong sphere (yellow diffuse, glossy 0.7, exponent
    200), a smooth copper sphere and a smooth glass sphere (IOR 1.51 in air), lit by the ceiling
    quad light and/or a 20 W point light under the ceiling. With ``sra`` the Phong sphere is an
    SRA layered one (GGX glass coat alpha 0.05 over an orange Lambert base, a 0.01 thick blue
    medium); the reference renders that material with the one-hit algorithms only."""
    s = Scene(_camera_for_box(width, height),
              name="cornell_mixed%s%s%s_%dx%d" % ("_area" if area else "", "_point" if point else "",
                                                 "_sra" if sra else "", width, height))
    _mixed_materials_box(s, ceiling=True)
    if sra:
        s.materials[s.spheres[0][2]] = Material(MAT_SRA_LAYERED, alpha=0.05, ior=GLASS_IOR, ior_outer=AIR_IOR,
                                                albedo=(0.81, 0.18, 0.06), inner_kind=MAT_LAMBERT,
                                                medium_attenuation=(5.0, 2.5, 0.5), medium_thickness=0.01)
    if area:
        _ceiling_light(s)
    if point:
        s.point_lights.append(((0.0, 0.0, 0.6), (20.0, 20.0, 20.0)))
    return s


def cornell_env_mixed(width: int = 256, height: int = 256, em_width: int = 512, em_height: int = 256,
                      em_seed: int = 7) -> Scene:
    """cornell_mixed with the ceiling removed, lit by the synthetic sky and the point light."""
    s = Scene(_camera_for_box(width, height), name="cornell_envmixed_%dx%d_em%dx%d" % (width, height, em_width, em_height))
    _mixed_materials_box(s, ceiling=False)
    s.point_lights.append(((0.0, 0.0, 0.6), (20.0, 20.0, 20.0)))
    s.env_map = synthetic_sky(em_width, em_height, seed=em_seed)
    return s


def icosphere(level: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosahedron subdivided 4-way ``level`` times with midpoints pushed to the sphere:
    (vertices [V, 3] float64, faces [20 * 4^level, 3] int, counter-clockwise seen from outside)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.asarray(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(level):
        mid = {}

        def m(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                p = verts[a] + verts[b]
                verts.append(p / np.linalg.norm(p))
                mid[key] = len(verts) - 1
            return mid[key]
        nf = []
        for a, b, c in faces:
            ab, bc, ca = m(a, b), m(b, c), m(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces)


def cornell_env_mesh(width: int = 512, height: int = 512, em_width: int = 1024, em_height: int = 512,
                     level: int = 5, em_seed: int = 7) -> Scene:
    """cornell_env with its two spheres as triangle meshes (icospheres of ``level`` subdivisions,
    20 * 4^level flat triangles each; 40968 triangles in all at level 5): the closest-hit and
    any-hit queries run through the device LBVH instead of the primitive list."""
    s = Scene(_camera_for_box(width, height), name="cornell_envmesh_%dx%d_l%d" % (width, height, level))
    _box(s, ceiling=False)
    m_diel = s.add_material(Material(MAT_GGX_DIELECTRIC, alpha=0.3, ior=1.5, ior_outer=1.0))
    m_cond = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=0.05, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                     absorb=COPPER_ABSORB))
    verts, faces = icosphere(level)
    for centre, mat in (((-0.45, 0.25, -0.65), m_diel), ((0.45, -0.25, -0.65), m_cond)):
        p = verts * 0.35 + np.asarray(centre)
        for a, b, c in faces:
            s.add_triangle(p[a], p[b], p[c], mat)
    s.env_map = synthetic_sky(em_width, em_height, seed=em_seed)
    return s


def cornell_env_diff(width: int = 256, height: int = 256, em_width: int = 512, em_height: int = 256,
                     em_seed: int = 7) -> Scene:
    """The environment-lit box for gradients: four Lambert materials (floor, back wall, red
    left, green right), the two spheres of cornell_env (GGX dielectric alpha 0.3, GGX
    conductor alpha 0.05) and two smaller ones (GGX conductor alpha 0.2, GGX dielectric
    alpha 0.15), i.e. four albedo triples and four roughnesses."""
    s = Scene(_camera_for_box(width, height), name="cornell_diff_%dx%d_em%dx%d" % (width, height, em_width, em_height))
    m_floor = s.add_material(Material(MAT_LAMBERT, WHITE))
    m_back = s.add_material(Material(MAT_LAMBERT, (0.55, 0.60, 0.70)))
    m_left = s.add_material(Material(MAT_LAMBERT, RED))
    m_right = s.add_material(Material(MAT_LAMBERT, GREEN))
    s.add_quad((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), m_floor, (0, 0, 1))
    s.add_quad((-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1), m_back, (0, -1, 0))
    s.add_quad((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1), m_left, (1, 0, 0))
    s.add_quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1), m_right, (-1, 0, 0))
    m_diel = s.add_material(Material(MAT_GGX_DIELECTRIC, alpha=0.3, ior=1.5, ior_outer=1.0))
    m_cond = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=0.05, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                     absorb=COPPER_ABSORB))
    m_cond2 = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=0.2, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                      absorb=COPPER_ABSORB))
    m_diel2 = s.add_material(Material(MAT_GGX_DIELECTRIC, alpha=0.15, ior=1.5, ior_outer=1.0))
    s.spheres.append(((-0.45, 0.25, -0.65), 0.35, m_diel))
    s.spheres.append(((0.45, -0.25, -0.65), 0.35, m_cond))
    s.spheres.append(((0.5, 0.6, -0.8), 0.2, m_cond2))
    s.spheres.append(((-0.55, -0.45, -0.8), 0.2, m_diel2))
    s.env_map = synthetic_sky(em_width, em_height, seed=em_seed)
    return s


def random_variant(seed: int, em_width: int = 256, em_height: int = 128,
                   side_range: Tuple[int, int] = (64, 512), spp_range: Tuple[int, int] = (4, 64),
                   max_spheres: int = 8, use_env: Optional[bool] = None):
    """One seeded Cornell-box variant: side log-uniform in ``side_range``, spp
    uniform in ``spp_range``, 0..max_spheres spheres of radius 0.1-0.4 with
    albedo U[0.05,0.9]^3 or GGX (alpha log-uniform in [0.01,0.8]), lit by the
    ceiling quad light or (every other seed by default) a synthetic sky.
    Returns (scene, spp)."""
    rng = np.random.default_rng(seed)
    side = int(round(math.exp(rng.uniform(math.log(side_range[0]), math.log(side_range[1])))))
    spp = int(rng.integers(spp_range[0], spp_range[1] + 1))
    if use_env is None:
        use_env = (seed % 2) == 1
    s = Scene(_camera_for_box(side, side), name="variant_%d" % seed)
    _box(s, white=tuple(rng.uniform(0.05, 0.9, 3)), left=tuple(rng.uniform(0.05, 0.9, 3)),
         right=tuple(rng.uniform(0.05, 0.9, 3)), ceiling=not use_env)
    n_sph = int(rng.integers(0, max_spheres + 1))
    placed = []
    for _ in range(n_sph):
        r = float(rng.uniform(0.1, 0.4))
        for _try in range(50):
            c = (float(rng.uniform(-1 + r, 1 - r)), float(rng.uniform(-1 + r, 1 - r)), -1.0 + r)
            if all((c[0] - q[0]) ** 2 + (c[1] - q[1]) ** 2 > (r + qr) ** 2 for q, qr in placed):
                break
        placed.append((c, r))
        kind = int(rng.integers(0, 3))
        alpha = float(math.exp(rng.uniform(math.log(0.01), math.log(0.8))))
        if kind == 0:
            m = s.add_material(Material(MAT_LAMBERT, tuple(rng.uniform(0.05, 0.9, 3))))
        elif kind == 1:
            m = s.add_material(Material(MAT_GGX_CONDUCTOR, alpha=alpha, ior=COPPER_IOR, ior_outer=AIR_IOR,
                                        absorb=COPPER_ABSORB))
        else:
            m = s.add_material(Material(MAT_GGX_DIELECTRIC, alpha=alpha, ior=1.5, ior_outer=1.0))
        s.spheres.append((c, r, m))
    if use_env:
        s.env_map = synthetic_sky(em_width, em_height, seed=seed + 1000)
    else:
        _ceiling_light(s)
    return s, spp
