"""Steerable-sampler data files (".emssd", format 2.1): pg3gpu_save_steerable and
pg3gpu_load_steerable against files the reference's own EnvironmentMapSteerableSampler wrote
(tests/golden/emssd_ref.npz, made by `tests/golden/make_golden.py emssd`) for the 64x32 sky of
the environment-map box: a uniform triangulation (minimum = maximum subdivision level 2) and an
adaptive one (levels 1-3). The CPU tests read the reference's files with a reader restated here
from the format (src/em_steerable_sampler.hxx:1659-1745, 1796-1960) and pin the vertex weights
the library builds on the device (luminance of the map's bilinear lookup times the 9 SH basis
values of the vertex direction) against the reference's; the GPU tests write and read files
through the C ABI. The library's own adaptive triangulation (the reference's refinement rule,
restated on the host) reproduces the reference's adaptive file leaf for leaf; the reference's
adaptive file loads and renders what the reference's render of the same scene shows."""
import ctypes
import os
import struct

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import _lib, scene as S

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = b"Environment Map Steerable Sampler Data, format ver. 2.1\n\0"


def _fixture():
    return np.load(os.path.join(HERE, "golden", "emssd_ref.npz"))


def parse(b):
    """Reads a format-2.1 file: parameters, vertex directions and weights, leaves (level, 3
    vertex indices) in file order, and the number of set nodes."""
    assert b[:len(HEADER)] == HEADER
    o = len(HEADER)
    params = struct.unpack_from("<fIIIffI", b, o)
    o += 28
    nv, = struct.unpack_from("<I", b, o)
    o += 4
    v = np.frombuffer(b, np.float32, nv * 12, o).reshape(nv, 12)
    o += 48 * nv
    nsets, ntris = struct.unpack_from("<II", b, o)
    o += 8
    leaves, sets = [], 0
    stack = [1]                      # children still to read at each open set node
    while stack:
        if stack[-1] == 0:
            stack.pop()
            continue
        stack[-1] -= 1
        is_tri, = struct.unpack_from("<I", b, o)
        o += 4
        if is_tri:
            leaves.append(struct.unpack_from("<IIII", b, o))
            o += 16
        else:
            n, = struct.unpack_from("<I", b, o)
            o += 4
            assert 1 <= n <= params[6]
            sets += 1
            stack.append(n)
    assert o == len(b), "trailing bytes"
    assert (sets, len(leaves)) == (nsets, ntris)
    return dict(params=params, dirs=v[:, :3].astype(np.float64), weights=v[:, 3:].astype(np.float64),
                leaves=np.array(leaves, np.int64), sets=sets)


def sh9(d):
    """The 9 real SH basis values the reference's vertex weights use (SteerableBasisValue::
    GenerateSphHarm, src/em_steerable_sampler.hxx:122-144)."""
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    return np.stack([np.full_like(x, 0.282095), 0.488603 * y, 0.488603 * z, 0.488603 * x,
                     1.092548 * x * y, 1.092548 * y * z, 0.315392 * (3 * z * z - 1), 1.092548 * x * z,
                     0.546274 * (x * x - y * y)], axis=1)


def bilinear_luminance(em, d):
    """Luminance of the map's bilinear lookup in directions d (the lat-long mapping and the tent
    filter of src/em_image.hxx:95-143, 269-302; texel centres at half-integers)."""
    H, W = em.shape[:2]
    lum = 0.212671 * em[..., 0] + 0.715160 * em[..., 1] + 0.072169 * em[..., 2]
    phi = -np.arctan2(d[:, 1], d[:, 0])
    theta = np.arccos(np.clip(d[:, 2], -1, 1))
    u = np.clip(0.5 + phi / (2 * np.pi), 0, 1)
    v = np.clip(theta / np.pi, 0, 1)
    xf, yf = u * W, v * H
    cx, cy = np.floor(xf + 0.5).astype(int), np.floor(yf + 0.5).astype(int)
    x0, y0 = cx - 1, cy - 1
    xl, yl = xf - (x0 + 0.5), yf - (y0 + 0.5)

    def tex(x, y):
        rx, ry = x.copy(), y.copy()
        over, under = y >= H, y < 0
        rx[over | under] += W // 2
        ry[over] = H - 1
        ry[under] = 0
        return lum[ry, np.mod(rx, W)]
    top = (1 - xl) * tex(x0, y0) + xl * tex(cx, y0)
    bot = (1 - xl) * tex(x0, cy) + xl * tex(cx, cy)
    return (1 - yl) * top + yl * bot


def by_direction(f):
    """Vertex weights keyed by the rounded direction (a vertex stored several times once)."""
    out = {}
    for d, w in zip(f["dirs"], f["weights"]):
        k = tuple(np.round(d, 5))
        if k in out:
            np.testing.assert_allclose(out[k], w, rtol=1e-6, atol=1e-9)
        out[k] = w
    return out


def leaf_set(f):
    """Leaf triangles as cyclically normalised triples of rounded vertex directions (orientation kept)."""
    out = set()
    for lv, a, b, c in f["leaves"]:
        tri = [tuple(np.round(f["dirs"][i], 5)) for i in (a, b, c)]
        k = min(range(3), key=lambda i: tri[i])
        out.add(tuple(tri[k:] + tri[:k]))
    return out


def test_reference_files_read_completely():
    z = _fixture()
    u = parse(z["uniform"].tobytes())
    assert u["params"][:4] == (5.0, 2, 2, 50) and u["params"][6] == 6
    assert np.float32(u["params"][4]) == np.float32(1.1) and np.float32(u["params"][5]) == np.float32(0.7)
    assert len(u["leaves"]) == 20 * 4 ** 2 and set(u["leaves"][:, 0]) == {2}
    assert len(by_direction(u)) == 10 * 4 ** 2 + 2          # 162 distinct directions, stored 312 times
    a = parse(z["adaptive"].tobytes())
    assert a["params"][1:3] == (1, 3) and len(set(a["leaves"][:, 0])) > 1


def test_file_name_is_the_reference_cache_path():
    z = _fixture()
    assert P.steerable_file_name("em.bin", 2) == str(z["uniform_name"])


def test_reference_vertex_weights_are_map_luminance_times_sh():
    # the formula of the library's device build (vertexWeightsKernel), on the reference's own file
    z = _fixture()
    u = parse(z["uniform"].tobytes())
    want = bilinear_luminance(z["env_map"].astype(np.float64), u["dirs"])[:, None] * sh9(u["dirs"])
    scale = np.abs(u["weights"]).max()
    np.testing.assert_allclose(u["weights"], want, rtol=1e-5, atol=1e-6 * scale)


def write_file(params, dirs, weights, leaves):
    """A format-2.1 file of the given leaves (level, 3 vertex indices) under a flat chain of
    6-child set nodes (the reader accepts any tree)."""
    out = bytearray(HEADER)
    out += struct.pack("<fIIIffI", *params)
    out += struct.pack("<I", len(dirs))
    for d, w in zip(dirs, weights):
        out += struct.pack("<12f", *np.concatenate([d, w]).astype(np.float32))
    nodes = [("leaf", tuple(l)) for l in leaves]
    sets = 0
    while len(nodes) > 1:
        nodes = [("set", nodes[i:i + 6]) for i in range(0, len(nodes), 6)]
        sets += len(nodes)
    out += struct.pack("<II", sets, len(leaves))

    def emit(n):
        nonlocal out
        if n[0] == "leaf":
            out += struct.pack("<IIIII", 1, *n[1])
        else:
            out += struct.pack("<II", 0, len(n[1]))
            for c in n[1]:
                emit(c)
    emit(nodes[0])
    return bytes(out)


def triangulate(em, lo, hi, err):
    """The library's adaptive triangulation (pg3gpu_steer_triangulate): levels, corners."""
    L = _lib.load()
    em = np.ascontiguousarray(em, np.float32)
    n = ctypes.c_uint32()
    _lib.check(L.pg3gpu_steer_triangulate(em.ctypes.data, em.shape[1], em.shape[0], lo, hi, err, ctypes.byref(n),
                                          None, None))
    lv = np.zeros(n.value, np.uint32)
    cr = np.zeros((n.value, 9), np.float32)
    _lib.check(L.pg3gpu_steer_triangulate(em.ctypes.data, em.shape[1], em.shape[0], lo, hi, err, ctypes.byref(n),
                                          lv.ctypes.data, cr.ctypes.data))
    return lv, cr


def test_adaptive_triangulation_is_the_references():
    # the reference's adaptive file (levels 1-3, error 0.05) and the library's build of the same
    # map and parameters: the same leaves, at the same levels, with bit-identical corners
    z = _fixture()
    ref = parse(z["adaptive"].tobytes())
    err, lo, hi = ref["params"][0], ref["params"][1], ref["params"][2]
    lv, cr = triangulate(z["env_map"], lo, hi, err)
    assert len(lv) == len(ref["leaves"])
    mine = {}
    for level, c in zip(lv, cr):
        tri = sorted(tuple(np.float32(x) for x in c[3 * j:3 * j + 3]) for j in range(3))
        mine[tuple(tri)] = int(level)
    for level, a, b, c in ref["leaves"]:
        tri = sorted(tuple(np.float32(x) for x in ref["dirs"][i]) for i in (a, b, c))
        assert mine.get(tuple(tri)) == level
    # leaves tile the sphere: planar areas sum to the subdivided icosahedron's below 4 pi
    assert sorted(set(lv.tolist())) == [1, 2, 3]


def test_adaptive_triangulation_parameters():
    sky = S.synthetic_sky(256, 128, seed=7)
    lv, _ = triangulate(sky, 4, 9, 5.0)                  # the reference's default build parameters
    assert lv.min() == 4 and lv.max() > 6                # refined around the suns only
    assert len(lv) < 20 * 4 ** 6
    lv2, _ = triangulate(sky, 3, 3, 5.0)                 # minimum = maximum: the uniform level
    assert len(lv2) == 20 * 4 ** 3 and set(lv2.tolist()) == {3}
    with pytest.raises(P.Pg3Error):
        triangulate(sky, 5, 4, 5.0)
    with pytest.raises(P.Pg3Error):
        triangulate(sky, 4, 13, 5.0)


def _ctx(env, sampler=None, level=2, seed=5, adaptive=None):
    # the reference's vertex weights are point samples of the map: the same build here
    sc = S.cornell_env(16, 16, 64, 32)
    sc.env_map = env
    kw = {}
    if adaptive:
        kw = dict(steer_max_subdiv_level=adaptive[0], steer_max_approx_error=adaptive[1])
    cfg = P.Config(scene=sc, max_path_length=6, em_sampler=sampler if sampler is not None else _lib.EM_STEERABLE,
                   steer_subdiv_level=level, steer_weights=_lib.STEER_WEIGHTS_POINT, **kw)
    return P.GpuPathTracer(cfg, seed=seed)


@pytest.mark.gpu
def test_saved_file_matches_the_reference(tmp_path):
    z = _fixture()
    ref = parse(z["uniform"].tobytes())
    p = str(tmp_path / "mine.emssd")
    with _ctx(z["env_map"]) as r:
        r.save_steerable(p)
    mine = parse(open(p, "rb").read())
    assert mine["params"] == ref["params"]
    assert len(mine["dirs"]) == 162 and mine["sets"] == ref["sets"]
    assert leaf_set(mine) == leaf_set(ref)               # the same triangles, the same orientation
    wm, wr = by_direction(mine), by_direction(ref)
    assert wm.keys() == wr.keys()
    scale = max(np.abs(w).max() for w in wr.values())
    for k in wr:
        np.testing.assert_allclose(wm[k], wr[k], rtol=1e-5, atol=1e-6 * scale)


@pytest.mark.gpu
def test_loading_the_reference_file(tmp_path):
    z = _fixture()
    src = str(tmp_path / str(z["uniform_name"]))
    open(src, "wb").write(z["uniform"].tobytes())
    out = str(tmp_path / "again.emssd")
    with _ctx(z["env_map"]) as built, _ctx(z["env_map"]) as loaded:
        loaded.load_steerable(src)
        loaded.save_steerable(out)
        for r in (built, loaded):
            r.RunIteration(P.renderer.kPathTracing, 0, 64)
        a, b = built.framebuffer()[0], loaded.framebuffer()[0]
    # the loaded weights are the file's, bit for bit
    wl, wr = by_direction(parse(open(out, "rb").read())), by_direction(parse(z["uniform"].tobytes()))
    for k in wr:
        assert np.array_equal(wl[k].astype(np.float32), wr[k].astype(np.float32))
    # and render what the weights built from the map render, up to the weights' last bits
    assert abs(a.sum() / b.sum() - 1) < 1e-3
    close = np.isclose(a, b, rtol=1e-3, atol=1e-4 * a.max())
    assert close.mean() > 0.99


@pytest.mark.gpu
def test_round_trip_is_byte_identical(tmp_path):
    z = _fixture()
    p1, p2 = str(tmp_path / "a.emssd"), str(tmp_path / "b.emssd")
    with _ctx(z["env_map"], level=3) as r1:
        r1.save_steerable(p1, max_approx_error=0.5)
    env2 = np.ascontiguousarray(z["env_map"][::-1])      # another map: the file's weights must win
    with _ctx(env2, level=3) as r2:
        r2.load_steerable(p1)
        r2.save_steerable(p2, max_approx_error=0.5)
    assert open(p1, "rb").read() == open(p2, "rb").read()
    assert parse(open(p1, "rb").read())["params"][:3] == (0.5, 3, 3)


@pytest.mark.gpu
def test_loading_the_reference_adaptive_file(tmp_path):
    # the reference's adaptive file replaces a uniform context's triangulation; the library's own
    # adaptive build of the same map and parameters renders the same image (same leaves, same
    # point-sampled weights), and saving writes the file's triangulation back
    z = _fixture()
    src = str(tmp_path / str(z["adaptive_name"]))
    open(src, "wb").write(z["adaptive"].tobytes())
    ref = parse(z["adaptive"].tobytes())
    out = str(tmp_path / "again.emssd")
    with _ctx(z["env_map"], level=1, adaptive=(3, 0.05)) as built, _ctx(z["env_map"]) as loaded:
        loaded.load_steerable(src)
        loaded.save_steerable(out)
        for r in (built, loaded):
            r.RunIteration(P.renderer.kPathTracing, 0, 256)
        a, b = built.framebuffer()[0], loaded.framebuffer()[0]
    again = parse(open(out, "rb").read())
    assert leaf_set(again) == leaf_set(ref)
    assert sorted(again["leaves"][:, 0].tolist()) == sorted(ref["leaves"][:, 0].tolist())
    assert again["params"][:3] == ref["params"][:3]
    wl, wr = by_direction(again), by_direction(ref)
    assert wl.keys() == wr.keys()
    for k in wr:
        assert np.array_equal(wl[k].astype(np.float32), wr[k].astype(np.float32))
    assert abs(a.sum() / b.sum() - 1) < 1e-3
    assert np.isclose(a, b, rtol=1e-3, atol=1e-4 * a.max()).mean() > 0.99


@pytest.mark.gpu
def test_loaded_adaptive_file_renders_the_reference_image():
    # the reference's adaptive sampler file of the environment-map box's 64x32 sky, loaded and
    # rendered at as many samples as the reference's golden of that scene (CDF sampler) holds
    import tempfile
    from _util import load_golden, scene_from_golden, z_ok, zscores
    z = _fixture()
    d, text, td = load_golden("cornell_env_32_cdf")
    scene = scene_from_golden(d)
    assert np.array_equal(scene.env_map, z["env_map"])
    cfg = P.Config(scene=scene, max_path_length=12, em_sampler=_lib.EM_STEERABLE, steer_subdiv_level=1,
                   steer_weights=_lib.STEER_WEIGHTS_POINT)
    spp = 65536
    with tempfile.TemporaryDirectory() as tmp, P.GpuPathTracer(cfg, seed=77) as r:
        src = os.path.join(tmp, str(z["adaptive_name"]))
        open(src, "wb").write(z["adaptive"].tobytes())
        r.load_steerable(src)
        r.RunIteration(P.renderer.kPathTracing, 0, spp)
        mean, var, n = r.framebuffer(with_variance=True)
    frac, zm, zs = z_ok(zscores(mean, var / spp, d["mean"], d["var_mean"]))
    assert frac >= 0.999 and abs(zm) < 0.25 and 0.7 < zs < 1.3, (frac, zm, zs)


@pytest.mark.gpu
def test_files_the_library_cannot_use_are_refused(tmp_path):
    z = _fixture()
    cut = str(tmp_path / "cut.emssd")
    open(cut, "wb").write(z["uniform"].tobytes()[:-7])
    # a triangulation with a hole (one leaf missing) and one with two overlapping leaves
    u = parse(z["uniform"].tobytes())
    hole = str(tmp_path / "hole.emssd")
    open(hole, "wb").write(write_file(u["params"], u["dirs"], u["weights"], u["leaves"][1:]))
    twice = str(tmp_path / "twice.emssd")
    open(twice, "wb").write(write_file(u["params"], u["dirs"], u["weights"],
                                       np.concatenate([u["leaves"], u["leaves"][:1]])))
    with _ctx(z["env_map"]) as r:
        for bad in (cut, hole, twice, str(tmp_path / "missing.emssd")):
            with pytest.raises(P.Pg3Error) as e:
                r.load_steerable(bad)
            assert e.value.status == _lib.ERR_INVALID_ARGUMENT, bad
        # the context still renders with its own triangulation
        r.RunIteration(P.renderer.kPathTracing, 0, 4)
        assert r.framebuffer()[0].sum() > 0
    with _ctx(z["env_map"], sampler=_lib.EM_CDF) as r:  # no steerable sampler
        with pytest.raises(P.Pg3Error) as e:
            r.save_steerable(str(tmp_path / "x.emssd"))
        assert e.value.status == _lib.ERR_INVALID_ARGUMENT
