"""Steerable-sampler data files (".emssd", format 2.1): pg3gpu_save_steerable and
pg3gpu_load_steerable against files the reference's own EnvironmentMapSteerableSampler wrote
(tests/golden/emssd_ref.npz, made by `tests/golden/make_golden.py emssd`) for the 64x32 sky of
the environment-map box: a uniform triangulation (minimum = maximum subdivision level 2) and an
adaptive one (levels 1-3). The CPU tests read the reference's files with a reader restated here
from the format (src/em_steerable_sampler.hxx:1659-1745, 1796-1960) and pin the vertex weights
the library builds on the device (luminance of the map's bilinear lookup times the 9 SH basis
values of the vertex direction) against the reference's; the GPU tests write and read files
through the C ABI."""
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


def _ctx(env, sampler=None, level=2, seed=5):
    # the reference's vertex weights are point samples of the map: the same build here
    sc = S.cornell_env(16, 16, 64, 32)
    sc.env_map = env
    cfg = P.Config(scene=sc, max_path_length=6, em_sampler=sampler if sampler is not None else _lib.EM_STEERABLE,
                   steer_subdiv_level=level, steer_weights=_lib.STEER_WEIGHTS_POINT)
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
def test_files_the_library_cannot_use_are_refused(tmp_path):
    z = _fixture()
    adaptive = str(tmp_path / "adaptive.emssd")
    open(adaptive, "wb").write(z["adaptive"].tobytes())
    cut = str(tmp_path / "cut.emssd")
    open(cut, "wb").write(z["uniform"].tobytes()[:-7])
    uniform = str(tmp_path / "uniform.emssd")
    open(uniform, "wb").write(z["uniform"].tobytes())
    with _ctx(z["env_map"]) as r:
        with pytest.raises(P.Pg3Error) as e:
            r.load_steerable(adaptive)
        assert e.value.status == _lib.ERR_UNSUPPORTED
        for bad in (cut, str(tmp_path / "missing.emssd")):
            with pytest.raises(P.Pg3Error) as e:
                r.load_steerable(bad)
            assert e.value.status == _lib.ERR_INVALID_ARGUMENT
    with _ctx(z["env_map"], level=3) as r:             # level 2 file, level 3 context
        with pytest.raises(P.Pg3Error) as e:
            r.load_steerable(uniform)
        assert e.value.status == _lib.ERR_UNSUPPORTED
    with _ctx(z["env_map"], sampler=_lib.EM_CDF) as r:  # no steerable sampler
        with pytest.raises(P.Pg3Error) as e:
            r.save_steerable(str(tmp_path / "x.emssd"))
        assert e.value.status == _lib.ERR_INVALID_ARGUMENT
