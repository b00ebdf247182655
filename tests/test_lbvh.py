"""The device LBVH is bit-identical to the CPU build of the same codes and order
(oracle/lbvh_oracle.cpp), and closest-hit / any-hit through it return the list
loop's answers (GPU tests); the CPU build's own invariants are checked on the CPU."""
import ctypes

import numpy as np
import pytest

import pg3render_gb300 as P
from pg3render_gb300 import scene as S

R = P.renderer


def _oracle_lbvh(tris, sph):
    import oracle as O
    L = O.lib()
    L.pg3o_lbvh.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int] + [ctypes.c_void_p] * 3
    n = len(tris) + len(sph)
    codes, ids = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
    nodes = np.zeros((n - 1, 16), np.float32)
    t = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    s = np.ascontiguousarray(sph, np.float32).reshape(-1, 4)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)   # noqa: E731
    assert L.pg3o_lbvh(p(t), len(t), p(s), len(s), p(codes), p(ids), p(nodes)) == 0
    return codes, ids, nodes


def _random_scene(ntri, nsph, seed, clustered=False):
    rng = np.random.default_rng(seed)
    s = S.Scene(S.Camera((0, -5, 0), (0, 1, 0), (0, 0, 1), 32, 32), name="soup")
    s.add_material(S.Material(S.MAT_LAMBERT, (0.5, 0.5, 0.5)))
    centres = rng.uniform(-1, 1, (ntri, 3))
    if clustered:   # many equal Morton codes
        centres = np.round(centres * 4) / 4
    for c in centres:
        d = rng.normal(size=(3, 3)) * 0.05
        s.add_triangle(c + d[0], c + d[1], c + d[2], 0)
    for c in rng.uniform(-1, 1, (nsph, 3)):
        s.spheres.append((tuple(c), float(rng.uniform(0.01, 0.1)), 0))
    s.background_const = (1.0, 1.0, 1.0)
    return s


def _tri_sph_arrays(s):
    tris = np.array([np.concatenate(t[:3]) for t in s.triangles], np.float32).reshape(-1, 9)
    sph = np.array([list(c) + [r] for c, r, m in s.spheres], np.float32).reshape(-1, 4)
    return tris, sph


def test_cpu_lbvh_invariants():
    s = _random_scene(500, 50, 1)
    tris, sph = _tri_sph_arrays(s)
    codes, ids, nodes = _oracle_lbvh(tris, sph)
    n = len(codes)
    assert np.all(np.diff(codes.astype(np.int64)) >= 0) and sorted(ids) == list(range(n))
    child = nodes[:, [3, 11]].view(np.int32)
    leaves = sorted(~c for c in child.ravel() if c < 0)
    inner = sorted(c for c in child.ravel() if c >= 0)
    assert leaves == list(range(n)) and inner == list(range(1, n - 1))   # a tree over all primitives
    # every child box lies inside its parent's box
    lo = np.minimum(nodes[:, 0:3], nodes[:, 8:11])
    hi = np.maximum(nodes[:, 4:7], nodes[:, 12:15])
    for v in range(n - 1):
        for side in (0, 1):
            c = child[v, side]
            if c >= 0:
                assert np.all(lo[c] >= lo[v]) and np.all(hi[c] <= hi[v])


@pytest.mark.gpu
@pytest.mark.parametrize("ntri,nsph,clustered", [(10, 2, False), (1000, 100, False), (20000, 0, True),
                                                 (100000, 5000, False)])
def test_device_lbvh_bit_exact(ntri, nsph, clustered):
    s = _random_scene(ntri, nsph, ntri, clustered)
    with P.GpuPathTracer(P.Config(scene=s, max_path_length=2, traversal=R.TRAVERSAL_BVH)) as r:
        gc, gi, gn = r.export_bvh()
    tris, sph = _tri_sph_arrays(s)
    oc, oi, on = _oracle_lbvh(tris, sph)
    assert np.array_equal(gc, oc)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gn.view(np.uint32), on.view(np.uint32))   # bitwise, boxes and child ids


@pytest.mark.gpu
def test_bvh_traversal_matches_list_on_soup():
    s = _random_scene(3000, 200, 7)
    outs = []
    for trav in (R.TRAVERSAL_LIST, R.TRAVERSAL_BVH):
        with P.GpuPathTracer(P.Config(scene=s, max_path_length=3, traversal=trav), seed=3) as r:
            outs.append(r.render_samples(R.kPathTracing, 0, 2))
            r.synchronize()
    assert np.array_equal(outs[0], outs[1])
