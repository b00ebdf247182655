// Host-side build of the steerable sampler's geometry (see pg3_steerable.h).
#include "pg3_steerable.h"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <map>
#include <memory>
#include <mutex>
#include <cstring>
#include <thread>
#include <tuple>
#include <utility>

namespace pg3 {

namespace {

struct D3 { double x, y, z; };
D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
D3 add(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
D3 crs(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dt(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
D3 nrm(D3 a) { const double l = std::sqrt(dt(a, a)); return {a.x / l, a.y / l, a.z / l}; }

// Runs body(i) for i in [0, n) on up to 16 host threads.
template <class F>
void parallelFor(uint32_t n, F body)
{
    const uint32_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const uint32_t nt = std::min(hw, std::max(1u, n / 16));
    if (nt <= 1) {
        for (uint32_t i = 0; i < n; ++i) body(i);
        return;
    }
    std::atomic<uint32_t> next(0);
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < nt; ++t)
        pool.emplace_back([&] {
            for (uint32_t i; (i = next.fetch_add(1)) < n;) body(i);
        });
    for (auto &th : pool) th.join();
}

}  // namespace


namespace {

bool buildGeometry(uint32_t level, SteerGeom &out, std::string &err)
{
    out = SteerGeom();
    out.level = level;

    // icosahedron: the 12 cyclic permutations of (+-t, +-1, 0), normalised -- the reference's
    // vertex set (Geom::UnitIcosahedron, src/geom.hxx:290-312), so both triangulate the sphere
    // with the same triangles at every level
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<D3> v;
    for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2) {
            v.push_back(nrm({s2 * t, (double)s1, 0.0}));
            v.push_back(nrm({(double)s1, 0.0, s2 * t}));
            v.push_back(nrm({0.0, s2 * t, (double)s1}));
        }
    double emin = 1e9;
    for (size_t i = 0; i < v.size(); ++i)
        for (size_t j = i + 1; j < v.size(); ++j) emin = std::fmin(emin, std::sqrt(dt(sub(v[i], v[j]), sub(v[i], v[j]))));
    auto adjacent = [&](size_t i, size_t j) { return std::sqrt(dt(sub(v[i], v[j]), sub(v[i], v[j]))) < emin * 1.001; };
    std::vector<int4> level0;
    for (size_t i = 0; i < v.size(); ++i)
        for (size_t j = i + 1; j < v.size(); ++j)
            for (size_t k = j + 1; k < v.size(); ++k)
                if (adjacent(i, j) && adjacent(j, k) && adjacent(i, k)) {
                    const D3 n = crs(sub(v[j], v[i]), sub(v[k], v[i]));
                    const bool ccw = dt(n, add(add(v[i], v[j]), v[k])) > 0;   // outward facing
                    level0.push_back(make_int4((int)i, ccw ? (int)j : (int)k, ccw ? (int)k : (int)j, 0));
                }
    if (level0.size() != 20) { err = "icosahedron construction failed"; return false; }

    // 4-way subdivision, children (A,ab,ca), (ab,B,bc), (ca,bc,C), (ab,bc,ca)
    std::map<std::pair<int, int>, int> mid;
    auto midpoint = [&](int a, int b) {
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        auto it = mid.find(key);
        if (it != mid.end()) return it->second;
        v.push_back(nrm(add(v[a], v[b])));
        const int id = (int)v.size() - 1;
        mid[key] = id;
        return id;
    };
    out.tri = level0;
    out.levelOffset.push_back(0);
    std::vector<int4> cur = level0;
    for (uint32_t l = 0; l < level; ++l) {
        std::vector<int4> next;
        next.reserve(cur.size() * 4);
        for (const int4 &T : cur) {
            const int ab = midpoint(T.x, T.y), bc = midpoint(T.y, T.z), ca = midpoint(T.z, T.x);
            next.push_back(make_int4(T.x, ab, ca, 0));
            next.push_back(make_int4(ab, T.y, bc, 0));
            next.push_back(make_int4(ca, bc, T.z, 0));
            next.push_back(make_int4(ab, bc, ca, 0));
        }
        out.levelOffset.push_back((uint32_t)out.tri.size());
        out.tri.insert(out.tri.end(), next.begin(), next.end());
        cur.swap(next);
    }
    out.levelOffset.push_back((uint32_t)out.tri.size());
    out.vdir.resize(v.size());
    for (size_t i = 0; i < v.size(); ++i) out.vdir[i] = make_float4((float)v[i].x, (float)v[i].y, (float)v[i].z, 0.f);
    // antipodal vertices: negation commutes with the midpoint normalisation, so -v is a vertex
    // with exactly the negated coordinates
    {
        std::map<std::tuple<float, float, float>, int> byDir;
        for (size_t i = 0; i < v.size(); ++i) byDir[std::make_tuple(out.vdir[i].x, out.vdir[i].y, out.vdir[i].z)] = (int)i;
        for (size_t i = 0; i < v.size(); ++i) {
            const auto it = byDir.find(std::make_tuple(-out.vdir[i].x, -out.vdir[i].y, -out.vdir[i].z));
            if (it == byDir.end()) { err = "steerable triangulation is not centrally symmetric"; return false; }
            int bits = it->second;
            float w;
            std::memcpy(&w, &bits, sizeof w);
            out.vdir[i].w = w;
        }
    }

    // leaves: planar area (the leaf weight is area x mean vertex weight,
    // src/em_steerable_sampler.hxx:1277-1296) and plane (unit normal, distance) for the
    // solid-angle Jacobian
    const uint32_t nLeaf = (uint32_t)cur.size();
    out.leafArea.resize(nLeaf);
    out.leafPlane.resize(nLeaf);
    auto fdir = [&](int id) { return D3{out.vdir[id].x, out.vdir[id].y, out.vdir[id].z}; };
    for (uint32_t i = 0; i < nLeaf; ++i) {
        const int4 T = cur[i];
        const D3 a = fdir(T.x), b = fdir(T.y), c = fdir(T.z);
        const D3 cr = crs(sub(b, a), sub(c, a));
        out.leafArea[i] = (float)(0.5 * std::sqrt(dt(cr, cr)));
        const D3 nT = nrm(cr);
        out.leafPlane[i] = make_float4((float)nT.x, (float)nT.y, (float)nT.z, (float)dt(nT, a));
    }

    // 6-ary tree topology, bottom-up over consecutive items (src/em_steerable_sampler.hxx:3755-3793)
    std::vector<int> layer(nLeaf);
    for (uint32_t i = 0; i < nLeaf; ++i) layer[i] = ~(int)i;
    do {
        out.layerStart.push_back((uint32_t)(out.nodeChild.size() / 8));
        std::vector<int> up;
        for (size_t s = 0; s < layer.size(); s += 6) {
            up.push_back((int)(out.nodeChild.size() / 8));
            for (size_t c = 0; c < 8; ++c)
                out.nodeChild.push_back(c < 6 && s + c < layer.size() ? layer[s + c] : INT_MIN);
        }
        layer.swap(up);
    } while (layer.size() > 1);
    out.layerStart.push_back((uint32_t)(out.nodeChild.size() / 8));
    out.root = layer[0];

    // leaf locator: inward edge normals of every leaf, and for every cell of a finer cube map
    // the leaves whose bounding cap meets the cell's bounding cap (a superset of the leaves
    // that touch the cell); cells with more than 8 keep the face locator. Caps meet when the
    // angle between their centres is at most the sum of their radii (plus a margin), i.e. when
    // the cosine of that angle is at least cos(rLeaf + rCell).
    out.leafEdge.resize((size_t)nLeaf * 3);
    std::vector<D3> capC(nLeaf);
    std::vector<double> capCos(nLeaf), capSin(nLeaf);
    for (uint32_t i = 0; i < nLeaf; ++i) {
        const int4 T = cur[i];
        const D3 a = fdir(T.x), b = fdir(T.y), c = fdir(T.z);
        const D3 e[3] = {nrm(crs(a, b)), nrm(crs(b, c)), nrm(crs(c, a))};
        for (int k = 0; k < 3; ++k)
            out.leafEdge[3 * (size_t)i + k] = make_float4((float)e[k].x, (float)e[k].y, (float)e[k].z, 0.f);
        capC[i] = nrm(add(add(a, b), c));
        const double r = std::acos(std::fmin(1.0, std::fmin(dt(capC[i], a), std::fmin(dt(capC[i], b), dt(capC[i], c)))));
        capCos[i] = std::cos(r);
        capSin[i] = std::sin(r);
    }
    const uint32_t LG = 4u << level;
    out.leafGrid = LG;
    out.leafCells.assign((size_t)6 * LG * LG, make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu));
    parallelFor(6 * LG, [&](uint32_t row) {
        const int f = (int)(row / LG);
        const uint32_t iv = row % LG;
        const int ax = f / 2, bx = (ax + 1) % 3, cx = (ax + 2) % 3;
        const double sg = (f & 1) ? -1.0 : 1.0;
        auto dirOf = [&](double u, double vv) {
            double p[3];
            p[ax] = sg; p[bx] = u; p[cx] = vv;
            return nrm({p[0], p[1], p[2]});
        };
        for (uint32_t iu = 0; iu < LG; ++iu) {
            const double u0 = -1.0 + 2.0 * iu / LG, u1 = -1.0 + 2.0 * (iu + 1) / LG;
            const double v0 = -1.0 + 2.0 * iv / LG, v1 = -1.0 + 2.0 * (iv + 1) / LG;
            const D3 cc = dirOf(0.5 * (u0 + u1), 0.5 * (v0 + v1));
            double rc = 0.0;
            for (const D3 &q : {dirOf(u0, v0), dirOf(u1, v0), dirOf(u0, v1), dirOf(u1, v1)})
                rc = std::fmax(rc, std::acos(std::fmin(1.0, dt(cc, q))));
            rc += 1e-4;
            const double cCos = std::cos(rc), cSin = std::sin(rc);
            uint32_t ids[8];
            int n = 0;
            bool many = false;
            for (uint32_t i = 0; i < nLeaf && !many; ++i) {
                // cos(rLeaf + rCell); both radii are far below pi/2 at every level
                const double lim = capCos[i] * cCos - capSin[i] * cSin;
                if (dt(cc, capC[i]) >= lim) {
                    // (leaf ids from 0xfffe on do not fit the 16-bit lists: the face locator serves)
                    if (n == 8 || i >= kSteerLeafMany) many = true;
                    else ids[n++] = i;
                }
            }
            uint4 &cell = out.leafCells[((size_t)f * LG + iv) * LG + iu];
            if (many) {
                cell = make_uint4(0xfffefffeu, 0xfffefffeu, 0xfffefffeu, 0xfffefffeu);
                continue;
            }
            uint32_t w[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
            for (int k = 0; k < n; ++k) {
                const uint32_t shift = (k & 1) ? 16u : 0u;
                w[k >> 1] = (w[k >> 1] & ~(0xffffu << shift)) | (ids[k] << shift);
            }
            cell = make_uint4(w[0], w[1], w[2], w[3]);
        }
    });

    // face locator: for every cell of a cube map over the sphere, the level-0 faces that
    // touch the cell (found by dense sampling of the cell enlarged by a margin)
    const int G = kSteerCells;
    out.faceCells.assign(2 * 6 * G * G, make_int4(-1, -1, -1, -1));
    D3 edgeN[20][3];
    for (int fi = 0; fi < 20; ++fi) {
        const int4 tf = level0[fi];
        const D3 A = fdir(tf.x), B = fdir(tf.y), C = fdir(tf.z);
        edgeN[fi][0] = crs(A, B);
        edgeN[fi][1] = crs(B, C);
        edgeN[fi][2] = crs(C, A);
    }
    std::atomic<bool> overflow(false);
    parallelFor(6 * G * G, [&](uint32_t cell) {
        const int f = (int)cell / (G * G), iv = ((int)cell / G) % G, iu = (int)cell % G;
        const int ax = f / 2, bx = (ax + 1) % 3, cx = (ax + 2) % 3;
        const double s = (f & 1) ? -1.0 : 1.0;
        int found[8], nf = 0;
        const int K = 24;
        for (int sv = 0; sv <= K; ++sv)
            for (int su = 0; su <= K; ++su) {
                const double u = -1.0 + 2.0 * (iu + (su / (double)K) * 1.1 - 0.05) / G;
                const double vv = -1.0 + 2.0 * (iv + (sv / (double)K) * 1.1 - 0.05) / G;
                double p[3];
                p[ax] = s; p[bx] = u; p[cx] = vv;
                const D3 w = nrm({p[0], p[1], p[2]});
                for (int fi = 0; fi < 20; ++fi) {
                    const double m = std::fmin(std::fmin(dt(w, edgeN[fi][0]), dt(w, edgeN[fi][1])), dt(w, edgeN[fi][2]));
                    if (m >= -1e-3) {
                        bool have = false;
                        for (int q = 0; q < nf; ++q) have |= (found[q] == fi);
                        if (!have) {
                            if (nf < 8) found[nf++] = fi;
                            else overflow = true;
                        }
                    }
                }
            }
        int4 &c0 = out.faceCells[2 * cell];
        int4 &c1 = out.faceCells[2 * cell + 1];
        c0.x = nf > 0 ? found[0] : -1;
        c0.y = nf > 1 ? found[1] : -1;
        c0.z = nf > 2 ? found[2] : -1;
        c0.w = nf > 3 ? found[3] : -1;
        c1.x = nf > 4 ? found[4] : -1;
        c1.y = nf > 5 ? found[5] : -1;
        c1.z = nf > 6 ? found[6] : -1;
        c1.w = nf > 7 ? found[7] : -1;
    });
    if (overflow) { err = "steerable face locator: more than 8 faces in a cube-map cell"; return false; }
    return true;
}

}  // namespace

const SteerGeom *steerGeometry(uint32_t level, std::string &err)
{
    if (level > 7) { err = "steerable subdivision level must be <= 7"; return nullptr; }
    static std::mutex mu;
    static std::unique_ptr<SteerGeom> cache[8];
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[level]) {
        std::unique_ptr<SteerGeom> g(new SteerGeom);
        if (!buildGeometry(level, *g, err)) return nullptr;
        cache[level] = std::move(g);
    }
    return cache[level].get();
}

}  // namespace pg3
