// Host-side build of the steerable sampler's geometry (see pg3_steerable.h).
#include "pg3_steerable.h"

#include <algorithm>
#include <array>
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

// Planar area (the leaf weight is area x mean vertex weight, src/em_steerable_sampler.hxx:1277-1296),
// plane (unit normal, distance from the origin: the solid-angle Jacobian) and the three inward
// great-circle normals of every leaf in out.leafTri.
void leafTables(SteerGeom &out)
{
    const uint32_t nLeaf = (uint32_t)out.leafTri.size();
    out.leafArea.resize(nLeaf);
    out.leafPlane.resize(nLeaf);
    out.leafEdge.resize((size_t)nLeaf * 3);
    auto fdir = [&](int id) { return D3{out.vdir[id].x, out.vdir[id].y, out.vdir[id].z}; };
    for (uint32_t i = 0; i < nLeaf; ++i) {
        const int4 T = out.leafTri[i];
        const D3 a = fdir(T.x), b = fdir(T.y), c = fdir(T.z);
        const D3 cr = crs(sub(b, a), sub(c, a));
        out.leafArea[i] = (float)(0.5 * std::sqrt(dt(cr, cr)));
        const D3 nT = nrm(cr);
        out.leafPlane[i] = make_float4((float)nT.x, (float)nT.y, (float)nT.z, (float)dt(nT, a));
        const D3 e[3] = {nrm(crs(a, b)), nrm(crs(b, c)), nrm(crs(c, a))};
        for (int k = 0; k < 3; ++k)
            out.leafEdge[3 * (size_t)i + k] = make_float4((float)e[k].x, (float)e[k].y, (float)e[k].z, 0.f);
    }
}

// 6-ary tree topology, bottom-up over consecutive leaves (src/em_steerable_sampler.hxx:3755-3793)
void buildTree(SteerGeom &out)
{
    const uint32_t nLeaf = out.numLeaves();
    out.nodeChild.clear();
    out.layerStart.clear();
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
}

// Face locator: for every cell of a cube map over the sphere, the level-0 faces (out.tri[0..19])
// that touch the cell (found by dense sampling of the cell enlarged by a margin).
bool buildFaceLocator(SteerGeom &out, std::string &err)
{
    auto fdir = [&](int id) { return D3{out.vdir[id].x, out.vdir[id].y, out.vdir[id].z}; };
    const int G = kSteerCells;
    out.faceCells.assign(2 * 6 * G * G, make_int4(-1, -1, -1, -1));
    D3 edgeN[20][3];
    for (int fi = 0; fi < 20; ++fi) {
        const int4 tf = out.tri[fi];
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

// Corners of cell (iu, iv) of face f of a cube map with G x G cells per face (the device's
// cubeFace / cubeCell mapping: face f has axis f / 2 and sign -1 for odd f, u and v on the next
// two axes).
void cubeCellCorners(int f, uint32_t iu, uint32_t iv, uint32_t G, D3 q[4])
{
    const int ax = f / 2, bx = (ax + 1) % 3, cx = (ax + 2) % 3;
    const double sg = (f & 1) ? -1.0 : 1.0;
    auto dirOf = [&](double u, double v) {
        double p[3];
        p[ax] = sg; p[bx] = u; p[cx] = v;
        return nrm({p[0], p[1], p[2]});
    };
    const double u0 = -1.0 + 2.0 * iu / G, u1 = -1.0 + 2.0 * (iu + 1) / G;
    const double v0 = -1.0 + 2.0 * iv / G, v1 = -1.0 + 2.0 * (iv + 1) / G;
    q[0] = dirOf(u0, v0);
    q[1] = dirOf(u1, v0);
    q[2] = dirOf(u0, v1);
    q[3] = dirOf(u1, v1);
}

// A convex spherical polygon lies in a spherical triangle (great-circle edges) when its corners do.
// Each corner must lie at least kStartMargin (radians) inside every edge (unit inward normals),
// which covers the float rounding of the device's cell index and of its edge and child tests.
constexpr double kStartMargin = 1e-5;
bool cornersInside(const D3 q[4], const D3 e[3])
{
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k)
            if (dt(q[i], e[k]) < kStartMargin) return false;
    return true;
}

// Start cells of a uniform level (kSteerUniformStartGrid^2 cells per face; none when 0): ~leaf
// where one leaf contains the whole cell, INT32_MIN elsewhere (the leaf-locator lists serve). A
// leaf that contains the cell contains its centre, so it is among the leaf-locator candidates of
// the centre's cell.
void buildUniformStartCells(SteerGeom &out)
{
    const uint32_t G = kSteerUniformStartGrid;
    out.startCells.clear();
    if (G == 0) return;
    const uint32_t nLeaf = out.numLeaves(), LG = out.leafGrid;
    out.startCells.assign((size_t)6 * G * G, INT_MIN);
    parallelFor(6 * G, [&](uint32_t row) {
        const int f = (int)(row / G);
        const uint32_t iv = row % G;
        for (uint32_t iu = 0; iu < G; ++iu) {
            D3 q[4];
            cubeCellCorners(f, iu, iv, G, q);
            // the centre's cell of the leaf locator (same face, same position on it)
            const uint32_t lu = (uint32_t)(((double)iu + 0.5) * LG / G), lv = (uint32_t)(((double)iv + 0.5) * LG / G);
            const uint4 cell = out.leafCells[((size_t)f * LG + lv) * LG + lu];
            if (cell.x == 0xfffefffeu) continue;   // more than 8 candidates: the face locator serves
            const uint32_t words[4] = {cell.x, cell.y, cell.z, cell.w};
            for (uint32_t k = 0; k < 8; ++k) {
                const uint32_t id = (words[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
                if (id == kSteerLeafNone || id >= nLeaf) break;
                D3 e[3];
                for (int j = 0; j < 3; ++j) {
                    const float4 E = out.leafEdge[3 * (size_t)id + j];
                    e[j] = D3{E.x, E.y, E.z};
                }
                if (cornersInside(q, e)) {
                    out.startCells[((size_t)f * G + iv) * G + iu] = ~(int)id;
                    break;
                }
            }
        }
    });
}

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

    out.leafTri.resize(cur.size());
    for (size_t i = 0; i < cur.size(); ++i) out.leafTri[i] = make_int4(cur[i].x, cur[i].y, cur[i].z, (int)level);
    out.minLevel = out.maxLevel = level;
    leafTables(out);
    buildTree(out);
    auto fdir = [&](int id) { return D3{out.vdir[id].x, out.vdir[id].y, out.vdir[id].z}; };

    // leaf locator: for every cell of a finer cube map the leaves whose bounding cap meets the
    // cell's bounding cap, found down the subdivision hierarchy (a triangle's children are
    // visited when its own cap meets the cell's: a leaf is kept only if the caps of all its
    // ancestors meet the cell's too, which every leaf that touches the cell satisfies); cells
    // with more than 8 keep the face locator. Caps meet when the angle between their centres is
    // at most the sum of their radii (plus a margin), i.e. when the cosine of that angle is at
    // least cos(r_triangle + r_cell).
    const size_t nTri = out.tri.size();
    std::vector<D3> capC(nTri);
    std::vector<double> capCos(nTri), capSin(nTri);
    for (size_t i = 0; i < nTri; ++i) {
        const int4 T = out.tri[i];
        const D3 a = fdir(T.x), b = fdir(T.y), c = fdir(T.z);
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
        std::vector<uint32_t> set, next;   // local indices within the current level
        for (uint32_t iu = 0; iu < LG; ++iu) {
            const double u0 = -1.0 + 2.0 * iu / LG, u1 = -1.0 + 2.0 * (iu + 1) / LG;
            const double v0 = -1.0 + 2.0 * iv / LG, v1 = -1.0 + 2.0 * (iv + 1) / LG;
            const D3 cc = dirOf(0.5 * (u0 + u1), 0.5 * (v0 + v1));
            double rc = 0.0;
            for (const D3 &q : {dirOf(u0, v0), dirOf(u1, v0), dirOf(u0, v1), dirOf(u1, v1)})
                rc = std::fmax(rc, std::acos(std::fmin(1.0, dt(cc, q))));
            rc += 1e-4;
            const double cCos = std::cos(rc), cSin = std::sin(rc);
            // cos(r_triangle + r_cell); both radii are far below pi/2 at every level
            auto meets = [&](size_t t) { return dt(cc, capC[t]) >= capCos[t] * cCos - capSin[t] * cSin; };
            set.clear();
            for (uint32_t t = 0; t < 20; ++t)
                if (meets(t)) set.push_back(t);
            for (uint32_t l = 0; l < level; ++l) {
                next.clear();
                for (uint32_t t : set)
                    for (uint32_t k = 0; k < 4; ++k)
                        if (meets(out.levelOffset[l + 1] + 4 * t + k)) next.push_back(4 * t + k);
                set.swap(next);
            }
            uint32_t ids[8];
            int n = 0;
            bool many = false;
            for (uint32_t i : set) {   // ascending leaf ids
                // (leaf ids from 0xfffe on do not fit the 16-bit lists: the face locator serves)
                if (n == 8 || i >= kSteerLeafMany) { many = true; break; }
                ids[n++] = i;
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

    if (!buildFaceLocator(out, err)) return false;
    buildUniformStartCells(out);
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


// ------------------------------------------------------------------------------------------
// Adaptive triangulation (the reference's TriangulateEm, src/em_steerable_sampler.hxx:2963-3472).
// The refinement rule is restated in float arithmetic in the reference's order of operations, so
// that the decisions near the error threshold come out as the reference's own build takes them.
// Every triangle's decision depends only on its own vertices and the map, so the build runs level
// by level over all candidate triangles in parallel (the reference's depth-first order gives the
// same set of leaves); edge midpoints are shared between the two triangles of an edge.
// ------------------------------------------------------------------------------------------
namespace {

struct F3 {
    float x, y, z;
};
F3 f3add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
F3 f3sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 f3mul(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
F3 f3div(F3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
float f3dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 f3cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
F3 f3normalize(F3 a) { return f3div(a, std::sqrt(f3dot(a, a))); }
// ((a + b) / 2).Normalize(): the reference's edge midpoint on the sphere (:3434-3436)
F3 f3mid(F3 a, F3 b) { return f3normalize(f3div(f3add(a, b), 2.f)); }

constexpr float kPiF = 3.14159265358979f;
constexpr float kPiDiv2F = 1.5707963f;

struct EmMap {
    const float *rgb;
    uint32_t W, H;
    // texel (x, y) after the reference's wrapping (NormalizeImgCoords, src/em_image.hxx:245-276)
    const float *at(int x, int y) const
    {
        int rx = x, ry = y;
        if (y >= (int)H) { rx = x + (int)W / 2; ry = (int)H - 1; }
        else if (y < 0) { rx = x + (int)W / 2; ry = 0; }
        int m = rx % (int)W;
        if (m < 0) m += (int)W;
        return rgb + 3 * ((size_t)ry * W + (size_t)m);
    }
    float lum(F3 d) const { return emLuminanceDir(rgb, W, H, d.x, d.y, d.z); }
};

struct AdaptiveParams {
    uint32_t minLevel, maxLevel;
    float maxError;
    uint32_t maxSamplesPerDim = 50;   // the reference's debugging defaults (:26-98)
    float oversampling = 0.7f;
    float maxSpan = 1.1f;
};

float sinOf(F3 d) { return std::sqrt(1.f - d.z * d.z); }

// The whole triangle being tested: its vertex directions and their map luminance.
struct WholeTri {
    F3 v[3];
    float L[3];
};

// Geom::Triangle::BarycentricCoords (src/geom.hxx:634-675)
void baryCoords(F3 p, F3 a, F3 b, F3 c, float &bx, float &by)
{
    const F3 N = f3cross(f3sub(b, a), f3sub(c, a));
    const float denom = f3dot(N, N);
    bx = f3dot(N, f3cross(f3sub(c, b), f3sub(p, b))) / denom;
    by = f3dot(N, f3cross(f3sub(a, c), f3sub(p, c))) / denom;
}

// IsEstimationErrorTooLarge (:3216-3268): test samples on a grid of the planar sub-triangle
// (s0, s1, s2), compared with the whole triangle's linear approximation.
bool errorTooLarge(const WholeTri &T, F3 s0, F3 s1, F3 s2, uint32_t n, const EmMap &em, const AdaptiveParams &P)
{
    const float bin = 1.f / (float)n;
    for (uint32_t i = 0; i <= n; ++i)
        for (uint32_t j = 0; j <= n; ++j) {
            const float ix = (float)i * bin;
            const float sx = ix * ix, sy = (float)j * bin;
            // Sampling::SampleUniformTriangle via Triangle::MapCartToBary (src/geom.hxx:820-833)
            const float xs = std::sqrt(sx);
            const float b0 = 1.f - xs, b1 = sy * xs, b2 = 1.f - b0 - b1;
            const F3 p = f3add(f3add(f3mul(s0, b0), f3mul(s1, b1)), f3mul(s2, b2));
            float wx, wy;
            baryCoords(p, T.v[0], T.v[1], T.v[2], wx, wy);
            wx = std::min(std::max(wx, 0.f), 1.f);
            wy = std::min(std::max(wy, 0.f), 1.f);
            const float wz = std::min(std::max(1.f - wx - wy, 0.f), 1.f);
            const float approx = wx * T.L[0] + wy * T.L[1] + wz * T.L[2];
            const float emVal = em.lum(f3normalize(p));
            const float mn = std::min(emVal, approx), mx = std::max(emVal, approx);
            const float numEps = 0.0001f;
            if ((mx + numEps) > ((mn + numEps) * (1.f + P.maxError))) return true;
        }
    return false;
}

// TriangleHasToBeSubdividedImpl (:3271-3388), for the sub-triangle (a, b, c) of T.
bool subdivImpl(F3 a, float sa, F3 b, float sb, F3 c, float sc, const WholeTri &T, const EmMap &em,
                const AdaptiveParams &P)
{
    if (em.H == 0 || em.W == 0) return false;
    const F3 centroid = f3div(f3add(f3add(a, b), c), 3.f);
    const F3 e01 = f3normalize(f3div(f3add(a, b), 2.f));
    const F3 e12 = f3normalize(f3div(f3add(b, c), 2.f));
    const F3 e20 = f3normalize(f3div(f3add(c, a), 2.f));
    const F3 cdir = f3normalize(centroid);
    const float s01 = sinOf(e01), s12 = sinOf(e12), s20 = sinOf(e20), sc0 = sinOf(cdir);
    const float minSin = std::min({sa, sb, sc, s01, s12, s20, sc0});
    const float maxSin = std::max({sa, sb, sc, s01, s12, s20, sc0});
    const float polePixelMidTheta = 0.5f * kPiDiv2F / (float)em.H;
    const float polePixelSin = std::sin(polePixelMidTheta);
    const float minSinC = std::max(minSin, polePixelSin), maxSinC = std::max(maxSin, polePixelSin);

    // SubdivTestSamplesPerDim (:3168-3213): x components use the minimal sine, y the maximal
    const float k2PiF = 2.f * kPiF;
    const float minPixX = kPiF / (float)em.H, minPixY = minSinC * k2PiF / (float)em.W;
    const float maxPixX = kPiF / (float)em.H, maxPixY = maxSinC * k2PiF / (float)em.W;
    const float lowX = std::min(minPixX, minPixY), lowY = std::min(maxPixX, maxPixY);
    const float angX = std::min(lowX / 2.f, kPiDiv2F - 0.1f), angY = std::min(lowY / 2.f, kPiDiv2F - 0.1f);
    const float dist = std::sqrt(f3dot(centroid, centroid));
    const float planX = std::tan(angX) * dist, planY = std::tan(angY) * dist;
    const F3 d01 = f3sub(a, b), d12 = f3sub(b, c), d20 = f3sub(c, a);
    const float avgEdgeSqr = (f3dot(d01, d01) + f3dot(d12, d12) + f3dot(d20, d20)) / 3.f;
    const float binX = planX * planX / 2.f, binY = planY * planY / 2.f;
    const float spdX = std::sqrt(avgEdgeSqr / binX / 2.f) * P.oversampling;
    const float spdY = std::sqrt(avgEdgeSqr / binY / 2.f) * P.oversampling;
    const float maxSpdF = spdX, minSpdF = spdY;
    const uint32_t maxSpd = (uint32_t)std::ceil(maxSpdF);
    if (P.maxSamplesPerDim != 0 && P.maxSamplesPerDim < maxSpd) return true;
    const float span = maxSpdF / minSpdF;
    if (span >= P.maxSpan && maxSpdF > 32.f) {
        if (subdivImpl(a, sa, e01, s01, e20, s20, T, em, P)) return true;
        if (subdivImpl(b, sb, e12, s12, e01, s01, T, em, P)) return true;
        if (subdivImpl(c, sc, e20, s20, e12, s12, T, em, P)) return true;
        if (subdivImpl(e01, s01, e12, s12, e20, s20, T, em, P)) return true;
        return false;
    }
    return errorTooLarge(T, a, b, c, maxSpd, em, P);
}

// TriangleHasToBeSubdivided (:3391-3420)
bool needsSubdivision(const WholeTri &T, uint32_t level, const EmMap &em, const AdaptiveParams &P)
{
    if (level < P.minLevel) return true;
    if (level >= P.maxLevel) return false;
    return subdivImpl(T.v[0], sinOf(T.v[0]), T.v[1], sinOf(T.v[1]), T.v[2], sinOf(T.v[2]), T, em, P);
}

// The 12 icosahedron vertices in float as the reference computes them (Geom::UnitIcosahedron,
// src/geom.hxx:291-313), in the index order of the uniform build's level 0.
std::vector<F3> icosahedronFloat(const SteerGeom &g0)
{
    const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
    const float s = std::sqrt(1.0f + t * t);
    const float sInv = 1.0f / s;
    auto comp = [&](float c) {
        const float a = std::fabs(c);
        const float m = a > 0.7f ? t * sInv : (a > 0.3f ? 1.f * sInv : 0.f);
        return c < 0.f ? -m : m;
    };
    std::vector<F3> v(12);
    for (int i = 0; i < 12; ++i) v[i] = {comp(g0.vdir[i].x), comp(g0.vdir[i].y), comp(g0.vdir[i].z)};
    return v;
}

// The hierarchy of an adaptive triangulation during its construction.
struct Hier {
    std::vector<F3> V;                          // vertex directions
    std::vector<std::array<int, 3>> tri;        // triangle corners
    std::vector<int> level;
    std::vector<int> firstChild;                // -1 leaf, else the first of 4 consecutive children
    std::vector<std::array<int, 3>> mids;       // edge midpoints (ab, bc, ca) of subdivided triangles
    std::map<std::pair<int, int>, int> edgeMid;

    int midpoint(int a, int b)
    {
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        auto it = edgeMid.find(key);
        if (it != edgeMid.end()) return it->second;
        V.push_back(f3mid(V[a], V[b]));
        const int id = (int)V.size() - 1;
        edgeMid[key] = id;
        return id;
    }
    // children (A,ab,ca), (ab,B,bc), (ca,bc,C), (ab,bc,ca): the uniform build's order
    void subdivide(int t)
    {
        const std::array<int, 3> T = tri[t];
        const int ab = midpoint(T[0], T[1]), bc = midpoint(T[1], T[2]), ca = midpoint(T[2], T[0]);
        firstChild[t] = (int)tri.size();
        mids[t] = {ab, bc, ca};
        const std::array<int, 3> ch[4] = {{T[0], ab, ca}, {ab, T[1], bc}, {ca, bc, T[2]}, {ab, bc, ca}};
        for (const auto &c : ch) {
            tri.push_back(c);
            level.push_back(level[t] + 1);
            firstChild.push_back(-1);
            mids.push_back({-1, -1, -1});
        }
    }
    void init(const SteerGeom &g0)
    {
        V = icosahedronFloat(g0);
        for (int f = 0; f < 20; ++f) {
            tri.push_back({g0.tri[f].x, g0.tri[f].y, g0.tri[f].z});
            level.push_back(0);
            firstChild.push_back(-1);
            mids.push_back({-1, -1, -1});
        }
    }
};

// Start cells of an adaptive triangulation: for every cell of a cube map (kSteerStartGrid^2 cells
// per face), the deepest triangle of the hierarchy that contains the whole cell (cornersInside),
// so that the device's point location starts there instead of at the level-0 face. A cell whose
// corners no single face contains keeps INT_MIN.
void buildStartCells(const Hier &h, const std::vector<int> &code, SteerGeom &g)
{
    const size_t nt = h.tri.size();
    auto dir = [&](int v) { return D3{h.V[(size_t)v].x, h.V[(size_t)v].y, h.V[(size_t)v].z}; };
    std::vector<std::array<D3, 3>> edge(nt);   // unit inward normals of every triangle's edges
    for (size_t t = 0; t < nt; ++t) {
        const D3 a = dir(h.tri[t][0]), b = dir(h.tri[t][1]), c = dir(h.tri[t][2]);
        edge[t] = {nrm(crs(a, b)), nrm(crs(b, c)), nrm(crs(c, a))};
    }
    const uint32_t G = kSteerStartGrid;
    g.startCells.assign((size_t)6 * G * G, INT_MIN);
    parallelFor(6 * G, [&](uint32_t row) {
        const int f = (int)(row / G);
        const uint32_t iv = row % G;
        for (uint32_t iu = 0; iu < G; ++iu) {
            D3 q[4];
            cubeCellCorners(f, iu, iv, G, q);
            auto holds = [&](size_t t) { return cornersInside(q, edge[t].data()); };
            int t = -1;
            for (int fi = 0; fi < 20 && t < 0; ++fi)
                if (holds((size_t)fi)) t = fi;
            if (t < 0) continue;
            for (bool deeper = true; deeper && h.firstChild[(size_t)t] >= 0;) {
                deeper = false;
                const int c0 = h.firstChild[(size_t)t];
                for (int k = 0; k < 4; ++k)
                    if (holds((size_t)(c0 + k))) {
                        t = c0 + k;
                        deeper = true;
                        break;
                    }
            }
            g.startCells[((size_t)f * G + iv) * G + iu] = code[(size_t)t];
        }
    });
}

// Leaves in depth-first order (face 0's subtree first, children in order), the quadtree codes and
// the common tables.
std::shared_ptr<SteerGeom> finishAdaptive(const Hier &h, const SteerGeom &g0, uint32_t minLevel, uint32_t maxLevel,
                                          float maxError, std::string &err)
{
    auto g = std::make_shared<SteerGeom>();
    g->adaptive = true;
    g->minLevel = minLevel;
    g->maxLevel = maxLevel;
    g->maxApproxError = maxError;
    g->vdir.resize(h.V.size());
    for (size_t i = 0; i < h.V.size(); ++i) {
        const int none = -1;
        float w;
        std::memcpy(&w, &none, sizeof w);   // no antipodal vertex: adaptive triangulations are not symmetric
        g->vdir[i] = make_float4(h.V[i].x, h.V[i].y, h.V[i].z, w);
    }
    g->tri.assign(g0.tri.begin(), g0.tri.begin() + 20);
    g->levelOffset = {0u, 20u};
    // depth-first numbering of leaves and of subdivided triangles
    std::vector<int> code(h.tri.size(), INT_MIN);
    std::vector<int> order;   // subdivided triangles in quadtree-node order
    uint32_t maxLeafLevel = 0;
    std::vector<int> stack;
    for (int f = 19; f >= 0; --f) stack.push_back(f);
    while (!stack.empty()) {
        const int t = stack.back();
        stack.pop_back();
        if (h.firstChild[t] < 0) {
            code[t] = ~(int)g->leafTri.size();
            g->leafTri.push_back(make_int4(h.tri[t][0], h.tri[t][1], h.tri[t][2], h.level[t]));
            maxLeafLevel = std::max(maxLeafLevel, (uint32_t)h.level[t]);
        } else {
            code[t] = (int)order.size();
            order.push_back(t);
            for (int c = 3; c >= 0; --c) stack.push_back(h.firstChild[t] + c);
        }
    }
    if (g->leafTri.size() > kSteerMaxAdaptiveLeaves) {
        err = "adaptive steerable triangulation: more than 2^22 leaves";
        return nullptr;
    }
    g->level = maxLeafLevel;
    g->qtree.assign(5 + 2 * order.size(), make_int4(0, 0, 0, 0));
    for (int f = 0; f < 20; ++f) (&g->qtree[f / 4].x)[f % 4] = code[f];
    for (size_t n = 0; n < order.size(); ++n) {
        const int t = order[n];
        const int c0 = h.firstChild[t];
        g->qtree[5 + 2 * n] = make_int4(h.mids[t][0], h.mids[t][1], h.mids[t][2], h.level[t]);
        g->qtree[5 + 2 * n + 1] = make_int4(code[c0], code[c0 + 1], code[c0 + 2], code[c0 + 3]);
    }
    leafTables(*g);
    buildTree(*g);
    g->leafGrid = 0;   // no leaf-locator cube map: the quadtree serves
    if (!buildFaceLocator(*g, err)) return nullptr;
    buildStartCells(h, code, *g);
    return g;
}

}  // namespace

float emLuminanceDir(const float *rgb, uint32_t W, uint32_t H, float dx, float dy, float dz)
{
    const EmMap em{rgb, W, H};
    // Dir2LatLong (src/geom.hxx:78-95)
    const float phi = -std::atan2(dy, dx);
    const float theta = std::acos(dz);
    const float kPiInvF = 1.f / kPiF;
    const float u = std::min(std::max(0.5f + phi * 0.5f * kPiInvF, 0.f), 1.f);
    const float v = std::min(std::max(theta * kPiInvF, 0.f), 1.f);
    // EnvironmentMapImage::Evaluate with the tent filter (src/em_image.hxx:95-143)
    const float xFull = u * (float)W, yFull = v * (float)H;
    const int cx = (int)(xFull + 0.5f), cy = (int)(yFull + 0.5f);
    const int x0 = cx - 1, y0 = cy - 1;
    const float xl = xFull - ((float)x0 + 0.5f), yl = yFull - ((float)y0 + 0.5f);
    const float *p00 = em.at(x0, y0), *p10 = em.at(cx, y0), *p01 = em.at(x0, cy), *p11 = em.at(cx, cy);
    float c[3];
    for (int k = 0; k < 3; ++k) {
        const float top = (1.f - xl) * p00[k] + xl * p10[k];
        const float bot = (1.f - xl) * p01[k] + xl * p11[k];
        c[k] = (1.f - yl) * top + yl * bot;
    }
    return 0.212671f * c[0] + 0.715160f * c[1] + 0.072169f * c[2];
}

std::shared_ptr<SteerGeom> steerAdaptiveGeometry(const float *rgb, uint32_t W, uint32_t H, uint32_t minLevel,
                                                 uint32_t maxLevel, float maxError, std::string &err)
{
    if (!rgb || W < 2 || H < 2) { err = "adaptive steerable triangulation needs an environment map"; return nullptr; }
    if (minLevel > maxLevel || maxLevel > kSteerMaxAdaptiveLevel) {
        err = "adaptive steerable triangulation: levels must satisfy min <= max <= " +
              std::to_string(kSteerMaxAdaptiveLevel);
        return nullptr;
    }
    if (!(maxError > 0.f) || !std::isfinite(maxError)) { err = "adaptive steerable triangulation: max error must be > 0"; return nullptr; }
    const SteerGeom *g0 = steerGeometry(0, err);
    if (!g0) return nullptr;
    const EmMap em{rgb, W, H};
    AdaptiveParams P;
    P.minLevel = minLevel;
    P.maxLevel = maxLevel;
    P.maxError = maxError;
    Hier h;
    h.init(*g0);
    std::vector<float> vlum;   // luminance of every vertex (point samples, :3084-3095)
    auto lumOf = [&](int v) {
        while (vlum.size() < h.V.size()) vlum.push_back(em.lum(h.V[vlum.size()]));
        return vlum[(size_t)v];
    };
    std::vector<int> frontier(20);
    for (int f = 0; f < 20; ++f) frontier[f] = f;
    size_t leaves = 0;
    while (!frontier.empty()) {
        std::vector<WholeTri> T(frontier.size());
        for (size_t i = 0; i < frontier.size(); ++i)
            for (int k = 0; k < 3; ++k) {
                const int v = h.tri[frontier[i]][k];
                T[i].v[k] = h.V[v];
                T[i].L[k] = lumOf(v);
            }
        std::vector<char> split(frontier.size());
        parallelFor((uint32_t)frontier.size(), [&](uint32_t i) {
            split[i] = needsSubdivision(T[i], (uint32_t)h.level[frontier[i]], em, P) ? 1 : 0;
        });
        std::vector<int> next;
        for (size_t i = 0; i < frontier.size(); ++i) {
            if (!split[i]) {
                ++leaves;
                continue;
            }
            h.subdivide(frontier[i]);
            for (int c = 0; c < 4; ++c) next.push_back(h.firstChild[frontier[i]] + c);
        }
        if (leaves + next.size() > kSteerMaxAdaptiveLeaves) {
            err = "adaptive steerable triangulation: more than 2^22 leaves (raise the error or lower the maximum level)";
            return nullptr;
        }
        frontier.swap(next);
    }
    return finishAdaptive(h, *g0, minLevel, maxLevel, maxError, err);
}

std::shared_ptr<SteerGeom> steerGeometryFromLeaves(const std::vector<std::array<float, 9>> &corners,
                                                   const std::vector<uint32_t> &levels, uint32_t minLevel,
                                                   uint32_t maxLevel, float maxError, std::string &err)
{
    if (corners.size() != levels.size() || corners.empty()) { err = "no leaves"; return nullptr; }
    if (corners.size() > kSteerMaxAdaptiveLeaves) { err = "more than 2^22 leaves"; return nullptr; }
    const SteerGeom *g0 = steerGeometry(0, err);
    if (!g0) return nullptr;
    Hier h;
    h.init(*g0);
    std::vector<char> isLeaf(20, 0);
    auto close = [](F3 a, F3 b) { return std::fabs(a.x - b.x) + std::fabs(a.y - b.y) + std::fabs(a.z - b.z) < 1e-4f; };
    for (size_t i = 0; i < corners.size(); ++i) {
        const std::array<float, 9> &c = corners[i];
        const F3 a = {c[0], c[1], c[2]}, b = {c[3], c[4], c[5]}, cc = {c[6], c[7], c[8]};
        const F3 w = f3normalize(f3add(f3add(a, b), cc));
        if (levels[i] > kSteerMaxAdaptiveLevel) { err = "a leaf deeper than level " + std::to_string(kSteerMaxAdaptiveLevel); return nullptr; }
        // the level-0 face containing the leaf's centre
        int t = -1;
        float best = -1e30f;
        for (int f = 0; f < 20; ++f) {
            const F3 A = h.V[h.tri[f][0]], B = h.V[h.tri[f][1]], C = h.V[h.tri[f][2]];
            const float m = std::min({f3dot(w, f3cross(A, B)), f3dot(w, f3cross(B, C)), f3dot(w, f3cross(C, A))});
            if (m > best) { best = m; t = f; }
        }
        for (uint32_t l = 0; l < levels[i]; ++l) {
            if (isLeaf[(size_t)t]) { err = "two leaves overlap"; return nullptr; }
            if (h.firstChild[t] < 0) {
                h.subdivide(t);
                isLeaf.resize(h.tri.size(), 0);
            }
            const F3 ab = h.V[h.mids[t][0]], bc = h.V[h.mids[t][1]], ca = h.V[h.mids[t][2]];
            int child = 3;
            if (f3dot(w, f3cross(ab, ca)) >= 0.f) child = 0;
            else if (f3dot(w, f3cross(bc, ab)) >= 0.f) child = 1;
            else if (f3dot(w, f3cross(ca, bc)) >= 0.f) child = 2;
            t = h.firstChild[t] + child;
        }
        if (h.firstChild[t] >= 0 || isLeaf[(size_t)t]) { err = "two leaves overlap"; return nullptr; }
        // the leaf's corners must be the triangle's, in any order
        for (const F3 &q : {a, b, cc}) {
            bool hit = false;
            for (int k = 0; k < 3; ++k) hit |= close(q, h.V[h.tri[t][k]]);
            if (!hit) { err = "a leaf is not a triangle of the icosahedron's subdivision at its level"; return nullptr; }
        }
        isLeaf[(size_t)t] = 1;
    }
    for (size_t t = 0; t < h.tri.size(); ++t)
        if (h.firstChild[t] < 0 && !isLeaf[t]) { err = "the leaves do not cover the sphere"; return nullptr; }
    return finishAdaptive(h, *g0, minLevel, maxLevel, maxError, err);
}

}  // namespace pg3
