// Steerable environment-map sampling on the device (tables from pg3_steerable.cpp).
//
// Target density (solid angle), for a surface normal n with clamped-cosine SH
// coefficients c(n) (src/em_steerable_sampler.hxx:657-688, with the reference's
// +0.15 compensation that keeps the approximation positive everywhere):
//   base(w) = g_T(p) / Z(n) * r^3 / d_T
// where T is the leaf triangle containing w, p the point where w meets T's plane
// (distance d_T from the origin, r = |p|), g_T the linear interpolation over T of
// the vertex values (vertex weight . c), and Z(n) the sum of all leaf integrals.
// Sampling draws T from the 6-ary tree (src/em_steerable_sampler.hxx:3798-3875),
// then p with density proportional to g_T on the planar triangle, then w = p/|p|;
// its pdf is exactly base(w). Directions below the horizon are mirrored through
// the origin as in the reference (:2196-2208), so the returned pdf is
// base(w) + base(-w) for both sampled and evaluated directions. A uniform triangulation is
// centrally symmetric: -w lies in the leaf of the antipodal vertices at the same barycentric
// coordinates and the same r / d_T, so base(-w) needs only those vertices' values. An adaptive
// triangulation (leaves at several levels, the reference's default build) is not: there -w is
// located on its own, through the quadtree of its icosahedron face (the ADAPTIVE variants).
#pragma once

#include <climits>

#include "pg3_device.cuh"

namespace pg3 {

constexpr int kSteerCellsDev = 8;   // must equal kSteerCells of the host build
constexpr uint32_t kSteerMaxAdaptiveDepth = 12;   // must equal kSteerMaxAdaptiveLevel of the host build
#ifndef PG3_STEER_START_GRID
#define PG3_STEER_START_GRID 256
#endif
constexpr int kSteerStartGridDev = PG3_STEER_START_GRID;   // must equal kSteerStartGrid of the host build

#ifndef PG3_STEER_UNIFORM_START_GRID
#define PG3_STEER_UNIFORM_START_GRID 256
#endif
constexpr int kSteerUniformStartGridDev = PG3_STEER_UNIFORM_START_GRID;   // kSteerUniformStartGrid

PG3_DI void steerCoeffs(float3 n, float c[9])
{
    const float c1 = .429043f, c2 = .511644f, c3 = .743125f, c4 = .886227f, c5 = .247708f;
    c[0] = c4 + 0.15f;
    c[1] = 2.f * c2 * n.y;
    c[2] = 2.f * c2 * n.z;
    c[3] = 2.f * c2 * n.x;
    c[4] = 2.f * c1 * n.x * n.y;
    c[5] = 2.f * c1 * n.y * n.z;
    c[6] = c3 * n.z * n.z - c5;
    c[7] = 2.f * c1 * n.x * n.z;
    c[8] = c1 * (n.x * n.x - n.y * n.y);
}

// w: 9 weights padded to 12 floats, 16-byte aligned (three vector loads)
PG3_DI float dot9(const float *__restrict__ w, const float c[9])
{
    const float4 *w4 = reinterpret_cast<const float4 *>(w);
    const float4 a = __ldg(&w4[0]), b = __ldg(&w4[1]), d = __ldg(&w4[2]);
    float s = 0.f;
    s += a.x * c[0]; s += a.y * c[1]; s += a.z * c[2]; s += a.w * c[3];
    s += b.x * c[4]; s += b.y * c[5]; s += b.z * c[6]; s += b.w * c[7];
    s += d.x * c[8];
    return s;
}

// Tables that follow the leaf planes in one allocation (pg3gpu_create): per leaf 3 inward edge
// normals, the leaf-locator cube map (6 x grid^2 cells of up to 8 16-bit leaf ids; uniform
// levels only, grid 0 for adaptive triangulations), and the 9 weights of the whole sphere.
PG3_DI uint32_t steerLeaves(const SteerView &T) { return T.numLeaves; }
PG3_DI uint32_t steerGrid(const SteerView &T) { return T.leafGrid; }
PG3_DI const float4 *steerEdges(const SteerView &T) { return T.leafPlane + steerLeaves(T); }
PG3_DI const uint4 *steerCells(const SteerView &T)
{
    return reinterpret_cast<const uint4 *>(T.leafPlane + 4 * steerLeaves(T));
}
PG3_DI const float *steerRootW(const SteerView &T)
{
    const uint32_t g = steerGrid(T);
    return reinterpret_cast<const float *>(T.leafPlane + 4 * steerLeaves(T) + 6 * g * g);
}

// Whole-sphere integral Z(n): every node value is positive (the clamped-cosine approximation
// with its +0.15 term is), so the sum over the root's children is one dot product with the
// summed weights.
PG3_DI float steerTotal(const SteerView &T, const float c[9]) { return fmaxf(dot9(steerRootW(T), c), 0.f); }

PG3_DI float3 vdir(const SteerView &T, int v) { return xyz(__ldg(&T.vdir[v])); }

// A vertex's value is its weights (the map's luminance L times the 9 SH basis values Y(d) at its
// direction d) dotted with c: L (c . Y(d)). With c fixed by the normal, c . Y(d) is a quadratic
// form in d, set up once per normal, so a vertex costs its direction and luminance (both in the
// leaf's record) instead of 9 weights; the form's even part (quadratic terms and constant) is the
// same at -d and its odd part (linear terms) changes sign, which gives the antipodal vertex of a
// uniform level as well (its luminance is in the record too).
struct SteerQuad {
    float a, bx, by, bz, m8, mzz, mxy, myz, mxz;   // m8: of x^2 - y^2
};
PG3_DI SteerQuad steerQuad(const float c[9])
{
    // Y: 0.282095; 0.488603 (y, z, x); 1.092548 (xy, yz); 0.315392 (3z^2 - 1); 1.092548 xz;
    // 0.546274 (x^2 - y^2) -- the basis of the build (pg3_steer_build.cu)
    SteerQuad q;
    q.a = 0.282095f * c[0] - 0.315392f * c[6];
    q.by = 0.488603f * c[1];
    q.bz = 0.488603f * c[2];
    q.bx = 0.488603f * c[3];
    q.mxy = 1.092548f * c[4];
    q.myz = 1.092548f * c[5];
    q.mzz = 3.f * 0.315392f * c[6];
    q.mxz = 1.092548f * c[7];
    q.m8 = 0.546274f * c[8];
    return q;
}
// the values of a vertex at direction d with luminance L and of its antipode (luminance La)
PG3_DI float2 vvalPair(const SteerQuad &q, float3 d, float L, float La)
{
    const float even = q.a + d.x * (q.m8 * d.x + q.mxy * d.y + q.mxz * d.z) + d.y * (q.myz * d.z - q.m8 * d.y) +
                       d.z * (q.mzz * d.z);
    const float odd = q.bx * d.x + q.by * d.y + q.bz * d.z;
    return make_float2(L * fmaxf(even + odd, 0.f), La * fmaxf(even - odd, 0.f));
}

// A leaf's record (SteerView::leafRec): corners with their luminance, the antipodes' luminance
// (read only when ANTI), the plane.
template <bool ANTI>
struct SteerLeaf {
    float4 A, B, C, anti, plane;
};
template <bool ANTI>
PG3_DI SteerLeaf<ANTI> steerLeaf(const SteerView &T, int leaf)
{
    const float4 *r = T.leafRec + 5 * (size_t)leaf;
    SteerLeaf<ANTI> L;
    L.A = __ldg(&r[0]);
    L.B = __ldg(&r[1]);
    L.C = __ldg(&r[2]);
    L.anti = ANTI ? __ldg(&r[3]) : make_float4(0.f, 0.f, 0.f, 0.f);
    L.plane = __ldg(&r[4]);
    return L;
}

// base density of the point p of a leaf's plane at distance d from the origin (value g there).
PG3_DI float steerLeafPdf(float d, float3 p, float g, float Z)
{
    const float r = length(p);
    return (Z > 0.f) ? fmaxf(g, 0.f) / Z * (r * r * r / d) : 0.f;
}

PG3_DI float faceMinEdge(const SteerView &T, int f, float3 w)
{
    const int4 t = __ldg(&T.tri[f]);
    const float3 a = vdir(T, t.x), b = vdir(T, t.y), c = vdir(T, t.z);
    return fminf(fminf(dot(w, cross(a, b)), dot(w, cross(b, c))), dot(w, cross(c, a)));
}

// Cube-map coordinates of a direction: face 0..5 (+x, -x, +y, -y, +z, -z) and the position
// (u, v) in [-1, 1]^2 on it.
PG3_DI int cubeFace(float3 w, float &u, float &v)
{
    const float ax = fabsf(w.x), ay = fabsf(w.y), az = fabsf(w.z);
    int a;
    float wa, wb, wc;
    if (ax >= ay && ax >= az) { a = 0; wa = w.x; wb = w.y; wc = w.z; }
    else if (ay >= az) { a = 1; wa = w.y; wb = w.z; wc = w.x; }
    else { a = 2; wa = w.z; wb = w.x; wc = w.y; }
    const float inv = 1.f / fabsf(wa);
    u = wb * inv;
    v = wc * inv;
    return 2 * a + (wa < 0.f ? 1 : 0);
}
PG3_DI int cubeCell(int face, float u, float v, int G)
{
    const int iu = min(max((int)((u + 1.f) * (0.5f * G)), 0), G - 1);
    const int iv = min(max((int)((v + 1.f) * (0.5f * G)), 0), G - 1);
    return (face * G + iv) * G + iu;
}

// The icosahedron face containing direction w: a cube-map cell gives at most eight candidate
// faces (all 20 are scanned if none contains w).
PG3_DI int steerFace(const SteerView &T, float3 w)
{
    float fu, fv;
    const int cell = cubeCell(cubeFace(w, fu, fv), fu, fv, kSteerCellsDev);
    const int4 ca = __ldg(&T.faceCells[2 * cell]), cb = __ldg(&T.faceCells[2 * cell + 1]);
    const int cs[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
    int best = cs[0] >= 0 ? cs[0] : 0;
    float bestMin = -1e30f;
    for (int i = 0; i < 8 && cs[i] >= 0; ++i) {
        const float m = faceMinEdge(T, cs[i], w);
        if (m > bestMin) { bestMin = m; best = cs[i]; }
    }
    if (bestMin < -1e-6f) {
        for (int f = 0; f < 20; ++f) {
            const float m = faceMinEdge(T, f, w);
            if (m > bestMin) { bestMin = m; best = f; }
        }
    }
    return best;
}

// Which of the four children of a subdivided triangle (children (A,ab,ca), (ab,B,bc), (ca,bc,C),
// (ab,bc,ca)) contains w: three great-circle tests against the edge midpoints.
PG3_DI int steerChild(float3 w, float3 ab, float3 bc, float3 ca)
{
    if (dot(w, cross(ab, ca)) >= 0.f) return 0;
    if (dot(w, cross(bc, ab)) >= 0.f) return 1;
    if (dot(w, cross(ca, bc)) >= 0.f) return 2;
    return 3;
}

// Leaf containing direction w through the uniform hierarchy: its face, then one of four
// children per subdivision level.
PG3_DI int steerLocateFaces(const SteerView &T, float3 w)
{
    int local = steerFace(T, w);
    for (uint32_t l = 0; l < T.level; ++l) {
        const uint32_t off = 20u * (((1u << (2 * (l + 1))) - 1u) / 3u);   // first triangle of level l+1
        const int4 mid = __ldg(&T.tri[off + 4 * local + 3]);   // (ab, bc, ca)
        const float3 ab = vdir(T, mid.x), bc = vdir(T, mid.y), ca = vdir(T, mid.z);
        local = 4 * local + steerChild(w, ab, bc, ca);
    }
    return local;
}

// Leaf containing direction w in an adaptive triangulation: the quadtree of the subdivided
// triangles down to a leaf (bounded by the deepest level), from the deepest triangle that holds w's
// start cell, or from w's level-0 face where the cell lies on several faces.
PG3_DI int steerLocateAdaptive(const SteerView &T, float3 w)
{
    int code = INT_MIN;
    if (T.startCells) {
        float fu, fv;
        const int cf = cubeFace(w, fu, fv);
        code = __ldg(&T.startCells[cubeCell(cf, fu, fv, kSteerStartGridDev)]);
    }
    if (code == INT_MIN) {
        const int f = steerFace(T, w);
        const int4 fc = __ldg(&T.qtree[f >> 2]);
        code = (f & 3) == 0 ? fc.x : (f & 3) == 1 ? fc.y : (f & 3) == 2 ? fc.z : fc.w;
    }
    for (uint32_t depth = 0; depth <= kSteerMaxAdaptiveDepth && code >= 0; ++depth) {
        const int4 mid = __ldg(&T.qtree[5 + 2 * code]);
        const int4 ch = __ldg(&T.qtree[5 + 2 * code + 1]);
        const int c = steerChild(w, vdir(T, mid.x), vdir(T, mid.y), vdir(T, mid.z));
        code = c == 0 ? ch.x : c == 1 ? ch.y : c == 2 ? ch.z : ch.w;
    }
    return code < 0 ? ~code : 0;
}

// Leaf containing direction w: the start cell names it where one leaf holds the whole cell;
// otherwise the leaf-locator cell lists every leaf that can touch it, so the one whose three edge
// planes all face w is among them (the face hierarchy decides for cells with more than eight
// candidates, and if rounding puts w outside all candidates).
PG3_DI int steerLocate(const SteerView &T, float3 w)
{
    float fu, fv;
    const int face = cubeFace(w, fu, fv);
    if (kSteerUniformStartGridDev > 0 && T.startCells) {   // the cell lies in one leaf
        const int s = __ldg(&T.startCells[cubeCell(face, fu, fv, kSteerUniformStartGridDev)]);
        if (s != INT_MIN) return ~s;
    }
    const uint4 cell = __ldg(&steerCells(T)[cubeCell(face, fu, fv, (int)steerGrid(T))]);
    if (cell.x != 0xfffefffeu) {
        const uint32_t words[4] = {cell.x, cell.y, cell.z, cell.w};
        const float4 *E = steerEdges(T);
        int best = -1;
        float bestMin = -1e30f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t id = (words[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
            if (id == 0xffffu) break;
            const float m = fminf(fminf(dot(w, xyz(__ldg(&E[3 * id]))), dot(w, xyz(__ldg(&E[3 * id + 1])))),
                                  dot(w, xyz(__ldg(&E[3 * id + 2]))));
            if (m > bestMin) { bestMin = m; best = (int)id; }
            if (m >= 0.f) break;
        }
        if (best >= 0 && bestMin >= -1e-6f) return best;
    }
    return steerLocateFaces(T, w);
}

// base(w) of one direction: its leaf, the point where w meets the leaf's plane, the linear
// interpolation of the leaf's vertex values there.
PG3_DI float steerBasePdf(const SteerView &T, int leaf, float3 w, const SteerQuad &q, float Z)
{
    const SteerLeaf<false> L = steerLeaf<false>(T, leaf);
    const float dw = dot(xyz(L.plane), w);
    if (!(dw > 0.f)) return 0.f;
    const float3 A = xyz(L.A), B = xyz(L.B), C = xyz(L.C);
    const float3 p = w * (L.plane.w / dw);
    const float3 n = cross(B - A, C - A);
    const float nn = dot(n, n);
    const float b0 = dot(cross(B - p, C - p), n) / nn;
    const float b1 = dot(cross(C - p, A - p), n) / nn;
    const float b2 = 1.f - b0 - b1;
    const float g = b0 * vvalPair(q, A, L.A.w, 0.f).x + b1 * vvalPair(q, B, L.B.w, 0.f).x +
                    b2 * vvalPair(q, C, L.C.w, 0.f).x;
    return steerLeafPdf(L.plane.w, p, g, Z);
}

// base(w) + base(-w). Uniform levels: w's leaf, w's barycentric coordinates there, and the values
// of the leaf's vertices and of their antipodes. Adaptive: -w is located in its own leaf.
template <bool ADAPTIVE>
PG3_DI float steerPairPdf(const SteerView &T, float3 w, const SteerQuad &q, float Z)
{
    if (ADAPTIVE)
        return steerBasePdf(T, steerLocateAdaptive(T, w), w, q, Z) + steerBasePdf(T, steerLocateAdaptive(T, -w), -w, q, Z);
    const int leaf = steerLocate(T, w);
    const SteerLeaf<true> L = steerLeaf<true>(T, leaf);
    const float dw = dot(xyz(L.plane), w);
    if (!(dw > 0.f)) return 0.f;
    const float3 A = xyz(L.A), B = xyz(L.B), C = xyz(L.C);
    const float3 p = w * (L.plane.w / dw);       // w meets the leaf's plane
    const float3 n = cross(B - A, C - A);
    const float nn = dot(n, n);
    const float b0 = dot(cross(B - p, C - p), n) / nn;
    const float b1 = dot(cross(C - p, A - p), n) / nn;
    const float b2 = 1.f - b0 - b1;
    const float2 va = vvalPair(q, A, L.A.w, L.anti.x), vb = vvalPair(q, B, L.B.w, L.anti.y),
                 vc = vvalPair(q, C, L.C.w, L.anti.z);
    const float g = b0 * va.x + b1 * vb.x + b2 * vc.x;
    const float ga = b0 * va.y + b1 * vb.y + b2 * vc.y;
    return steerLeafPdf(L.plane.w, p, g, Z) + steerLeafPdf(L.plane.w, p, ga, Z);
}

// Pdf of the mirrored-hemisphere sampler for a direction above the surface (front side).
template <bool ADAPTIVE = false>
PG3_DI float steerPdf(const SteerView &T, float3 w, float3 n)
{
    if (dot(w, n) < 0.f) return 0.f;
    float c[9];
    steerCoeffs(n, c);
    const float Z = steerTotal(T, c);
    if (!(Z > 0.f)) return 0.f;
    return steerPairPdf<ADAPTIVE>(T, w, steerQuad(c), Z);
}

// Samples a direction in the upper hemisphere of n. Returns false when the map is black.
template <bool ADAPTIVE = false>
PG3_DI bool steerSample(const SceneView &S, float3 n, float u0, float u1, float u2, float3 &wig, float &pdf,
                        float3 &radCos)
{
    const SteerView &T = S.steer;
    float c[9];
    steerCoeffs(n, c);
    const float Z = steerTotal(T, c);
    if (!(Z > 0.f)) { pdf = 0.f; radCos = f3(0.f); wig = n; return false; }
    // tree descent with the rescaled uniform (src/em_steerable_sampler.hxx:3798-3875)
    int node = T.root;
    float u = u0;
    int leaf = -1;
    for (int depth = 0; depth < 32; ++depth) {
        // a node: the 6 children's weights coefficient-major, packed (54 floats in 14 float4,
        // element 6 k + i: coefficient k of child i), then its first child and child count
        const float4 *w4 = reinterpret_cast<const float4 *>(T.nodeW) + kSteerNodeVec4 * node;
        float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float4 tail;
#pragma unroll
        for (int j = 0; j < kSteerNodeVec4; ++j) {
            const float4 a = __ldg(&w4[j]);
            const float v[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int e = 4 * j + t;
                if (e < 54) acc[e % 6] += v[t] * c[e / 6];
            }
            if (j == kSteerNodeVec4 - 1) tail = a;
        }
        // a node's children are consecutive nodes, or consecutive leaves (codes ~leaf), so the
        // record's tail names them all (no load of the node's child slots)
        int ids[6];
        const int first = __float_as_int(tail.z), count = __float_as_int(tail.w);
#pragma unroll
        for (int i = 0; i < 6; ++i) ids[i] = (i < count) ? ((first >= 0) ? first + i : first - i) : INT_MIN;
        float val[6], cum = 0.f;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            val[i] = (ids[i] != INT_MIN) ? fmaxf(acc[i], 0.f) : 0.f;
            cum += val[i];
        }
        // children occupy the first slots; the first one whose running sum exceeds t wins,
        // rounding past the end falls back to the last child. The scan is unrolled over the
        // six slots with the chosen child's value and id carried in registers (an indexed
        // pick would place ids[] and val[] in local memory).
        const float t = u * 0.999999f * cum;
        float lo = 0.f, vPick = 0.f;
        int idPick = INT_MIN;
        bool alive = true, found = false;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            alive = alive && ids[i] != INT_MIN;
            if (alive && !found) {
                vPick = val[i];
                idPick = ids[i];
                if (t < lo + val[i]) found = true;
                else lo += val[i];
            }
        }
        if (idPick == INT_MIN) { atomicOr(S.errorFlag, kErrSteerDescent); return false; }
        if (!found) lo -= vPick;
        u = fminf((t - lo) / fmaxf(vPick, 1e-30f), 1.f);
        const int id = idPick;
        if (id < 0) { leaf = ~id; break; }
        node = id;
    }
    if (leaf < 0) { atomicOr(S.errorFlag, kErrSteerDescent); return false; }

    // exact sample of the linear density on the planar triangle: pick corner i with
    // probability v_i / sum, then barycentric b_i from its marginal 6b(1-b) (inverse of
    // 3b^2 - 2b^3), the other two uniformly along the remaining segment
    const SteerLeaf<!ADAPTIVE> L = steerLeaf<!ADAPTIVE>(T, leaf);
    const float4 A4 = L.A, B4 = L.B, C4 = L.C;
    const SteerQuad q = steerQuad(c);
    const float2 va = vvalPair(q, xyz(A4), A4.w, L.anti.x), vb = vvalPair(q, xyz(B4), B4.w, L.anti.y),
                 vc = vvalPair(q, xyz(C4), C4.w, L.anti.z);
    const float v0 = va.x, v1 = vb.x, v2 = vc.x;
    const float vs = v0 + v1 + v2;
    const float ts = u * vs;
    const int corner = (vs > 0.f) ? ((ts < v0) ? 0 : ((ts < v0 + v1) ? 1 : 2)) : min((int)(u * 3.f), 2);
    const float bi = 0.5f - sinf(asinf(clampf(1.f - 2.f * u1, -1.f, 1.f)) * (1.f / 3.f));
    const float rest = 1.f - bi;
    const float bj = rest * u2, bk = rest - bj;
    float b0, b1, b2;
    if (corner == 0) { b0 = bi; b1 = bj; b2 = bk; }
    else if (corner == 1) { b1 = bi; b2 = bj; b0 = bk; }
    else { b2 = bi; b0 = bj; b1 = bk; }
    const float3 p = xyz(A4) * b0 + xyz(B4) * b1 + xyz(C4) * b2;
    const float3 w0 = normalize(p);
    if (ADAPTIVE) {
        // -w0 lies in a leaf of its own
        pdf = steerLeafPdf(L.plane.w, p, b0 * v0 + b1 * v1 + b2 * v2, Z) +
              steerBasePdf(T, steerLocateAdaptive(T, -w0), -w0, q, Z);
    } else {
        // -w0 lies in the antipodal leaf at the same barycentric coordinates
        const float ga = b0 * va.y + b1 * vb.y + b2 * vc.y;
        pdf = steerLeafPdf(L.plane.w, p, b0 * v0 + b1 * v1 + b2 * v2, Z) + steerLeafPdf(L.plane.w, p, ga, Z);
    }
    float cosIn = dot(w0, n);
    wig = w0;
    if (cosIn < 0.f) { wig = -w0; cosIn = -cosIn; }
    radCos = emEvaluateDir(S, wig) * cosIn;
    return true;
}

}  // namespace pg3
