// Ray queries: closest hit and any hit, over the primitive list or the LBVH.
//
// The reference tests every primitive in list order (src/scene_graph.hxx:33-82).
// For the small scenes of the benchmarks that loop is also what is fastest on a
// GPU (all lanes read the same primitive: one broadcast load per test), so it is
// kept; larger scenes use the linear BVH built on the device (pg3_lbvh.cu).
// Both return the same hit: the BVH visits leaves in a different order but a
// leaf only replaces the current hit when strictly closer, and ties are broken
// towards the lower primitive index exactly as the list loop breaks them.
#pragma once

#include <climits>

#include "pg3_device.cuh"

namespace pg3 {

constexpr int kBvhStackSize = 64;

PG3_DI bool slabHit(float3 lo, float3 hi, float3 org, float3 inv, float tmin, float tmax, float &tEnter)
{
    const float tx0 = (lo.x - org.x) * inv.x, tx1 = (hi.x - org.x) * inv.x;
    const float ty0 = (lo.y - org.y) * inv.y, ty1 = (hi.y - org.y) * inv.y;
    const float tz0 = (lo.z - org.z) * inv.z, tz1 = (hi.z - org.z) * inv.z;
    const float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    const float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
    tEnter = t0;
    return t0 <= t1;
}

// Test primitive `prim` (triangles first, then spheres); updates tmax on a closer hit.
PG3_DI bool hitPrim(const SceneView &S, uint32_t prim, float3 org, float3 dir, float tmin, float &tmax)
{
    if (prim >= S.ntri + S.nsph) { atomicOr(S.errorFlag, kErrTraversalStack); return false; }
    if (prim < S.ntri) {
        const float4 a = __ldg(&S.tri[3 * prim]), b = __ldg(&S.tri[3 * prim + 1]), c = __ldg(&S.tri[3 * prim + 2]);
        return hitTriangle(a, b, c, org, dir, tmin, tmax);
    }
    return hitSphere(__ldg(&S.sph[prim - S.ntri]), org, dir, tmin, tmax);
}

// Conservative enlargement of a slab interval so that a primitive hit exactly on a
// box face is never culled by rounding in the slab test.
PG3_DI float bvhPad(float t) { return t * 1.0000004f + 1e-7f; }

// A lower-indexed primitive may also win at exactly the current distance (the list loop
// keeps the first of equally distant hits): widen its bound by one ulp.
PG3_DI float tieBound(float tmax, uint32_t p, int best)
{
    return (best >= 0 && (int)p < best) ? __int_as_float(__float_as_int(tmax) + 1) : tmax;
}

PG3_DI bool intersectBvh(const SceneView &S, float3 org, float3 dir, float tmin, Hit &h)
{
    const uint32_t nprim = S.ntri + S.nsph;
    float tmax = 1e36f;
    int best = -1;
    if (nprim == 1) {
        if (hitPrim(S, 0, org, dir, tmin, tmax)) best = 0;
        h.t = tmax; h.prim = best;
        return best >= 0;
    }
    const float3 inv = make_float3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    int stack[kBvhStackSize];
    int sp = 0;
    int node = (int)S.bvhRoot;
    // a well-formed tree visits each of its nprim - 1 inner nodes at most once
    for (uint32_t guard = 0;; ++guard) {
        if (guard >= nprim || (uint32_t)node >= nprim - 1) { atomicOr(S.errorFlag, kErrTraversalStack); break; }
        const BvhNode nd = S.bvh[node];
        const int cl = __float_as_int(nd.lo_l.w), cr = __float_as_int(nd.lo_r.w);
        float el, er;
        const bool hl = slabHit(xyz(nd.lo_l), xyz(nd.hi_l), org, inv, tmin, bvhPad(tmax), el);
        const bool hr = slabHit(xyz(nd.lo_r), xyz(nd.hi_r), org, inv, tmin, bvhPad(tmax), er);
        int next = -1, other = -1;
        // leaves are processed immediately; inner children are pushed nearest-first
        if (hl) {
            if (cl < 0) {
                const uint32_t p = (uint32_t)(~cl);
                float t = tieBound(tmax, p, best);
                if (hitPrim(S, p, org, dir, tmin, t)) { tmax = t; best = (int)p; }
            } else next = cl;
        }
        if (hr) {
            if (cr < 0) {
                const uint32_t p = (uint32_t)(~cr);
                float t = tieBound(tmax, p, best);
                if (hitPrim(S, p, org, dir, tmin, t)) { tmax = t; best = (int)p; }
            } else if (next < 0) next = cr;
            else {
                other = cr;
                if (er < el) { other = next; next = cr; }
            }
        }
        if (other >= 0) {
            if (sp < kBvhStackSize) stack[sp++] = other;
            else atomicOr(S.errorFlag, kErrTraversalStack);
        }
        if (next < 0) {
            if (sp == 0) break;
            node = stack[--sp];
        } else node = next;
    }
    h.t = tmax;
    h.prim = best;
    return best >= 0;
}

PG3_DI bool occludedBvh(const SceneView &S, float3 pt, float3 dir, float dist)
{
    const float3 org = pt + dir * kEpsRay;
    const float tmax0 = dist - 2.f * kEpsRay;
    const uint32_t nprim = S.ntri + S.nsph;
    if (nprim == 1) { float t = tmax0; return hitPrim(S, 0, org, dir, 0.f, t); }
    const float3 inv = make_float3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    int stack[kBvhStackSize];
    int sp = 0;
    int node = (int)S.bvhRoot;
    for (uint32_t guard = 0;; ++guard) {
        if (guard >= nprim || (uint32_t)node >= nprim - 1) { atomicOr(S.errorFlag, kErrTraversalStack); break; }
        const BvhNode nd = S.bvh[node];
        const int cl = __float_as_int(nd.lo_l.w), cr = __float_as_int(nd.lo_r.w);
        float el, er;
        const bool hl = slabHit(xyz(nd.lo_l), xyz(nd.hi_l), org, inv, 0.f, bvhPad(tmax0), el);
        const bool hr = slabHit(xyz(nd.lo_r), xyz(nd.hi_r), org, inv, 0.f, bvhPad(tmax0), er);
        int next = -1;
        if (hl) {
            if (cl < 0) { float t = tmax0; if (hitPrim(S, (uint32_t)(~cl), org, dir, 0.f, t)) return true; }
            else next = cl;
        }
        if (hr) {
            if (cr < 0) { float t = tmax0; if (hitPrim(S, (uint32_t)(~cr), org, dir, 0.f, t)) return true; }
            else if (next < 0) next = cr;
            else {
                if (sp < kBvhStackSize) stack[sp++] = cr;
                else atomicOr(S.errorFlag, kErrTraversalStack);
            }
        }
        if (next < 0) {
            if (sp == 0) break;
            node = stack[--sp];
        } else node = next;
    }
    return false;
}

// ------------------------------------------------------------------------------------------
// 4-wide BVH (BvhNode4): half the levels of the binary tree, four slab tests per node from
// coordinate-major boxes. The children's entry distances order the pushes (farthest first), so
// the nearest inner child is visited next; leaves are tested as they are met, with the same tie
// rule as the list loop, so both trees return the same hit.
// ------------------------------------------------------------------------------------------
PG3_DI const BvhNode4 *bvh4(const SceneView &S) { return reinterpret_cast<const BvhNode4 *>(S.bvh); }

// Slab test of the 4 children of a wide node; mask bit k set when child k is hit (entry t in te[k]).
PG3_DI uint32_t slabHit4(const BvhNode4 &n, float3 org, float3 inv, float tmin, float tmax, float te[4])
{
    const float lx[4] = {n.lox.x, n.lox.y, n.lox.z, n.lox.w}, hx[4] = {n.hix.x, n.hix.y, n.hix.z, n.hix.w};
    const float ly[4] = {n.loy.x, n.loy.y, n.loy.z, n.loy.w}, hy[4] = {n.hiy.x, n.hiy.y, n.hiy.z, n.hiy.w};
    const float lz[4] = {n.loz.x, n.loz.y, n.loz.z, n.loz.w}, hz[4] = {n.hiz.x, n.hiz.y, n.hiz.z, n.hiz.w};
    const int ch[4] = {n.child.x, n.child.y, n.child.z, n.child.w};
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float t;
        if (ch[k] != INT_MIN &&
            slabHit(make_float3(lx[k], ly[k], lz[k]), make_float3(hx[k], hy[k], hz[k]), org, inv, tmin, tmax, t))
            mask |= 1u << k;
        te[k] = t;
    }
    return mask;
}

PG3_DI bool intersectBvh4(const SceneView &S, float3 org, float3 dir, float tmin, Hit &h)
{
    const uint32_t nprim = S.ntri + S.nsph;
    float tmax = 1e36f;
    int best = -1;
    if (nprim == 1) {
        if (hitPrim(S, 0, org, dir, tmin, tmax)) best = 0;
        h.t = tmax; h.prim = best;
        return best >= 0;
    }
    const float3 inv = make_float3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    const BvhNode4 *nodes = bvh4(S);
    int stack[kBvhStackSize];
    int sp = 0;
    int node = 0;
    // a well-formed tree has fewer than nprim nodes, each visited at most once
    for (uint32_t guard = 0;; ++guard) {
        if (guard >= nprim) { atomicOr(S.errorFlag, kErrTraversalStack); break; }
        const BvhNode4 nd = nodes[node];
        float te[4];
        const uint32_t mask = slabHit4(nd, org, inv, tmin, bvhPad(tmax), te);
        const int ch[4] = {nd.child.x, nd.child.y, nd.child.z, nd.child.w};
        // inner children hit, ordered by entry distance (at most 4: insertion into registers)
        int id[4] = {-1, -1, -1, -1};
        float dt[4] = {0.f, 0.f, 0.f, 0.f};
        int cnt = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!(mask & (1u << k))) continue;
            if (ch[k] < 0) {
                const uint32_t p = (uint32_t)(~ch[k]);
                float t = tieBound(tmax, p, best);
                if (hitPrim(S, p, org, dir, tmin, t)) { tmax = t; best = (int)p; }
            } else {
                // keep id/dt sorted nearest first
                int c = ch[k];
                float tc = te[k];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (j < cnt && tc < dt[j]) {
                        const int ci = id[j];
                        const float ct = dt[j];
                        id[j] = c;
                        dt[j] = tc;
                        c = ci;
                        tc = ct;
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j == cnt) { id[j] = c; dt[j] = tc; }
                ++cnt;
            }
        }
        // push the farther ones (farthest first), continue with the nearest
#pragma unroll
        for (int j = 3; j >= 1; --j) {
            if (j < cnt) {
                if (sp < kBvhStackSize) stack[sp++] = id[j];
                else atomicOr(S.errorFlag, kErrTraversalStack);
            }
        }
        if (cnt > 0) node = id[0];
        else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    h.t = tmax;
    h.prim = best;
    return best >= 0;
}

PG3_DI bool occludedBvh4(const SceneView &S, float3 pt, float3 dir, float dist)
{
    const float3 org = pt + dir * kEpsRay;
    const float tmax0 = dist - 2.f * kEpsRay;
    const uint32_t nprim = S.ntri + S.nsph;
    if (nprim == 1) { float t = tmax0; return hitPrim(S, 0, org, dir, 0.f, t); }
    const float3 inv = make_float3(1.f / dir.x, 1.f / dir.y, 1.f / dir.z);
    const BvhNode4 *nodes = bvh4(S);
    int stack[kBvhStackSize];
    int sp = 0;
    int node = 0;
    for (uint32_t guard = 0;; ++guard) {
        if (guard >= nprim) { atomicOr(S.errorFlag, kErrTraversalStack); break; }
        const BvhNode4 nd = nodes[node];
        float te[4];
        const uint32_t mask = slabHit4(nd, org, inv, 0.f, bvhPad(tmax0), te);
        const int ch[4] = {nd.child.x, nd.child.y, nd.child.z, nd.child.w};
        int next = -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (!(mask & (1u << k))) continue;
            if (ch[k] < 0) {
                float t = tmax0;
                if (hitPrim(S, (uint32_t)(~ch[k]), org, dir, 0.f, t)) return true;
            } else if (next < 0) next = ch[k];
            else if (sp < kBvhStackSize) stack[sp++] = ch[k];
            else atomicOr(S.errorFlag, kErrTraversalStack);
        }
        if (next < 0) {
            if (sp == 0) break;
            node = stack[--sp];
        } else node = next;
    }
    return false;
}

// TRAV: 0 the primitive list, 1 the binary LBVH, 2 the 4-wide BVH; -1 reads S.useBvh; -2 reads it
// among the list and the binary LBVH only (the batch pipeline, whose instances never use the wide
// tree, keeps its query kernels free of the wide traversal's registers).
template <int TRAV = -1>
PG3_DI bool intersectClosest(const SceneView &S, float3 org, float3 dir, float tmin, Hit &h)
{
    const int t = (TRAV >= 0) ? TRAV : (TRAV == -2 ? (S.useBvh ? 1 : 0) : S.useBvh);
    return t == 2 ? intersectBvh4(S, org, dir, tmin, h)
                  : t == 1 ? intersectBvh(S, org, dir, tmin, h) : intersectList(S, org, dir, tmin, h);
}
template <int TRAV = -1>
PG3_DI bool occludedAny(const SceneView &S, float3 pt, float3 dir, float dist)
{
    const int t = (TRAV >= 0) ? TRAV : (TRAV == -2 ? (S.useBvh ? 1 : 0) : S.useBvh);
    return t == 2 ? occludedBvh4(S, pt, dir, dist) : t == 1 ? occludedBvh(S, pt, dir, dist) : occludedList(S, pt, dir, dist);
}

}  // namespace pg3
