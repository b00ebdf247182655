// Stage code shared by the wavefront pipelines: the single-scene pipeline and its path-replay
// adjoint (pg3_wavefront.cu) and the many-scene pipeline (pg3_batch.cu).
//
// A path lives in a slot, which indexes its radiance accumulator. Its state (beta, ew, pn; 48
// bytes) travels with its ray: the state record at position i of a state queue belongs to the ray
// at position i of the ray queue of the same parity, so a shade kernel reads ray, hit and state
// of a bucket entry at one index, and writes the next state where it appends the next ray. Rays
// and shadow records name their path by a tag: the slot in the low 24 bits and, in the batch
// pipeline, the scene instance in the high 8 bits.
//
// shadeVertex is one vertex of the estimator of pg3_estimator.cuh (src/path_tracer.hxx:167-430)
// for one material kind K: emitter / background MIS, the light sample (folded into a shadow
// record), Russian roulette and the BSDF sample (the next ray). With GRAD it also carries the
// adjoint of path-replay backpropagation (Vicini, Speierer and Jakob, "Path Replay
// Backpropagation", SIGGRAPH 2021): the adjoint pass re-runs the same instructions on the same
// random numbers as a primal pass that stored each path's radiance, and at every vertex
//   - the radiance that arrived after the previous vertex's BSDF sample is the path's stored
//     total minus what has accumulated so far; times d ln f / d theta of that vertex it is the
//     previous vertex's BSDF-sample gradient (deferred by one vertex so that the previous
//     vertex's light sample, resolved by the shadow stage, is already accumulated),
//   - a light sample carries its own gradient in its shadow record, scattered if unoccluded,
//   - background emission scatters into the environment-map texels of its bilinear lookup.
// Sampling decisions (directions, pdfs, MIS weights, light picking, roulette probabilities) are
// treated as constants of the current parameters ("detached"), as in the paper.
#pragma once

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "pg3_estimator.cuh"
#include "pg3_kernels.h"

namespace pg3 {

namespace cg = cooperative_groups;

constexpr int kWaveBlock = PG3_WAVE_BLOCK;
// Material buckets: one per kind, the two Dirac materials share one (their kernels are short).
// A shade kernel's K is its kind, kShadeSmooth the shared Dirac bucket, -1 the miss bucket.
enum : int {
    kBucketMiss = 0, kBucketLambert = 1, kBucketConductor = 2, kBucketDielectric = 3, kBucketPhong = 4,
    kBucketSmooth = 5, kNumBuckets = 6
};
constexpr int kShadeSmooth = kMatSmoothConductor;
PG3_DI constexpr int bucketOfShade(int K) { return (K < 0) ? kBucketMiss : 1 + K; }
PG3_DI int bucketOfKind(int kind) { return min(1 + kind, (int)kBucketSmooth); }
constexpr uint32_t kFlagFinite = 1u << 16, kFlagRefl = 1u << 17;
constexpr uint32_t kSlotBits = 24, kSlotMask = (1u << kSlotBits) - 1u;
constexpr uint32_t kMaxSlots = 1u << kSlotBits;

struct Counters {
    uint32_t ray[2];
    uint32_t bucket[kNumBuckets];
    uint32_t shadow;
    uint32_t pad;
};

struct Queues {
    float4 *ray[2];           // 2 float4 per entry: origin + tmin, direction + tag
    float2 *hit;              // (t, primitive as int bits)
    uint32_t *bucket[kNumBuckets];   // consecutive: bucket[b] = bucket[0] + b * bucketStride
    size_t bucketStride;
    float4 *st[2];            // per ray-queue entry, 3 float4: beta.xyz + parent bsdf pdf, emission
                              // weight.xyz + parent light-estimate sum, parent normal.xyz + flags
                              // (path length | finite | compute-reflected)
    float4 *shadow;           // kShadowWords<GRAD> float4 per record
    float2 *pend;             // GRAD, per slot: material of the previous vertex (int bits), its d att
    Counters *cnt;
    uint32_t cap;             // entries of every queue; an append past it is dropped and flagged
    unsigned int *err;        // device error word (kErrQueueOverflow)
};

template <bool GRAD> constexpr int kShadowWords = GRAD ? 5 : 3;

// Queue q of a pair, chosen by a select: indexing the pointer pair of a kernel parameter with a
// run-time value would copy the whole parameter to local memory.
PG3_DI float4 *rayQ(const Queues &Q, int q) { return q ? Q.ray[1] : Q.ray[0]; }
PG3_DI float4 *stQ(const Queues &Q, int q) { return q ? Q.st[1] : Q.st[0]; }
PG3_DI uint32_t *bucketQ(const Queues &Q, int b) { return Q.bucket[0] + (size_t)b * Q.bucketStride; }

// Append by the lanes that call it (the active lanes of a warp are grouped; each group's leader
// reserves its slots): usable inside divergent code, unlike warpAppend.
PG3_DI uint32_t activeAppend(uint32_t *counter)
{
    const unsigned m = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// Shadow records are appended where the light sample is taken (PG3_EARLY_SHADOW), so that the
// record's 12 floats are not held through the BSDF sample until the end of the vertex (+1.4% on
// the environment-map benchmark).
#ifndef PG3_EARLY_SHADOW
#define PG3_EARLY_SHADOW 1
#endif

// Warp-aggregated append: lanes with `want` get consecutive slots of *counter.
PG3_DI uint32_t warpAppend(uint32_t *counter, bool want)
{
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

PG3_DI void countWarp(unsigned long long *dst, uint32_t v)
{
    const uint32_t s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
}

// ------------------------------------------------------------------------------------------
// gradient scatter
// ------------------------------------------------------------------------------------------
// Lanes that add to the same texel are summed within the warp first (sun lobes send many
// light samples of a warp to the same few texels).
PG3_DI void warpAggregatedAdd3(float *base, uint32_t key, float3 v)
{
    cg::coalesced_group act = cg::coalesced_threads();
    cg::coalesced_group grp = cg::labeled_partition(act, key);
    const float x = cg::reduce(grp, v.x, cg::plus<float>());
    const float y = cg::reduce(grp, v.y, cg::plus<float>());
    const float z = cg::reduce(grp, v.z, cg::plus<float>());
    if (grp.thread_rank() == 0) {
        float *p = base + 3 * (size_t)key;
        if (x != 0.f) atomicAdd(p, x);
        if (y != 0.f) atomicAdd(p + 1, y);
        if (z != 0.f) atomicAdd(p + 2, z);
    }
}

// d/d texel of the bilinear lookup emEvaluateDir(S, dir), times the radiance weight w.
PG3_DI void gradEmDir(const SceneView &S, float *gEm, float3 dir, float3 w)
{
    float u, v;
    dir2LatLong(dir, u, v);
    const float xf = u * (float)S.emW, yf = v * (float)S.emH;
    const int cx = (int)(xf + 0.5f), cy = (int)(yf + 0.5f);
    const int x0 = cx - 1, y0 = cy - 1;
    const float xl = xf - ((float)x0 + 0.5f), yl = yf - ((float)y0 + 0.5f);
    uint32_t ax, ay, bx, by;
    emWrap(S, x0, y0, ax, ay);
    emWrap(S, cx, cy, bx, by);
    warpAggregatedAdd3(gEm, ay * S.emW + ax, w * ((1.f - xl) * (1.f - yl)));
    warpAggregatedAdd3(gEm, ay * S.emW + bx, w * (xl * (1.f - yl)));
    warpAggregatedAdd3(gEm, by * S.emW + ax, w * ((1.f - xl) * yl));
    warpAggregatedAdd3(gEm, by * S.emW + bx, w * (xl * yl));
}

// Per-block material gradients (shared memory, 4 floats per material), flushed at block end.
PG3_DI void gradMatAdd(float *sGrad, int mat, float4 g)
{
    float *p = sGrad + 4 * mat;
    if (g.x != 0.f) atomicAdd(p, g.x);
    if (g.y != 0.f) atomicAdd(p + 1, g.y);
    if (g.z != 0.f) atomicAdd(p + 2, g.z);
    if (g.w != 0.f) atomicAdd(p + 3, g.w);
}

// Gradient of everything that followed a BSDF sample of material `mat`: `after` is that radiance
// times dLoss/dradiance. Lambert: every later term is linear in albedo_c; GGX: times d ln f / da.
PG3_DI void gradContinuation(const SceneView &S, float *sGrad, int mat, float dAtt, float3 after)
{
    if ((uint32_t)mat >= S.nmat) return;   // sGrad holds 4 * nmat floats
    const DevMaterial m = loadMat(S, mat);
    if (m.kind == kMatLambert)
        gradMatAdd(sGrad, mat, make_float4(m.r > 0.f ? after.x / m.r : 0.f, m.g > 0.f ? after.y / m.g : 0.f,
                                           m.b > 0.f ? after.z / m.b : 0.f, 0.f));
    else
        gradMatAdd(sGrad, mat, make_float4(0.f, 0.f, 0.f, (after.x + after.y + after.z) * dAtt));
}

template <bool GRAD>
PG3_DI void initBlockGrad(float *sGrad, uint32_t nmat)
{
    if (!GRAD) return;
    for (uint32_t i = threadIdx.x; i < 4 * nmat; i += blockDim.x) sGrad[i] = 0.f;
    __syncthreads();
}
template <bool GRAD>
PG3_DI void flushBlockGrad(const float *sGrad, uint32_t nmat, float *gMat)
{
    if (!GRAD) return;
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 4 * nmat; i += blockDim.x)
        if (sGrad[i] != 0.f) atomicAdd(&gMat[i], sGrad[i]);
}

// ------------------------------------------------------------------------------------------
// one vertex
// ------------------------------------------------------------------------------------------
PG3_DI void prefetchL1(const void *p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }

// Software pipelining of a shade kernel's grid-stride loop: while a thread shades one entry of
// its bucket it pulls the next entry's ray and hit, then its path state, towards L1, so the
// next iteration's loads (bucket -> ray, hit, state) find them on chip.
struct NextEntry {
    const float4 *ray = nullptr;   // the next entry's ray record (null: none)
    const float2 *hit = nullptr;   // its hit record
    const float4 *st = nullptr;    // and its state record
};
PG3_DI void prefetchNextRay(const NextEntry &nx)
{
    if (nx.ray) {
        prefetchL1(nx.ray);
        prefetchL1(nx.ray + 1);
        prefetchL1(nx.hit);
    }
}
PG3_DI void prefetchNextState(const NextEntry &nx)
{
    if (nx.st) {
        prefetchL1(nx.st);
        prefetchL1(nx.st + 2);
    }
}
struct ShadeOut {
    bool shadow = false, next = false;
    float4 s0, s1, s2;        // shadow record: origin + distance, direction + tag, contribution
    float4 s3, s4;            // GRAD: material gradient (albedo rgb, roughness), environment weight + material
    float4 r0, r1;            // next ray
    float4 t0, t1, t2;        // its path state record
};

// acc: the path's radiance accumulated before this vertex (GRAD adjoint only).
// st: the entry's path state record (3 float4).
// EARLY: append the shadow record where the light sample is taken (PG3_EARLY_SHADOW); a caller
// that still edits the record after the vertex (the batch pipeline marks a path's last light
// sample) takes it in `o` instead.
template <int K, int EMK, bool GRAD, bool EARLY = (PG3_EARLY_SHADOW != 0)>
PG3_DI void shadeVertex(const SceneView &S, const Queues &Q, uint32_t idx, float4 r0, float4 r1, const float4 *st,
                        uint32_t slot, uint32_t tag, uint32_t pixel, uint32_t sample, PathCounters &pc, ShadeOut &o,
                        float3 &L, const GradArgs &G, float *sGrad, float3 acc, const NextEntry &nx = NextEntry())
{
    const float3 org = xyz(r0), dir = xyz(r1);
    const float4 sb = st[0], se = st[1], sn = st[2];
    const uint32_t flags = __float_as_uint(sn.w);
    const uint32_t pl = flags & 0xffffu;
    const bool prevFinite = (flags & kFlagFinite) != 0, computeRefl = (flags & kFlagRefl) != 0;
    const float3 beta = xyz(sb), ew = xyz(se), prevN = xyz(sn);
    const float prevBsdfPdf = sb.w, prevSum = se.w;
    const bool adj = GRAD && G.adjoint;
    float3 delta = f3(0.f);
    if (adj) {
        delta = make_float3(__ldg(&G.dLdI[3 * (size_t)pixel]), __ldg(&G.dLdI[3 * (size_t)pixel + 1]),
                            __ldg(&G.dLdI[3 * (size_t)pixel + 2])) * G.invSpp;
        const float2 pd = Q.pend[slot];
        const int pm = __float_as_int(pd.x);
        if (pm >= 0) {
            const float3 tot = make_float3(G.totR[slot], G.totG[slot], G.totB[slot]);
            gradContinuation(S, sGrad, pm, pd.y, delta * (tot - acc));
        }
    }
    L = f3(0.f);
    if (K < 0) {
        // background (src/path_tracer.hxx:408-429)
        if (pl >= S.minPL && S.bgKind != kBgNone) {
            float pdf = 0.f;
            const Frame pf = frameFromZ(prevN);
            const float3 Le = bgEmission<EMK>(S, dir, pl > 1 && prevFinite, pf, pdf);
            float mis = 1.f;
            if (pl == 1) L = Le;
            else if (prevFinite) {
                mis = misPower(prevBsdfPdf, pdf * pickProb(S, org, prevN, prevSum, S.bgLightId));
                L = ew * Le * mis;
            } else L = ew * Le;
            if (adj && S.bgKind == kBgEnvMap && G.gEm)
                gradEmDir(S, G.gEm, dir, delta * ((pl == 1) ? f3(1.f) : ew * mis));
        }
        if (computeRefl) ++pc.bg;
        return;
    }
    const float2 hh = Q.hit[idx];
    Hit h;
    h.t = hh.x;
    h.prim = __float_as_int(hh.y);
    float3 pt, nrm;
    int matId;
    hitAttributes(S, h, org, dir, pt, nrm, matId);
    prefetchNextRay(nx);
    const Frame frame = frameFromZ(nrm);
    const float3 wol = toLocal(frame, -dir);
    const int lightId = __ldg(&S.mat2light[matId]);
    if (lightId >= 0 && pl >= S.minPL) {
        float pdfA = 0.f;
        const float3 Le = areaEmission(S.lights[lightId], pt, wol.z, org, pdfA);
        if (pl == 1) L = Le;
        else if (!isZero(Le))
            L = prevFinite ? ew * Le * misPower(prevBsdfPdf, pdfA * pickProb(S, org, prevN, prevSum, lightId))
                           : ew * Le;
    }
    const DevMaterial mat = loadMat(S, matId);
    bool go = computeRefl;
    if (go && mat.zeroRefl) { ++pc.blocker; go = false; }
    if (go && S.maxPL > 0 && pl >= S.maxPL) { ++pc.maxl; go = false; }
    if (go && pl >= kMaxPathLengthHard) { ++pc.safety; go = false; }
    if (!go) return;
    constexpr bool kLights = K != kShadeSmooth;   // Dirac materials take no light samples
    const Rand4 ra = draw(S, pixel, sample, pl, 0);
    const Rand4 rb = draw(S, pixel, sample, pl, 1);
    const float sum = (kLights && S.lightCount > 1) ? estimateSum(S, pt, nrm) : 0.f;
    if (kLights && pl + 1 >= S.minPL) {
        int lid;
        float lprob = 0.f;
        pickLight(S, pt, nrm, sum, ra.a, lid, lprob);
        if (lid >= 0) {
            float3 wig, smp;
            float dist, pdfW;
            if (lid == S.bgLightId) {
                bgSample<EMK>(S, frame, ra.b, ra.c, ra.d, wig, pdfW, smp);
                dist = kFloatMax;
            } else {
                tableSample(S.lights[lid], pt, nrm, ra.b, ra.c, wig, dist, smp, pdfW);
            }
            if (maxc(smp) > 0.f) {
                BsdfRec br;
                evalBsdfK<K, GRAD>(mat, toLocal(frame, wig), wol, br);
                const float w = lightSampleWeight(pdfW, lprob, 1u, br.pdfW * br.compProb, 1u);
                const float3 c = beta * (smp * br.att) * w;
                o.shadow = true;
                o.s0 = make_float4(pt.x, pt.y, pt.z, dist);
                o.s1 = make_float4(wig.x, wig.y, wig.z, __uint_as_float(tag));
                o.s2 = make_float4(c.x, c.y, c.z, 0.f);
                if (GRAD) {
                    o.s3 = make_float4(0.f, 0.f, 0.f, 0.f);
                    o.s4 = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
                    if (adj) {
                        if (K == kMatLambert) {
                            const float3 g = delta * beta * smp * (w * br.dAtt);
                            o.s3 = make_float4(g.x, g.y, g.z, 0.f);
                        } else {
                            o.s3 = make_float4(0.f, 0.f, 0.f, dot(delta, c) * br.dAtt);
                        }
                        float3 e = f3(0.f);
                        if (lid == S.bgLightId && S.bgKind == kBgEnvMap && G.gEm)
                            e = delta * beta * br.att * (fabsf(dot(wig, nrm)) * w);
                        o.s4 = make_float4(e.x, e.y, e.z, __int_as_float(matId));
                    }
                }
                if (EARLY) {
                    constexpr int SW = kShadowWords<GRAD>;
                    const uint32_t sp = activeAppend(&Q.cnt->shadow);
                    if (sp >= Q.cap) atomicOr(Q.err, kErrQueueOverflow);
                    else {
                        float4 *d = Q.shadow + (size_t)SW * sp;
                        d[0] = o.s0;
                        d[1] = o.s1;
                        d[2] = o.s2;
                        if (GRAD) {
                            d[3] = o.s3;
                            d[4] = o.s4;
                        }
                    }
                    o.shadow = false;
                }
            }
        }
    }
    prefetchNextState(nx);
    // Russian roulette (src/path_tracer.hxx:267-303)
    float rrProb = 1.0f;
    bool cut = false;
    if (S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL)) {
        rrProb = rrContinuation<K>(mat, wol);
        cut = rb.a > rrProb;
    }
    // BSDF sample (src/path_tracer.hxx:305-322)
    BsdfRec br;
    if (K == kShadeSmooth) sampleBsdfSmooth<GRAD>(mat, wol, rb.d, br);
    else sampleBsdfK<K, GRAD>(mat, wol, rb.b, rb.c, rb.d, br);
    if (isBlocker(br)) {
        ++pc.blocker;
        return;
    }
    const bool finite = br.pdfW != infF();
    const float cosAbs = fabsf(br.wil.z);
    const float3 f = finite ? br.att * (cosAbs / (br.pdfW * br.compProb)) : br.att / br.compProb;
    const float3 ew2 = beta * f;
    const float3 beta2 = ew2 / rrProb;
    if (cut) ++pc.rr;
    o.t0 = make_float4(beta2.x, beta2.y, beta2.z, br.pdfW * br.compProb);
    o.t1 = make_float4(ew2.x, ew2.y, ew2.z, sum);
    const uint32_t nf = (pl + 1) | (finite ? kFlagFinite : 0u) | (cut ? 0u : kFlagRefl);
    o.t2 = make_float4(nrm.x, nrm.y, nrm.z, __uint_as_float(nf));
    if (GRAD) Q.pend[slot] = make_float2(__int_as_float(matId), br.dAtt);
    const float3 nd = toWorld(frame, br.wil);
    o.next = true;
    o.r0 = make_float4(pt.x, pt.y, pt.z, epsRayCos(cosAbs));
    o.r1 = make_float4(nd.x, nd.y, nd.z, __uint_as_float(tag));
}

// Appends a vertex's shadow record and next ray with its state (all lanes of the warp call this).
template <bool GRAD>
PG3_DI void emitRecords(const Queues &Q, int nextQueue, const ShadeOut &o)
{
    constexpr int SW = kShadowWords<GRAD>;
    const uint32_t sp = warpAppend(&Q.cnt->shadow, o.shadow);
    if (o.shadow && sp >= Q.cap) atomicOr(Q.err, kErrQueueOverflow);
    else if (o.shadow) {
        float4 *d = Q.shadow + (size_t)SW * sp;
        d[0] = o.s0;
        d[1] = o.s1;
        d[2] = o.s2;
        if (GRAD) {
            d[3] = o.s3;
            d[4] = o.s4;
        }
    }
    float4 *nq = rayQ(Q, nextQueue);
    const uint32_t rp = warpAppend(&Q.cnt->ray[nextQueue], o.next);
    if (o.next && rp >= Q.cap) atomicOr(Q.err, kErrQueueOverflow);
    else if (o.next) {
        nq[2 * (size_t)rp] = o.r0;
        nq[2 * (size_t)rp + 1] = o.r1;
        float4 *ns = stQ(Q, nextQueue) + 3 * (size_t)rp;
        ns[0] = o.t0;
        ns[1] = o.t1;
        ns[2] = o.t2;
    }
}

// Gradient part of an unoccluded shadow record.
template <bool GRAD>
PG3_DI void shadowGrad(const SceneView &S, const float4 *rec, float3 dir, const GradArgs &G, float *sGrad)
{
    if (!GRAD || !G.adjoint) return;
    const float4 g = rec[3], e = rec[4];
    const int mat = __float_as_int(e.w);
    if (mat < 0 || (uint32_t)mat >= S.nmat) return;   // sGrad holds 4 * nmat floats
    gradMatAdd(sGrad, mat, g);
    if (e.x != 0.f || e.y != 0.f || e.z != 0.f) gradEmDir(S, G.gEm, dir, xyz(e));
}

// Camera ray of (pixel, sample) (src/path_tracer_base.hxx:66-87, src/camera.hxx:91-100).
PG3_DI void cameraRay(const SceneView &S, uint32_t pixel, uint32_t sample, float3 &dir)
{
    const uint32_t px = pixel % S.width, py = pixel / S.width;
    const Rand4 rc = draw(S, pixel, sample, 0, 0);
    const float nx = ((float)px + rc.a) * (2.f / S.width) - 1.f;
    const float ny = ((float)py + rc.b) * (2.f / S.height) - 1.f;
    dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
}

// State of a camera ray at position pos of ray queue q.
// A camera path's state before its first vertex: throughput 1, no previous BSDF pdf or
// contribution, path length 1, finite, reflectance to compute.
PG3_DI void initialPathState(float4 st[3])
{
    st[0] = make_float4(1.f, 1.f, 1.f, 0.f);
    st[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    st[2] = make_float4(0.f, 0.f, 1.f, __uint_as_float(1u | kFlagFinite | kFlagRefl));
}
PG3_DI void initPathState(const Queues &Q, int q, uint32_t pos)
{
    float4 init[3];
    initialPathState(init);
    float4 *st = stQ(Q, q) + 3 * (size_t)pos;
    st[0] = init[0];
    st[1] = init[1];
    st[2] = init[2];
}

// Closest hit of one ray and its material bucket (-1 none). TRAV: the traversal (intersectClosest).
template <int TRAV = -1>
PG3_DI int extendOne(const SceneView &S, const Queues &Q, const float4 *rq, uint32_t i)
{
    const float4 r0 = rq[2 * i], r1 = rq[2 * i + 1];
    Hit h;
    const bool hit = intersectClosest<TRAV>(S, xyz(r0), xyz(r1), r0.w, h);
    Q.hit[i] = make_float2(h.t, __int_as_float(h.prim));
    if (!hit) return kBucketMiss;
    const int mat = ((uint32_t)h.prim < S.ntri) ? __float_as_int(__ldg(&triShade(S)[h.prim]).w)
                                                : __ldg(&S.sphMat[h.prim - S.ntri]);
    return bucketOfKind(__ldg(&S.mats[mat].kind));
}

// Appends queue index i to its bucket (-1: none); all lanes of the warp call this. Lanes of the
// same bucket are grouped with one match, and each group's leader reserves its slots.
PG3_DI void bucketAppend(const Queues &Q, int bucket, uint32_t i)
{
    const unsigned peers = __match_any_sync(0xffffffffu, bucket);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (bucket >= 0 && lane == leader) base = atomicAdd(&Q.cnt->bucket[bucket], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (bucket >= 0) {
        const uint32_t pos = base + __popc(peers & ((1u << lane) - 1u));
        if (pos < Q.cap) bucketQ(Q, bucket)[pos] = i;
        else atomicOr(Q.err, kErrQueueOverflow);
    }
}

}  // namespace pg3
