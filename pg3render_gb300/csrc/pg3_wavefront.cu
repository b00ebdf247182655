// Wavefront pipeline: the path estimator of pg3_estimator.cuh split into stage
// kernels that communicate through structure-of-arrays queues in HBM/L2.
//
// Per launch chunk (up to `capacity` paths, one slot per path):
//   raygen            camera rays of all slots -> ray queue A; path state init
//   per bounce:
//     extend          closest hit of every queued ray; the ray's queue index is
//                     appended to one of four buckets (miss, Lambert, GGX
//                     conductor, GGX dielectric) with warp-aggregated atomics
//     shade<kind>     one kernel per bucket: emitter MIS, light sample (the BSDF
//                     value and MIS weight are folded into a shadow record),
//                     Russian roulette, BSDF sample -> next ray queue
//     shadow          any-hit test of every shadow record; unoccluded records
//                     add their contribution to the path's radiance
//     advance         zero the counters consumed by this bounce
// Each stage kernel holds only its own material's code, which keeps it inside
// the instruction cache, and a warp shades hits of one material kind only.
// Launches are persistent grids that stride over the counts they read from
// device memory, so the host never waits for queue sizes.
//
// Records (bytes): ray 32 (org+tmin, dir+slot), hit 8 (t, primitive), path state
// 48 (beta+parent pdf, emission weight+light-estimate sum, parent normal+flags),
// shadow 48 (org+dist, dir+slot, contribution). Radiance accumulates in the
// per-sample output buffer that the accumulation kernel reads afterwards.
#include <algorithm>

#include "pg3_estimator.cuh"
#include "pg3_kernels.h"

namespace pg3 {

namespace {

constexpr int kWaveBlock = 256;
enum : int { kBucketMiss = 0, kBucketLambert = 1, kBucketConductor = 2, kBucketDielectric = 3, kNumBuckets = 4 };
constexpr uint32_t kFlagFinite = 1u << 16, kFlagRefl = 1u << 17;

struct Counters {
    uint32_t ray[2];
    uint32_t bucket[kNumBuckets];
    uint32_t shadow;
    uint32_t pad;
};

struct Queues {
    float4 *ray[2];           // 2 float4 per entry
    float2 *hit;              // (t, primitive as int bits)
    uint32_t *bucket[kNumBuckets];
    float4 *beta;             // beta.xyz, parent bsdf pdf
    float4 *ew;               // emission weight.xyz, parent light-estimate sum
    float4 *pn;               // parent normal.xyz, flags (path length | finite | compute-reflected)
    float4 *shadow;           // 3 float4 per record
    Counters *cnt;
};

// Warp-aggregated append: lanes with `want` get consecutive slots of *counter.
__device__ __forceinline__ uint32_t warpAppend(uint32_t *counter, bool want)
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

__device__ __forceinline__ void countWarp(unsigned long long *dst, uint32_t v)
{
    const uint32_t s = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(dst, (unsigned long long)s);
}

__global__ void __launch_bounds__(kWaveBlock) raygenKernel(const __grid_constant__ SceneView S, Queues Q,
                                                           uint64_t base, uint32_t count, uint32_t npix,
                                                           uint32_t sample0, float *outR, float *outG, float *outB,
                                                           DevStats *stats)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint64_t g = base + i;
        const uint32_t pixel = (uint32_t)(g % npix), sample = sample0 + (uint32_t)(g / npix);
        const uint32_t px = pixel % S.width, py = pixel / S.width;
        const Rand4 rc = draw(S, pixel, sample, 0, 0);
        const float nx = ((float)px + rc.a) * (2.f / S.width) - 1.f;
        const float ny = ((float)py + rc.b) * (2.f / S.height) - 1.f;
        const float3 dir = normalize(S.camFwd + S.camRight * (nx * S.tanX) - S.camUp * (ny * S.tanY));
        Q.ray[0][2 * i] = make_float4(S.camPos.x, S.camPos.y, S.camPos.z, 0.f);
        Q.ray[0][2 * i + 1] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(i));
        Q.beta[i] = make_float4(1.f, 1.f, 1.f, 0.f);
        Q.ew[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        Q.pn[i] = make_float4(0.f, 0.f, 1.f, __uint_as_float(1u | kFlagFinite | kFlagRefl));
        outR[i] = 0.f;
        outG[i] = 0.f;
        outB[i] = 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Q.cnt->ray[0] = count;
        atomicAdd(&stats->paths, (unsigned long long)count);
    }
}

__global__ void __launch_bounds__(kWaveBlock) extendKernel(const __grid_constant__ SceneView S, Queues Q, int cur,
                                                           DevStats *stats)
{
    const uint32_t n = Q.cnt->ray[cur];
    const float4 *rq = Q.ray[cur];
    uint32_t rays = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool active = i < n;
        int bucket = -1;
        if (active) {
            const float4 r0 = rq[2 * i], r1 = rq[2 * i + 1];
            Hit h;
            const bool hit = intersectClosest(S, xyz(r0), xyz(r1), r0.w, h);
            Q.hit[i] = make_float2(h.t, __int_as_float(h.prim));
            if (!hit) bucket = kBucketMiss;
            else {
                const int mat = ((uint32_t)h.prim < S.ntri) ? __ldg(&S.triMat[h.prim]) : __ldg(&S.sphMat[h.prim - S.ntri]);
                bucket = 1 + __ldg(&S.mats[mat].kind);
            }
            ++rays;
        }
#pragma unroll
        for (int b = 0; b < kNumBuckets; ++b) {
            const uint32_t pos = warpAppend(&Q.cnt->bucket[b], bucket == b);
            if (bucket == b) Q.bucket[b][pos] = i;
        }
    }
    countWarp(&stats->extRays, rays);
}

struct ShadeOut {
    bool shadow = false, next = false;
    float4 s0, s1, s2;        // shadow record
    float4 r0, r1;            // next ray
};

// Resident blocks per SM the shade kernels are compiled for (register budget 65536 / (256 x N)).
#ifndef PG3_SHADE_MIN_BLOCKS
#define PG3_SHADE_MIN_BLOCKS 2
#endif

template <int K, int EMK>
__global__ void __launch_bounds__(kWaveBlock, PG3_SHADE_MIN_BLOCKS) shadeKernel(const __grid_constant__ SceneView S, Queues Q, int cur,
                                                          uint64_t base0, uint32_t npix, uint32_t sample0,
                                                          float *outR, float *outG, float *outB, DevStats *stats)
{
    constexpr int kBucket = (K < 0) ? kBucketMiss : 1 + K;
    const uint32_t n = Q.cnt->bucket[kBucket];
    const float4 *rq = Q.ray[cur];
    float4 *nq = Q.ray[cur ^ 1];
    PathCounters pc;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        const bool active = j < n;
        ShadeOut o;
        uint32_t slot = 0;
        if (active) {
            const uint32_t idx = Q.bucket[kBucket][j];
            const float4 r0 = rq[2 * idx], r1 = rq[2 * idx + 1];
            const float3 org = xyz(r0), dir = xyz(r1);
            slot = __float_as_uint(r1.w);
            const float4 sb = Q.beta[slot], se = Q.ew[slot], sn = Q.pn[slot];
            const uint32_t flags = __float_as_uint(sn.w);
            const uint32_t pl = flags & 0xffffu;
            const bool prevFinite = (flags & kFlagFinite) != 0, computeRefl = (flags & kFlagRefl) != 0;
            const float3 beta = xyz(sb), ew = xyz(se), prevN = xyz(sn);
            const float prevBsdfPdf = sb.w, prevSum = se.w;
            float3 L = f3(0.f);
            if (K < 0) {
                // background (src/path_tracer.hxx:408-429)
                if (pl >= S.minPL && S.bgKind != kBgNone) {
                    float pdf = 0.f;
                    const Frame pf = frameFromZ(prevN);
                    const float3 Le = bgEmission<EMK>(S, dir, pl > 1 && prevFinite, pf, pdf);
                    if (pl == 1) L = Le;
                    else if (prevFinite) L = ew * Le * misPower(prevBsdfPdf, pdf * pickProb(S, org, prevN, prevSum, S.bgLightId));
                    else L = ew * Le;
                }
                if (computeRefl) ++pc.bg;
            } else {
                const float2 hh = Q.hit[idx];
                Hit h;
                h.t = hh.x;
                h.prim = __float_as_int(hh.y);
                float3 pt, nrm;
                int matId;
                hitAttributes(S, h, org, dir, pt, nrm, matId);
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
                if (go) {
                    const uint64_t g = base0 + slot;
                    const uint32_t pixel = (uint32_t)(g % npix), sample = sample0 + (uint32_t)(g / npix);
                    const Rand4 ra = draw(S, pixel, sample, pl, 0);
                    const Rand4 rb = draw(S, pixel, sample, pl, 1);
                    const float sum = (S.lightCount > 1) ? estimateSum(S, pt, nrm) : 0.f;
                    if (pl + 1 >= S.minPL) {
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
                                areaSample(S.lights[lid], pt, nrm, ra.b, ra.c, wig, dist, smp, pdfW);
                            }
                            if (maxc(smp) > 0.f) {
                                BsdfRec br;
                                evalBsdfK<K>(mat, toLocal(frame, wig), wol, br);
                                const float lightPdf = pdfW * lprob;
                                const float3 c = beta * (smp * br.att) * (misPower(lightPdf, br.pdfW * br.compProb) / lightPdf);
                                o.shadow = true;
                                o.s0 = make_float4(pt.x, pt.y, pt.z, dist);
                                o.s1 = make_float4(wig.x, wig.y, wig.z, __uint_as_float(slot));
                                o.s2 = make_float4(c.x, c.y, c.z, 0.f);
                            }
                        }
                    }
                    float rrProb = 1.0f;
                    bool cut = false;
                    if (S.maxPL == 0 || (S.rrMinPL > 0 && pl >= S.rrMinPL)) {
                        rrProb = mat.rrProb;
                        cut = rb.a > rrProb;
                    }
                    BsdfRec br;
                    sampleBsdfK<K>(mat, wol, rb.b, rb.c, rb.d, br);
                    if (isBlocker(br)) {
                        ++pc.blocker;
                    } else {
                        const bool finite = br.pdfW != infF();
                        const float cosAbs = fabsf(br.wil.z);
                        const float3 f = finite ? br.att * (cosAbs / (br.pdfW * br.compProb)) : br.att / br.compProb;
                        const float3 ew2 = beta * f;
                        const float3 beta2 = ew2 / rrProb;
                        if (cut) ++pc.rr;
                        Q.beta[slot] = make_float4(beta2.x, beta2.y, beta2.z, br.pdfW * br.compProb);
                        Q.ew[slot] = make_float4(ew2.x, ew2.y, ew2.z, sum);
                        const uint32_t nf = (pl + 1) | (finite ? kFlagFinite : 0u) | (cut ? 0u : kFlagRefl);
                        Q.pn[slot] = make_float4(nrm.x, nrm.y, nrm.z, __uint_as_float(nf));
                        const float3 nd = toWorld(frame, br.wil);
                        o.next = true;
                        o.r0 = make_float4(pt.x, pt.y, pt.z, epsRayCos(cosAbs));
                        o.r1 = make_float4(nd.x, nd.y, nd.z, __uint_as_float(slot));
                    }
                }
            }
            if (!isZero(L)) {
                outR[slot] += L.x;
                outG[slot] += L.y;
                outB[slot] += L.z;
            }
        }
        const uint32_t sp = warpAppend(&Q.cnt->shadow, o.shadow);
        if (o.shadow) {
            Q.shadow[3 * sp] = o.s0;
            Q.shadow[3 * sp + 1] = o.s1;
            Q.shadow[3 * sp + 2] = o.s2;
        }
        const uint32_t rp = warpAppend(&Q.cnt->ray[cur ^ 1], o.next);
        if (o.next) {
            nq[2 * rp] = o.r0;
            nq[2 * rp + 1] = o.r1;
        }
    }
    countWarp(&stats->byBackground, pc.bg);
    countWarp(&stats->byBlocker, pc.blocker);
    countWarp(&stats->byMax, pc.maxl);
    countWarp(&stats->bySafety, pc.safety);
    countWarp(&stats->byRR, pc.rr);
}

__global__ void __launch_bounds__(kWaveBlock) shadowKernel(const __grid_constant__ SceneView S, Queues Q,
                                                           float *outR, float *outG, float *outB, DevStats *stats)
{
    const uint32_t n = Q.cnt->shadow;
    uint32_t cnt = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        if (j < n) {
            const float4 s0 = Q.shadow[3 * j], s1 = Q.shadow[3 * j + 1];
            ++cnt;
            if (!occludedAny(S, xyz(s0), xyz(s1), s0.w)) {
                const float4 c = Q.shadow[3 * j + 2];
                const uint32_t slot = __float_as_uint(s1.w);
                outR[slot] += c.x;
                outG[slot] += c.y;
                outB[slot] += c.z;
            }
        }
    }
    countWarp(&stats->shadowRays, cnt);
}

__global__ void advanceKernel(Counters *c, int cur)
{
    c->ray[cur] = 0;
    for (int b = 0; b < kNumBuckets; ++b) c->bucket[b] = 0;
    c->shadow = 0;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

Queues carve(void *scratch, uint64_t cap)
{
    char *p = reinterpret_cast<char *>(scratch);
    Queues q;
    auto take = [&](size_t bytes) { char *r = p; p += align256(bytes); return r; };
    q.cnt = (Counters *)take(sizeof(Counters));
    q.ray[0] = (float4 *)take(32 * cap);
    q.ray[1] = (float4 *)take(32 * cap);
    q.hit = (float2 *)take(8 * cap);
    for (int b = 0; b < kNumBuckets; ++b) q.bucket[b] = (uint32_t *)take(4 * cap);
    q.beta = (float4 *)take(16 * cap);
    q.ew = (float4 *)take(16 * cap);
    q.pn = (float4 *)take(16 * cap);
    q.shadow = (float4 *)take(48 * cap);
    return q;
}

}  // namespace

// The four shade kernels of one bounce, specialised on the environment-map sampler.
template <int EMK>
void launchShade(const SceneView &S, const Queues &Q, int cur, uint64_t base, uint32_t npix, uint32_t sample0,
                 float *r, float *g, float *b, DevStats *stats, int grid, cudaStream_t st)
{
    shadeKernel<-1, EMK><<<grid, kWaveBlock, 0, st>>>(S, Q, cur, base, npix, sample0, r, g, b, stats);
    shadeKernel<kMatLambert, EMK><<<grid, kWaveBlock, 0, st>>>(S, Q, cur, base, npix, sample0, r, g, b, stats);
    shadeKernel<kMatGgxConductor, EMK><<<grid, kWaveBlock, 0, st>>>(S, Q, cur, base, npix, sample0, r, g, b, stats);
    shadeKernel<kMatGgxDielectric, EMK><<<grid, kWaveBlock, 0, st>>>(S, Q, cur, base, npix, sample0, r, g, b, stats);
}

size_t wavefrontBytes(uint64_t cap)
{
    return align256(sizeof(Counters)) + 2 * align256(32 * cap) + align256(8 * cap) + kNumBuckets * align256(4 * cap) +
           3 * align256(16 * cap) + align256(48 * cap);
}

cudaError_t launchWavefront(const SceneView &S, bool naive, uint32_t sample0, uint64_t numPaths, uint32_t npix,
                            float *outR, float *outG, float *outB, DevStats *stats, void *scratch, uint64_t capacity,
                            int gridBlocks, cudaStream_t stream, uint64_t *launches)
{
    if (naive) return cudaErrorNotSupported;   // the BSDF-only tracer runs as a megakernel
    Queues Q = carve(scratch, capacity);
    const uint32_t maxBounces = S.maxPL > 0 ? S.maxPL : kMaxPathLengthHard;
    for (uint64_t base = 0; base < numPaths; base += capacity) {
        const uint32_t count = (uint32_t)std::min<uint64_t>(capacity, numPaths - base);
        float *r = outR + base, *g = outG + base, *b = outB + base;
        cudaMemsetAsync(Q.cnt, 0, sizeof(Counters), stream);
        const int gen = (int)std::min<uint64_t>((count + kWaveBlock - 1) / kWaveBlock, (uint64_t)gridBlocks * 4);
        raygenKernel<<<gen, kWaveBlock, 0, stream>>>(S, Q, base, count, npix, sample0, r, g, b, stats);
        *launches += 1;
        for (uint32_t bounce = 0; bounce < maxBounces; ++bounce) {
            const int cur = bounce & 1;
            extendKernel<<<gridBlocks, kWaveBlock, 0, stream>>>(S, Q, cur, stats);
            const int emk = (S.bgKind == kBgEnvMap) ? S.emSampler : kEmCosine;   // no map: constant/area paths
            if (emk == kEmCdf) launchShade<kEmCdf>(S, Q, cur, base, npix, sample0, r, g, b, stats, gridBlocks, stream);
            else if (emk == kEmSteerable)
                launchShade<kEmSteerable>(S, Q, cur, base, npix, sample0, r, g, b, stats, gridBlocks, stream);
            else launchShade<kEmCosine>(S, Q, cur, base, npix, sample0, r, g, b, stats, gridBlocks, stream);
            shadowKernel<<<gridBlocks, kWaveBlock, 0, stream>>>(S, Q, r, g, b, stats);
            advanceKernel<<<1, 1, 0, stream>>>(Q.cnt, cur);
            *launches += 7;
            if (S.maxPL == 0 && (bounce & 7) == 7) {
                // roulette-ended paths: stop once the queue is empty (checked every 8 bounces)
                uint32_t left = 0;
                cudaMemcpyAsync(&left, &Q.cnt->ray[cur ^ 1], sizeof left, cudaMemcpyDeviceToHost, stream);
                cudaStreamSynchronize(stream);
                if (left == 0) break;
            }
        }
    }
    return cudaGetLastError();
}


}  // namespace pg3
