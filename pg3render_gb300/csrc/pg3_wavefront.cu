// Wavefront pipeline: the path estimator of pg3_estimator.cuh split into stage
// kernels that communicate through structure-of-arrays queues in HBM/L2.
//
// Per launch chunk (up to `capacity` paths, one slot per path):
//   raygen            camera rays of all slots -> ray queue A; path state init
//   per bounce:
//     extend          closest hit of every queued ray; the ray's queue index is
//                     appended to one of six buckets (miss, Lambert, GGX
//                     conductor, GGX dielectric, Phong, smooth conductor or
//                     dielectric) with warp-aggregated atomics
//     shade<kind>     one kernel per bucket (kinds the scene has): emitter MIS,
//                     light sample (the BSDF
//                     value and MIS weight are folded into a shadow record),
//                     Russian roulette, BSDF sample -> next ray queue
//     shadow          any-hit test of every shadow record; unoccluded records
//                     add their contribution to the path's radiance
// The counters a bounce has consumed are reset by the next stage that no longer reads them:
// shadow zeroes the ray queue's and the buckets' counters, the next extend the shadow counter.
// Each stage kernel holds only its own material's code, which keeps it inside
// the instruction cache, and a warp shades hits of one material kind only.
// Launches are persistent grids that stride over the counts they read from
// device memory, so the host never waits for queue sizes.
//
// Records (bytes): ray 32 (org+tmin, dir+slot), hit 8 (t, primitive), path state
// 48 (beta+parent pdf, emission weight+light-estimate sum, parent normal+flags),
// shadow 48 (org+dist, dir+slot, contribution). Radiance accumulates in the
// per-sample output buffer that the accumulation kernel reads afterwards.
//
// The GRAD instantiations run the path-replay adjoint (pg3_wave.cuh): the same
// stages with 80-byte shadow records and an 8-byte per-slot pending-gradient word.
#include <algorithm>

#include "pg3_kernels.h"
#include "pg3_wave.cuh"

namespace pg3 {

namespace {

// Programmatic dependent launch between the stage kernels of a bounce: each stage kernel is
// launched while its predecessor drains, its blocks wait in griddepcontrol.wait until the
// predecessor has completed and its writes are visible, and only then let their own successor
// launch. The launch latency and block start-up of ~97 launches per chunk overlap the tail
// of the previous kernel. griddepcontrol.wait is a no-op in a kernel launched without the
// attribute, so every other launch path of these kernels is unchanged.
#ifndef PG3_PDL
#define PG3_PDL 1
#endif

PG3_DI void stageEntry()
{
#if PG3_PDL
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

template <typename... Params, typename... Args>
void launchStage(bool pdl, void (*kernel)(Params...), int grid, int threads, size_t smem, cudaStream_t st,
                 Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = (PG3_PDL && pdl) ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

// The first bounce's shade kernels take the camera paths' initial state from registers instead of
// the state queue, so raygen writes no state (48 bytes per path less to write and to read).
#ifndef PG3_FIRST_STATE_CONST
#define PG3_FIRST_STATE_CONST 1
#endif

// The first sample index of a launch: sample0, plus a device word when one is given (a captured
// graph replays with a new word: a differentiable-rendering graph, a per-call render graph).
template <bool GRAD>
PG3_DI uint32_t sampleBase(uint32_t sample0, const GradArgs &G)
{
    return G.sampleOffset ? sample0 + *G.sampleOffset : sample0;
}

template <bool GRAD>
__global__ void __launch_bounds__(kWaveBlock) raygenKernel(const __grid_constant__ SceneView S, Queues Q,
                                                           uint64_t base, uint32_t count, uint32_t npix,
                                                           uint32_t sample0, float *outR, float *outG, float *outB,
                                                           DevStats *stats, GradArgs G)
{
    stageEntry();
    sample0 = sampleBase<GRAD>(sample0, G);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint64_t g = base + i;
        const uint32_t pixel = (uint32_t)(g % npix), sample = sample0 + (uint32_t)(g / npix);
        float3 dir;
        cameraRay(S, pixel, sample, dir);
        Q.ray[0][2 * i] = make_float4(S.camPos.x, S.camPos.y, S.camPos.z, 0.f);
        Q.ray[0][2 * i + 1] = make_float4(dir.x, dir.y, dir.z, __uint_as_float(i));
        // (no path state: the first bounce's shade kernels start from the initial one)
#if !PG3_FIRST_STATE_CONST
        initPathState(Q, 0, i);
#endif
        if (GRAD) Q.pend[i] = make_float2(__int_as_float(-1), 0.f);
        outR[i] = 0.f;
        outG[i] = 0.f;
        outB[i] = 0.f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Q.cnt->ray[0] = count;
        atomicAdd(&stats->paths, (unsigned long long)count);
    }
}

// Resident blocks per SM the ray-query kernels (extend, shadow) are compiled and launched for:
// their few registers allow more warps than the shade kernels' grid provides.
#ifndef PG3_QUERY_MIN_BLOCKS
#define PG3_QUERY_MIN_BLOCKS 6
#endif
// ... for the binary LBVH (5: its traversal stack and node boxes fit 48 registers without spill),
// and for the 4-wide BVH, whose node records and sorted children need more registers
#ifndef PG3_LBVH_QUERY_MIN_BLOCKS
#define PG3_LBVH_QUERY_MIN_BLOCKS 5
#endif
#ifndef PG3_BVH4_QUERY_MIN_BLOCKS
#define PG3_BVH4_QUERY_MIN_BLOCKS 4
#endif
// TRAV: 0 the primitive list, 1 the binary LBVH, 2 the 4-wide BVH (SceneView::useBvh)
constexpr int queryMinBlocks(int TRAV)
{
    return TRAV == 0 ? PG3_QUERY_MIN_BLOCKS : TRAV == 1 ? PG3_LBVH_QUERY_MIN_BLOCKS : PG3_BVH4_QUERY_MIN_BLOCKS;
}

template <int TRAV>
__global__ void __launch_bounds__(kWaveBlock, queryMinBlocks(TRAV)) extendKernel(const __grid_constant__ SceneView S, Queues Q, int cur,
                                                           DevStats *stats)
{
    stageEntry();
    // the previous bounce's shadow records are consumed: its counter starts the new bounce at zero
    // (no stage reads or appends shadow records while rays are extended)
    if (blockIdx.x == 0 && threadIdx.x == 0) Q.cnt->shadow = 0;
    const uint32_t n = Q.cnt->ray[cur];
    const float4 *rq = rayQ(Q, cur);
    uint32_t rays = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        int bucket = -1;
        if (i < n) {
            if (i + stride < n) {   // the next iteration's ray, while this one is traced
                prefetchL1(rq + 2 * (size_t)(i + stride));
                prefetchL1(rq + 2 * (size_t)(i + stride) + 1);
            }
            bucket = extendOne<TRAV>(S, Q, rq, i);
            ++rays;
        }
        bucketAppend(Q, bucket, i);
    }
    countWarp(&stats->extRays, rays);
}

// Block shape each shade kernel of the render paths is compiled and launched for: threads per
// block and resident blocks per SM (register budget 65536 / (threads x blocks), taken per quarter
// SM: 17-20 warps per SM leave 96 registers a thread, 16 leave 128). The material kernels take
// 256 x 2 (128 registers; at 96 the conductor and dielectric spill about 100 bytes and ran 0.6%
// slower). The Lambert kernel fits 96 registers with at most 4 bytes of spill: 128 x 5 keeps 20
// warps per SM where 256-thread blocks hold 16, faster with the steerable and CDF samplers and
// slower with the cosine sampler, which keeps 256 x 2. The miss (background) kernel, which holds
// no material code, takes 128 x 9 (36 warps, 56 registers, at most 12 bytes of spill; 256 x 4
// held 32). The gradient instantiations keep 256 x 2 and 256 x 4 for the miss kernel: with the
// adjoint's sums the Lambert kernel spills over 100 bytes at 96 registers.
#ifndef PG3_SHADE_MIN_BLOCKS
#define PG3_SHADE_MIN_BLOCKS 2
#endif
#ifndef PG3_MISS_MIN_BLOCKS
#define PG3_MISS_MIN_BLOCKS 9
#endif
#ifndef PG3_LAMBERT_THREADS
#define PG3_LAMBERT_THREADS 128
#endif
#ifndef PG3_LAMBERT_MIN_BLOCKS
#define PG3_LAMBERT_MIN_BLOCKS 5
#endif
#ifndef PG3_CONDUCTOR_MIN_BLOCKS
#define PG3_CONDUCTOR_MIN_BLOCKS PG3_SHADE_MIN_BLOCKS
#endif
#ifndef PG3_DIELECTRIC_MIN_BLOCKS
#define PG3_DIELECTRIC_MIN_BLOCKS PG3_SHADE_MIN_BLOCKS
#endif
#ifndef PG3_CONDUCTOR_THREADS
#define PG3_CONDUCTOR_THREADS 256
#endif
#ifndef PG3_DIELECTRIC_THREADS
#define PG3_DIELECTRIC_THREADS 256
#endif
#ifndef PG3_MISS_THREADS
#define PG3_MISS_THREADS 128
#endif
constexpr bool lambertShape(int K, int EMK, bool GRAD) { return K == kMatLambert && EMK != kEmCosine && !GRAD; }
constexpr int shadeThreads(int K, int EMK, bool GRAD)
{
    return lambertShape(K, EMK, GRAD) ? PG3_LAMBERT_THREADS
           : GRAD ? kWaveBlock
           : K < 0 ? PG3_MISS_THREADS
           : K == kMatGgxConductor ? PG3_CONDUCTOR_THREADS
           : K == kMatGgxDielectric ? PG3_DIELECTRIC_THREADS : kWaveBlock;
}
constexpr int shadeMinBlocks(int K, int EMK, bool GRAD)
{
    return GRAD                          ? (K < 0 ? 4 : 2)   // 256-thread blocks: 64 / 128 registers
           : K < 0                       ? PG3_MISS_MIN_BLOCKS
           : lambertShape(K, EMK, GRAD)  ? PG3_LAMBERT_MIN_BLOCKS
           : K == kMatLambert         ? PG3_SHADE_MIN_BLOCKS
           : K == kMatGgxConductor    ? PG3_CONDUCTOR_MIN_BLOCKS
           : K == kMatGgxDielectric   ? PG3_DIELECTRIC_MIN_BLOCKS
                                      : PG3_SHADE_MIN_BLOCKS;
}

// Path lengths of this launch's terminations into the histogram of the reference's introspection
// data (RendererIntrospectionData::AddCorePathLength, src/renderer.hxx:80-118: bins of
// floor(log2(length + 1)), the safety limit left out). Every path of a bounce has the same length.
PG3_DI void countLengths(DevStats *st, uint32_t len, uint32_t n)
{
    const uint32_t s = __reduce_add_sync(0xffffffffu, n);
    if ((threadIdx.x & 31) == 0 && s) {
        const int bin = min(31 - __clz(len + 1), kLenBins - 1);
        atomicAdd(&st->lenHist[bin], (unsigned long long)s);
        atomicMax(&st->minLenC, ~len);
        atomicMax(&st->maxLen, len);
    }
}

// pathLen: the length of the paths whose vertices this bounce shades (bounce + 1)
template <int K, int EMK, bool GRAD>
__global__ void __launch_bounds__(shadeThreads(K, EMK, GRAD), shadeMinBlocks(K, EMK, GRAD))
    shadeKernel(const __grid_constant__ SceneView S, Queues Q, int cur, uint32_t base0, uint32_t npix,
                uint32_t sample0, float *outR, float *outG, float *outB, DevStats *stats, GradArgs G,
                uint32_t pathLen)
{
    extern __shared__ float sGrad[];
    // the block's gradient sums read nothing the previous stage writes: cleared before the wait
    initBlockGrad<GRAD>(sGrad, S.nmat);
    stageEntry();
    sample0 = sampleBase<GRAD>(sample0, G);
    constexpr int kBucket = bucketOfShade(K);
    const uint32_t n = Q.cnt->bucket[kBucket];
    const float4 *rq = rayQ(Q, cur);
    const uint32_t stride = gridDim.x * blockDim.x;
    PathCounters pc;
    // the bucket entry of the next iteration is loaded one iteration ahead
    uint32_t nextIdx = (blockIdx.x * blockDim.x + threadIdx.x < n) ? Q.bucket[kBucket][blockIdx.x * blockDim.x + threadIdx.x] : 0u;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t j = base + threadIdx.x;
        ShadeOut o;
        if (j < n) {
            const uint32_t idx = nextIdx;
            NextEntry nx;
            const bool first = PG3_FIRST_STATE_CONST && pathLen == 1;   // camera rays: the initial state
            if (j + stride < n) {
                nextIdx = Q.bucket[kBucket][j + stride];
                nx.ray = rq + 2 * (size_t)nextIdx;
                nx.hit = Q.hit + nextIdx;
                nx.st = first ? nullptr : stQ(Q, cur) + 3 * (size_t)nextIdx;
            }
            float4 st0[3];
            const float4 *stp = stQ(Q, cur) + 3 * (size_t)idx;
            if (first) {
                initialPathState(st0);
                stp = st0;
            }
            const float4 r0 = rq[2 * idx], r1 = rq[2 * idx + 1];
            const uint32_t slot = __float_as_uint(r1.w) & kSlotMask;
            const uint32_t g = base0 + slot;
            const uint32_t pixel = g % npix, sample = sample0 + g / npix;
            float3 acc = f3(0.f);
            if (GRAD && G.adjoint) acc = make_float3(outR[slot], outG[slot], outB[slot]);
            float3 L;
            shadeVertex<K, EMK, GRAD>(S, Q, idx, r0, r1, stp, slot, slot, pixel, sample, pc, o, L, G, sGrad, acc, nx);
            if (!isZero(L)) {
                outR[slot] += L.x;
                outG[slot] += L.y;
                outB[slot] += L.z;
            }
        }
        emitRecords<GRAD>(Q, cur ^ 1, o);
    }
    countWarp(&stats->byBackground, pc.bg);
    countWarp(&stats->byBlocker, pc.blocker);
    countWarp(&stats->byMax, pc.maxl);
    countWarp(&stats->bySafety, pc.safety);
    countWarp(&stats->byRR, pc.rr);
    // a path leaving to the background has the length of its last vertex (src/path_tracer.hxx:428)
    countLengths(stats, K < 0 ? pathLen - 1 : pathLen, pc.rr + pc.bg + pc.blocker + pc.maxl);
    flushBlockGrad<GRAD>(sGrad, S.nmat, G.gMat);
}

template <bool GRAD, int TRAV>
__global__ void __launch_bounds__(kWaveBlock, queryMinBlocks(TRAV)) shadowKernel(const __grid_constant__ SceneView S, Queues Q,
                                                           int cur, float *outR, float *outG, float *outB,
                                                           DevStats *stats, GradArgs G)
{
    constexpr int SW = kShadowWords<GRAD>;
    extern __shared__ float sGrad[];
    initBlockGrad<GRAD>(sGrad, S.nmat);   // before the wait: reads nothing the shade stage writes
    stageEntry();
    // this bounce's ray queue and buckets are consumed (extend and the shade kernels have
    // completed): their counters start at zero for the next bounce's appends. No stage of the
    // shadow pass reads them.
    if (blockIdx.x == 0 && threadIdx.x < 1 + kNumBuckets) {
        if (threadIdx.x == 0) Q.cnt->ray[cur] = 0;
        else Q.cnt->bucket[threadIdx.x - 1] = 0;
    }
    const uint32_t n = Q.cnt->shadow;
    uint32_t cnt = 0;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t j = base + threadIdx.x;
        if (j < n) {
            const float4 *rec = Q.shadow + (size_t)SW * j;
            if (j + stride < n) {   // the next iteration's record, while this ray is tested
                const float4 *nr = Q.shadow + (size_t)SW * (j + stride);
                prefetchL1(nr);
                prefetchL1(nr + 1);
                prefetchL1(nr + 2);
            }
            const float4 s0 = rec[0], s1 = rec[1];
            ++cnt;
            if (!occludedAny<TRAV>(S, xyz(s0), xyz(s1), s0.w)) {
                const float4 c = rec[2];
                const uint32_t slot = __float_as_uint(s1.w) & kSlotMask;
                outR[slot] += c.x;
                outG[slot] += c.y;
                outB[slot] += c.z;
                shadowGrad<GRAD>(S, rec, xyz(s1), G, sGrad);
            }
        }
    }
    countWarp(&stats->shadowRays, cnt);
    flushBlockGrad<GRAD>(sGrad, S.nmat, G.gMat);
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

Queues carve(void *scratch, uint64_t cap, bool grad)
{
    char *p = reinterpret_cast<char *>(scratch);
    Queues q;
    auto take = [&](size_t bytes) { char *r = p; p += align256(bytes); return r; };
    q.cnt = (Counters *)take(sizeof(Counters));
    q.ray[0] = (float4 *)take(32 * cap);
    q.ray[1] = (float4 *)take(32 * cap);
    q.hit = (float2 *)take(8 * cap);
    for (int b = 0; b < kNumBuckets; ++b) q.bucket[b] = (uint32_t *)take(4 * cap);
    q.bucketStride = align256(4 * cap) / 4;
    q.st[0] = (float4 *)take(48 * cap);
    q.st[1] = (float4 *)take(48 * cap);
    q.shadow = (float4 *)take((grad ? 80 : 48) * cap);
    q.pend = grad ? (float2 *)take(8 * cap) : nullptr;
    q.cap = (uint32_t)cap;
    q.err = nullptr;
    return q;
}

// One shade kernel: grid = SMs x 1024 / kWaveBlock on entry; the kernel gets PG3_SHADE_WAVES waves
// of the blocks it is compiled to keep resident per SM.
#ifndef PG3_SHADE_WAVES
#define PG3_SHADE_WAVES 1
#endif
template <int K, int EMK, bool GRAD>
void launchShadeKind(const SceneView &S, const Queues &Q, int cur, uint32_t base, uint32_t npix, uint32_t sample0,
                     float *r, float *g, float *b, DevStats *stats, int grid, size_t smem, const GradArgs &G,
                     cudaStream_t st, bool pdl, int &launched, uint32_t pathLen)
{
    const int blocks = std::max(1, grid / (1024 / kWaveBlock)) * PG3_SHADE_WAVES * shadeMinBlocks(K, EMK, GRAD);
    launchStage(pdl, shadeKernel<K, EMK, GRAD>, blocks, shadeThreads(K, EMK, GRAD), smem, st, S, Q, cur, base, npix, sample0, r, g, b, stats, G,
                pathLen);
    ++launched;
}

// The shade kernels of one bounce (the miss bucket and the material kinds of the scene),
// specialised on the environment-map sampler. Returns the number of launches.
template <int EMK, bool GRAD>
int launchShade(const SceneView &S, uint32_t kindMask, const Queues &Q, int cur, uint32_t base, uint32_t npix,
                uint32_t sample0, float *r, float *g, float *b, DevStats *stats, int grid, size_t smem,
                const GradArgs &G, cudaStream_t st, bool pdl, uint32_t pathLen)
{
    int n = 0;
    launchShadeKind<-1, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    if (kindMask & (1u << kMatLambert))
        launchShadeKind<kMatLambert, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    if (kindMask & (1u << kMatGgxConductor))
        launchShadeKind<kMatGgxConductor, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    if (kindMask & (1u << kMatGgxDielectric))
        launchShadeKind<kMatGgxDielectric, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    if (kindMask & (1u << kMatPhong))
        launchShadeKind<kMatPhong, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    if (kindMask & ((1u << kMatSmoothConductor) | (1u << kMatSmoothDielectric)))
        launchShadeKind<kShadeSmooth, EMK, GRAD>(S, Q, cur, base, npix, sample0, r, g, b, stats, grid, smem, G, st, pdl, n, pathLen);
    return n;
}

template <bool GRAD>
cudaError_t runWavefront(const SceneView &S, uint32_t kindMask, uint32_t sample0, uint64_t numPaths, uint32_t npix, float *outR,
                         float *outG, float *outB, DevStats *stats, void *scratch, uint64_t capacity, int gridBlocks,
                         cudaStream_t stream, uint64_t *launches, const GradArgs &G0, bool pdlInCapture = false)
{
    Queues Q = carve(scratch, capacity, GRAD);
    Q.err = S.errorFlag;
    const uint32_t maxBounces = S.maxPL > 0 ? S.maxPL : kMaxPathLengthHard;
    // (gridBlocks is SMs x the shade kernels' 1024 threads per SM)
    const int trav = S.useBvh;
    const int queryGrid = std::max(1, gridBlocks / (1024 / kWaveBlock)) *
                          (trav == 2 ? queryMinBlocks(2) : trav == 1 ? queryMinBlocks(1) : queryMinBlocks(0));
    const size_t smem = GRAD ? 16 * (size_t)S.nmat : 0;
    cudaStreamCaptureStatus capturing = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(stream, &capturing);
    for (uint64_t base = 0; base < numPaths; base += capacity) {
        const uint32_t count = (uint32_t)std::min<uint64_t>(capacity, numPaths - base);
        float *r = outR + base, *g = outG + base, *b = outB + base;
        GradArgs G = G0;
        if (GRAD && G.adjoint) {
            G.totR += base;
            G.totG += base;
            G.totB += base;
        }
        cudaMemsetAsync(Q.cnt, 0, sizeof(Counters), stream);
        const int gen = (int)std::min<uint64_t>((count + kWaveBlock - 1) / kWaveBlock, (uint64_t)gridBlocks * 4);
        raygenKernel<GRAD><<<gen, kWaveBlock, 0, stream>>>(S, Q, base, count, npix, sample0, r, g, b, stats, G);
        *launches += 1;
        for (uint32_t bounce = 0; bounce < maxBounces; ++bounce) {
            const int cur = bounce & 1;
            const bool pdl = capturing == cudaStreamCaptureStatusNone || pdlInCapture;
            if (trav == 2) launchStage(pdl, extendKernel<2>, queryGrid, kWaveBlock, 0, stream, S, Q, cur, stats);
            else if (trav == 1) launchStage(pdl, extendKernel<1>, queryGrid, kWaveBlock, 0, stream, S, Q, cur, stats);
            else launchStage(pdl, extendKernel<0>, queryGrid, kWaveBlock, 0, stream, S, Q, cur, stats);
            const int emk = (S.bgKind == kBgEnvMap) ? S.emSampler : kEmCosine;   // no map: constant/area paths
            const uint32_t b32 = (uint32_t)base;
            int shades;
            if (emk == kEmCdf)
                shades = launchShade<kEmCdf, GRAD>(S, kindMask, Q, cur, b32, npix, sample0, r, g, b, stats, gridBlocks, smem, G, stream, pdl,
                                                                  bounce + 1);
            else if (emk == kEmSteerable)
                shades = launchShade<kEmSteerable, GRAD>(S, kindMask, Q, cur, b32, npix, sample0, r, g, b, stats, gridBlocks, smem, G, stream, pdl,
                                                                  bounce + 1);
            else if (emk == kEmSteerableAdaptive)
                shades = launchShade<kEmSteerableAdaptive, GRAD>(S, kindMask, Q, cur, b32, npix, sample0, r, g, b, stats, gridBlocks, smem, G, stream, pdl,
                                                                  bounce + 1);
            else
                shades = launchShade<kEmCosine, GRAD>(S, kindMask, Q, cur, b32, npix, sample0, r, g, b, stats, gridBlocks, smem, G, stream, pdl,
                                                                  bounce + 1);
            if (trav == 2) launchStage(pdl, shadowKernel<GRAD, 2>, queryGrid, kWaveBlock, smem, stream, S, Q, cur, r, g, b, stats, G);
            else if (trav == 1) launchStage(pdl, shadowKernel<GRAD, 1>, queryGrid, kWaveBlock, smem, stream, S, Q, cur, r, g, b, stats, G);
            else launchStage(pdl, shadowKernel<GRAD, 0>, queryGrid, kWaveBlock, smem, stream, S, Q, cur, r, g, b, stats, G);
            *launches += 2 + shades;
            if (S.maxPL == 0 && (bounce & 7) == 7 && capturing == cudaStreamCaptureStatusNone) {
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

}  // namespace

size_t wavefrontBytes(uint64_t cap, bool grad)
{
    return align256(sizeof(Counters)) + 2 * align256(32 * cap) + align256(8 * cap) + kNumBuckets * align256(4 * cap) +
           2 * align256(48 * cap) + align256((grad ? 80 : 48) * cap) + (grad ? align256(8 * cap) : 0);
}

cudaError_t launchWavefront(const SceneView &S, uint32_t kindMask, uint32_t sample0, uint64_t numPaths, uint32_t npix,
                            float *outR, float *outG, float *outB, DevStats *stats, void *scratch, uint64_t capacity,
                            int gridBlocks, cudaStream_t stream, uint64_t *launches, const GradArgs *grad,
                            const uint32_t *sampleOffset, bool pdlInCapture)
{
    if (capacity > kMaxSlots || numPaths > 0xffffffffull) return cudaErrorInvalidValue;
    if (grad)
        return runWavefront<true>(S, kindMask, sample0, numPaths, npix, outR, outG, outB, stats, scratch, capacity,
                                  gridBlocks, stream, launches, *grad);
    GradArgs none{};
    none.sampleOffset = sampleOffset;
    return runWavefront<false>(S, kindMask, sample0, numPaths, npix, outR, outG, outB, stats, scratch, capacity,
                               gridBlocks, stream, launches, none, pdlInCapture);
}

}  // namespace pg3
