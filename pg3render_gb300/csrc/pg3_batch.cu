// Batched rendering: many scene instances on one persistent wavefront (pg3gpu_batch_* of
// include/pg3gpu.h). No counterpart in the reference, which renders one scene per process
// (src/pg3render.cxx:65-162).
//
// Paths of all instances share `capacity` slots. One step of the device-side loop:
//   regen     start camera paths of the next global path indices in the free slots the
//             previous step's advance granted (the global index runs over all instances:
//             instance i owns [first_i, first_i + npix_i * spp_i))
//   extend    closest hit, bucketed by material kind (instance scenes from shared memory)
//   shade x4  the vertex of pg3_wave.cuh; a path that ends adds its radiance to its instance's
//             framebuffer (fp64 atomics, sum and sum of squares) and frees its slot, unless its
//             last light sample is still pending, which then carries a `last` mark
//   shadow    any-hit; `last` records finish their path after adding their contribution
//   advance   one thread: swaps the ray queues, grants the free slots to regen when fewer
//             than `threshold` paths are active, ends the loop when no path is active and
//             none is left, or after maxSteps (a bound that a correct run never reaches)
// With a CUDA graph, the steps are the body of a conditional while node, so a whole run is
// one graph launch; advance writes the loop condition.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "pg3_ctx.h"
#include "pg3_kernels.h"
#include "pg3_wave.cuh"

using namespace pg3;

namespace {

constexpr uint32_t kMaxInst = PG3GPU_BATCH_MAX_INSTANCES;
static_assert(kMaxInst <= 256, "instance ids ride in the 8 high bits of a tag");
static_assert(kMaxInst * sizeof(SceneView) <= 48 * 1024, "instance scenes must fit the default shared memory");
constexpr unsigned int kErrStepLimit = 8u;

struct BatchInst {
    double *sum, *sumsq;
    unsigned long long firstPath;   // global index of the instance's first path of a run
    uint32_t npix, sample0;
};

struct BatchCtl {
    unsigned long long nextPath, regenBase, totalPaths;
    uint32_t cur, regenCount, regenFreeTop, freeTop;
    uint32_t capacity, threshold, steps, maxSteps;
    uint32_t done, pad;
};

struct BatchQ {
    Queues q;
    float *outR, *outG, *outB;   // per slot: radiance of its path
    uint32_t *local;             // per slot: path index within its instance's run
    uint32_t *freeList;
};

// Copies the instance scenes to shared memory (8-byte words).
PG3_DI const SceneView *stageViews(const SceneView *views, uint32_t n, unsigned char *smem)
{
    static_assert(sizeof(SceneView) % 8 == 0, "SceneView is copied in 8-byte words");
    const uint32_t words = n * (uint32_t)(sizeof(SceneView) / 8);
    const uint2 *src = reinterpret_cast<const uint2 *>(views);
    uint2 *dst = reinterpret_cast<uint2 *>(smem);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    return reinterpret_cast<const SceneView *>(smem);
}

PG3_DI uint32_t findInstance(const BatchInst *inst, uint32_t n, unsigned long long g)
{
    uint32_t lo = 0, hi = n;   // inst[lo].firstPath <= g, and g < inst[hi].firstPath when hi < n
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (inst[mid].firstPath <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

PG3_DI void finishPath(const BatchInst *inst, uint32_t id, uint32_t pixel, const BatchQ &B, uint32_t slot)
{
    const double r = B.outR[slot], g = B.outG[slot], b = B.outB[slot];
    double *s = inst[id].sum + 3 * (size_t)pixel, *q = inst[id].sumsq + 3 * (size_t)pixel;
    atomicAdd(s, r);
    atomicAdd(s + 1, g);
    atomicAdd(s + 2, b);
    atomicAdd(q, r * r);
    atomicAdd(q + 1, g * g);
    atomicAdd(q + 2, b * b);
}

// All lanes of the warp call this; lanes with `rel` push their slot to the free list.
PG3_DI void releaseSlot(const BatchQ &B, BatchCtl *ctl, bool rel, uint32_t slot)
{
    const uint32_t pos = warpAppend(&ctl->freeTop, rel);
    if (rel && pos < B.q.cap) B.freeList[pos] = slot;
    else if (rel) atomicOr(B.q.err, kErrQueueOverflow);
}

__global__ void batchInit(BatchQ B, BatchCtl *ctl, uint32_t capacity, unsigned long long total, uint32_t threshold,
                          uint32_t maxSteps)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t i = t; i < capacity; i += gridDim.x * blockDim.x) B.freeList[i] = capacity - 1 - i;
    if (t == 0) {
        *B.q.cnt = Counters{};
        const uint32_t k = (uint32_t)min((unsigned long long)capacity, total);
        BatchCtl c{};
        c.totalPaths = total;
        c.nextPath = k;
        c.regenBase = 0;
        c.regenCount = k;
        c.regenFreeTop = capacity;
        c.freeTop = capacity - k;
        c.capacity = capacity;
        c.threshold = threshold;
        c.maxSteps = maxSteps;
        c.done = total == 0;
        *ctl = c;
    }
}

__global__ void __launch_bounds__(kWaveBlock) batchRegen(const SceneView *views, const BatchInst *inst,
                                                         uint32_t ninst, BatchQ B, const BatchCtl *ctl,
                                                         DevStats *stats)
{
    const uint32_t k = ctl->regenCount;
    if (k == 0) return;
    const unsigned long long g0 = ctl->regenBase;
    const uint32_t top = ctl->regenFreeTop;
    const int cur = (int)ctl->cur;
    float4 *rq = rayQ(B.q, cur);
    for (uint32_t base = blockIdx.x * blockDim.x; base < k; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool want = i < k;
        float4 r0, r1;
        if (want) {
            const unsigned long long g = g0 + i;
            const uint32_t id = findInstance(inst, ninst, g);
            const uint32_t local = (uint32_t)(g - inst[id].firstPath);
            const uint32_t npix = inst[id].npix;
            const uint32_t pixel = local % npix, sample = inst[id].sample0 + local / npix;
            const SceneView &S = views[id];
            const uint32_t slot = B.freeList[top - 1 - i];   // i < k <= top <= capacity
            float3 dir;
            cameraRay(S, pixel, sample, dir);
            r0 = make_float4(S.camPos.x, S.camPos.y, S.camPos.z, 0.f);
            r1 = make_float4(dir.x, dir.y, dir.z, __uint_as_float(slot | (id << kSlotBits)));
            B.local[slot] = local;
            B.outR[slot] = 0.f;
            B.outG[slot] = 0.f;
            B.outB[slot] = 0.f;
        }
        const uint32_t pos = warpAppend(&B.q.cnt->ray[cur], want);
        if (want && pos < B.q.cap) {
            rq[2 * (size_t)pos] = r0;
            rq[2 * (size_t)pos + 1] = r1;
            initPathState(B.q, cur, pos);
        } else if (want) {
            atomicOr(B.q.err, kErrQueueOverflow);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&stats->paths, (unsigned long long)k);
}

__global__ void __launch_bounds__(kWaveBlock) batchExtend(const SceneView *views, uint32_t ninst, BatchQ B,
                                                          const BatchCtl *ctl, DevStats *stats)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SceneView *sv = stageViews(views, ninst, smem);
    const int cur = (int)ctl->cur;
    const uint32_t n = B.q.cnt->ray[cur];
    const float4 *rq = rayQ(B.q, cur);
    uint32_t rays = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        int bucket = -1;
        if (i < n) {
            const uint32_t id = __float_as_uint(rq[2 * i + 1].w) >> kSlotBits;
            bucket = extendOne<-2>(sv[id], B.q, rq, i);
            ++rays;
        }
        bucketAppend(B.q, bucket, i);
    }
    countWarp(&stats->extRays, rays);
}

// resident 256-thread blocks per SM the batch shade kernels are compiled for (128 registers)
#ifndef PG3_BATCH_SHADE_MIN_BLOCKS
#define PG3_BATCH_SHADE_MIN_BLOCKS 2
#endif

template <int K, int EMK>
__global__ void __launch_bounds__(kWaveBlock, PG3_BATCH_SHADE_MIN_BLOCKS)
    batchShade(const SceneView *views, const BatchInst *inst, uint32_t ninst, BatchQ B, BatchCtl *ctl,
               DevStats *stats)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SceneView *sv = stageViews(views, ninst, smem);
    constexpr int kBucket = bucketOfShade(K);
    const int cur = (int)ctl->cur;
    const uint32_t n = B.q.cnt->bucket[kBucket];
    const float4 *rq = rayQ(B.q, cur);
    const GradArgs G{};
    PathCounters pc;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        ShadeOut o;
        bool rel = false;
        uint32_t slot = 0;
        if (j < n) {
            const uint32_t idx = B.q.bucket[kBucket][j];
            const float4 r0 = rq[2 * idx], r1 = rq[2 * idx + 1];
            const uint32_t tag = __float_as_uint(r1.w);
            slot = tag & kSlotMask;
            const uint32_t id = tag >> kSlotBits;
            const uint32_t local = B.local[slot];
            const uint32_t npix = __ldg(&inst[id].npix);
            const uint32_t pixel = local % npix, sample = __ldg(&inst[id].sample0) + local / npix;
            float3 L;
            shadeVertex<K, EMK, false, false>(sv[id], B.q, idx, r0, r1, stQ(B.q, cur) + 3 * (size_t)idx, slot, tag, pixel, sample,
                                       pc, o, L, G, nullptr, f3(0.f));
            if (!isZero(L)) {
                B.outR[slot] += L.x;
                B.outG[slot] += L.y;
                B.outB[slot] += L.z;
            }
            if (!o.next) {
                if (o.shadow) o.s2.w = 1.f;   // the shadow stage finishes this path
                else {
                    finishPath(inst, id, pixel, B, slot);
                    rel = true;
                }
            }
        }
        emitRecords<false>(B.q, cur ^ 1, o);
        releaseSlot(B, ctl, rel, slot);
    }
    countWarp(&stats->byBackground, pc.bg);
    countWarp(&stats->byBlocker, pc.blocker);
    countWarp(&stats->byMax, pc.maxl);
    countWarp(&stats->bySafety, pc.safety);
    countWarp(&stats->byRR, pc.rr);
}

__global__ void __launch_bounds__(kWaveBlock) batchShadow(const SceneView *views, const BatchInst *inst,
                                                          uint32_t ninst, BatchQ B, BatchCtl *ctl, DevStats *stats)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const SceneView *sv = stageViews(views, ninst, smem);
    const uint32_t n = B.q.cnt->shadow;
    uint32_t cnt = 0;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t j = base + threadIdx.x;
        bool rel = false;
        uint32_t slot = 0;
        if (j < n) {
            const float4 *rec = B.q.shadow + 3 * (size_t)j;
            const float4 s0 = rec[0], s1 = rec[1], c = rec[2];
            const uint32_t tag = __float_as_uint(s1.w);
            slot = tag & kSlotMask;
            const uint32_t id = tag >> kSlotBits;
            ++cnt;
            if (!occludedAny<-2>(sv[id], xyz(s0), xyz(s1), s0.w)) {
                B.outR[slot] += c.x;
                B.outG[slot] += c.y;
                B.outB[slot] += c.z;
            }
            if (c.w != 0.f) {
                finishPath(inst, id, B.local[slot] % __ldg(&inst[id].npix), B, slot);
                rel = true;
            }
        }
        releaseSlot(B, ctl, rel, slot);
    }
    countWarp(&stats->shadowRays, cnt);
}

__global__ void batchAdvance(BatchQ B, BatchCtl *ctl, unsigned int *err, cudaGraphConditionalHandle handle,
                             int useGraph)
{
    if (ctl->done) {   // a run that has already ended (host-driven steps past its end)
        if (useGraph) cudaGraphSetConditional(handle, 0u);
        return;
    }
    Counters *c = B.q.cnt;
    const uint32_t cur = ctl->cur;
    c->ray[cur] = 0;
    for (int b = 0; b < kNumBuckets; ++b) c->bucket[b] = 0;
    c->shadow = 0;
    const uint32_t ncur = cur ^ 1u;
    const uint32_t active = c->ray[ncur];
    ctl->cur = ncur;
    const uint32_t steps = ++ctl->steps;
    const unsigned long long remaining = ctl->totalPaths - ctl->nextPath;
    uint32_t k = 0;
    if (remaining > 0 && active < ctl->threshold) k = (uint32_t)min((unsigned long long)ctl->freeTop, remaining);
    ctl->regenCount = k;
    ctl->regenFreeTop = ctl->freeTop;
    ctl->regenBase = ctl->nextPath;
    ctl->freeTop -= k;
    ctl->nextPath += k;
    bool done = (active == 0 && remaining == 0);
    if (!done && steps >= ctl->maxSteps) {
        atomicOr(err, kErrStepLimit);
        done = true;
    }
    ctl->done = done ? 1u : 0u;
    if (useGraph) cudaGraphSetConditional(handle, done ? 0u : 1u);
}

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

size_t batchBytes(uint64_t cap)
{
    return a256(sizeof(Counters)) + a256(sizeof(BatchCtl)) + 2 * a256(32 * cap) + a256(8 * cap) +
           kNumBuckets * a256(4 * cap) + 2 * a256(48 * cap) + a256(48 * cap) + 3 * a256(4 * cap) + 2 * a256(4 * cap);
}

void carveBatch(void *scratch, uint64_t cap, BatchQ &B, BatchCtl *&ctl)
{
    char *p = reinterpret_cast<char *>(scratch);
    auto take = [&](size_t bytes) { char *r = p; p += a256(bytes); return r; };
    B.q.cnt = (Counters *)take(sizeof(Counters));
    ctl = (BatchCtl *)take(sizeof(BatchCtl));
    B.q.ray[0] = (float4 *)take(32 * cap);
    B.q.ray[1] = (float4 *)take(32 * cap);
    B.q.hit = (float2 *)take(8 * cap);
    for (int b = 0; b < kNumBuckets; ++b) B.q.bucket[b] = (uint32_t *)take(4 * cap);
    B.q.bucketStride = a256(4 * cap) / 4;
    B.q.st[0] = (float4 *)take(48 * cap);
    B.q.st[1] = (float4 *)take(48 * cap);
    B.q.shadow = (float4 *)take(48 * cap);
    B.q.pend = nullptr;
    B.q.cap = (uint32_t)cap;
    B.outR = (float *)take(4 * cap);
    B.outG = (float *)take(4 * cap);
    B.outB = (float *)take(4 * cap);
    B.local = (uint32_t *)take(4 * cap);
    B.freeList = (uint32_t *)take(4 * cap);
}

}  // namespace

struct pg3gpu_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t captureStream = nullptr;
    std::vector<pg3gpu_ctx *> inst;
    std::vector<uint32_t> spp;
    std::vector<BatchInst> hostInst;
    uint64_t totalPaths = 0;
    uint32_t maxLen = 0;
    int emk = kEmCosine;
    uint32_t kindMask = 0;           // material kinds of all instances (bit per kind)
    int sms = 0;
    SceneView *dViews = nullptr;
    BatchInst *dInst = nullptr;
    DevStats *dStats = nullptr;
    unsigned int *dErr = nullptr;
    pg3gpu_batch_tuning tuning{};
    void *dScratch = nullptr;
    uint64_t scratchCap = 0;
    BatchQ B{};
    BatchCtl *dCtl = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle handle = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    uint64_t runs = 0;
    uint64_t launches = 0;
    uint64_t stepsCounted = 0;
    bool stepsPending = false;
    std::string lastError;
};

namespace {

thread_local std::string g_batchCreateError;

int bfail(pg3gpu_batch *b, int status, const std::string &msg)
{
    if (b) b->lastError = msg;
    else g_batchCreateError = msg;
    return status;
}

int bcuda(pg3gpu_batch *b, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return PG3GPU_OK;
    return bfail(b, e == cudaErrorMemoryAllocation ? PG3GPU_ERR_OUT_OF_MEMORY : PG3GPU_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

uint32_t effBlock(const pg3gpu_batch *b) { return b->tuning.block_size == 128 ? 128u : 256u; }
uint32_t effBlocksPerSm(const pg3gpu_batch *b)
{
    if (b->tuning.blocks_per_sm) return std::min<uint32_t>(b->tuning.blocks_per_sm, 16u);
    return 1024u / effBlock(b);   // 4 x 256 or 8 x 128 threads
}
uint64_t effCapacity(const pg3gpu_batch *b)
{
    uint64_t cap = b->tuning.capacity ? b->tuning.capacity : (1ull << 22);
    cap = std::min<uint64_t>(cap, kMaxSlots);
    cap = std::min<uint64_t>(cap, std::max<uint64_t>(b->totalPaths, 1024));
    return std::max<uint64_t>(cap, 1024);
}
float effThreshold(const pg3gpu_batch *b)
{
    const float t = b->tuning.regen_threshold;
    return (t > 0.f) ? std::min(t, 0.875f) : 0.5f;
}

void destroyGraph(pg3gpu_batch *b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

struct StepShape {
    int grid, block;
    size_t smem;
    uint32_t capacity, threshold, maxSteps;
};

StepShape stepShape(const pg3gpu_batch *b)
{
    StepShape s;
    s.block = (int)effBlock(b);
    s.grid = b->sms * (int)effBlocksPerSm(b);
    s.smem = b->inst.size() * sizeof(SceneView);
    s.capacity = (uint32_t)b->scratchCap;
    const uint32_t thr = (uint32_t)std::max(1.0, std::floor(effThreshold(b) * (double)s.capacity));
    s.threshold = thr;
    // a run refills at least capacity - threshold slots between two steps without a refill, and
    // a path lives at most maxLen + 1 steps: twice the steps this allows is out of reach
    const uint64_t minIssue = std::max<uint64_t>(1, s.capacity - thr);
    const uint64_t refills = b->totalPaths / minIssue + 2;
    const uint64_t bound = 2 * refills * (uint64_t)(b->maxLen + 2);
    s.maxSteps = (uint32_t)std::min<uint64_t>(bound, 0x7fffffffull);
    return s;
}

// Shade kernels of the miss bucket and of the material kinds present in the batch.
int shadeLaunches(uint32_t kindMask)
{
    int n = 1;
    for (int k = kMatLambert; k <= kMatPhong; ++k) n += (kindMask >> k) & 1u;
    return n + ((kindMask & ((1u << kMatSmoothConductor) | (1u << kMatSmoothDielectric))) ? 1 : 0);
}
int stepLaunches(const pg3gpu_batch *b) { return 4 + shadeLaunches(b->kindMask); }

template <int EMK>
void launchShadeBatch(const pg3gpu_batch *b, const StepShape &s, cudaStream_t st)
{
    const uint32_t n = (uint32_t)b->inst.size();
    const uint32_t m = b->kindMask;
    batchShade<-1, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    if (m & (1u << kMatLambert))
        batchShade<kMatLambert, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    if (m & (1u << kMatGgxConductor))
        batchShade<kMatGgxConductor, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    if (m & (1u << kMatGgxDielectric))
        batchShade<kMatGgxDielectric, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    if (m & (1u << kMatPhong))
        batchShade<kMatPhong, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    if (m & ((1u << kMatSmoothConductor) | (1u << kMatSmoothDielectric)))
        batchShade<kShadeSmooth, EMK><<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
}

// One step of the loop (regen, extend, the shade kernels, shadow, advance).
void launchStep(const pg3gpu_batch *b, const StepShape &s, cudaStream_t st, int useGraph)
{
    const uint32_t n = (uint32_t)b->inst.size();
    const int regenGrid = std::max(1, std::min(s.grid * 4, (int)((s.capacity + s.block - 1) / s.block)));
    batchRegen<<<regenGrid, s.block, 0, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    batchExtend<<<s.grid, s.block, s.smem, st>>>(b->dViews, n, b->B, b->dCtl, b->dStats);
    if (b->emk == kEmCdf) launchShadeBatch<kEmCdf>(b, s, st);
    else if (b->emk == kEmSteerable) launchShadeBatch<kEmSteerable>(b, s, st);
    else if (b->emk == kEmSteerableAdaptive) launchShadeBatch<kEmSteerableAdaptive>(b, s, st);
    else launchShadeBatch<kEmCosine>(b, s, st);
    batchShadow<<<s.grid, s.block, s.smem, st>>>(b->dViews, b->dInst, n, b->B, b->dCtl, b->dStats);
    batchAdvance<<<1, 1, 0, st>>>(b->B, b->dCtl, b->dErr, b->handle, useGraph);
}

void launchInit(const pg3gpu_batch *b, const StepShape &s, cudaStream_t st)
{
    const int g = std::max(1, std::min(b->sms * 4, (int)((s.capacity + 255) / 256)));
    batchInit<<<g, 256, 0, st>>>(b->B, b->dCtl, s.capacity, b->totalPaths, s.threshold, s.maxSteps);
}

int ensureScratch(pg3gpu_batch *b)
{
    const uint64_t cap = effCapacity(b);
    if (b->dScratch && cap == b->scratchCap) return PG3GPU_OK;
    destroyGraph(b);
    if (b->dScratch) {
        cudaStreamSynchronize(b->stream);
        cudaFree(b->dScratch);
        b->dScratch = nullptr;
        b->scratchCap = 0;
    }
    if (int st = bcuda(b, cudaMalloc(&b->dScratch, batchBytes(cap)), "batch queues")) return st;
    b->scratchCap = cap;
    carveBatch(b->dScratch, cap, b->B, b->dCtl);
    b->B.q.err = b->dErr;
    return PG3GPU_OK;
}

int buildGraph(pg3gpu_batch *b)
{
    if (b->exec) return PG3GPU_OK;
    const StepShape s = stepShape(b);
    cudaGraph_t g = nullptr;
    if (int st = bcuda(b, cudaGraphCreate(&g, 0), "cudaGraphCreate")) return st;
    b->graph = g;
    if (int st = bcuda(b, cudaGraphConditionalHandleCreate(&b->handle, g, 1, cudaGraphCondAssignDefault),
                       "cudaGraphConditionalHandleCreate"))
        return st;
    cudaStream_t cs = b->captureStream;
    if (int st = bcuda(b, cudaStreamBeginCaptureToGraph(cs, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                       "capture (init)"))
        return st;
    launchInit(b, s, cs);
    cudaGraph_t captured = nullptr;
    if (int st = bcuda(b, cudaStreamEndCapture(cs, &captured), "end capture (init)")) return st;
    size_t count = 0;
    if (int st = bcuda(b, cudaGraphGetNodes(g, nullptr, &count), "cudaGraphGetNodes")) return st;
    if (count != 1) return bfail(b, PG3GPU_ERR_CUDA, "batch graph: unexpected init node count");
    cudaGraphNode_t initNode;
    if (int st = bcuda(b, cudaGraphGetNodes(g, &initNode, &count), "cudaGraphGetNodes")) return st;
    cudaGraphNodeParams p{};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = b->handle;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t loop;
    if (int st = bcuda(b, cudaGraphAddNode(&loop, g, &initNode, nullptr, 1, &p), "conditional node")) return st;
    cudaGraph_t body = p.conditional.phGraph_out[0];
    if (int st = bcuda(b, cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
                       "capture (body)"))
        return st;
    launchStep(b, s, cs, 1);
    if (int st = bcuda(b, cudaStreamEndCapture(cs, &captured), "end capture (body)")) return st;
    if (int st = bcuda(b, cudaGraphInstantiate(&b->exec, g, 0), "cudaGraphInstantiate")) return st;
    return PG3GPU_OK;
}

// Reads how many steps the last run took (stream idle) and counts its launches.
void collectSteps(pg3gpu_batch *b)
{
    if (!b->stepsPending || !b->dCtl) return;
    uint32_t steps = 0;
    if (cudaMemcpy(&steps, &b->dCtl->steps, sizeof steps, cudaMemcpyDeviceToHost) == cudaSuccess)
        b->launches += 1 + (uint64_t)stepLaunches(b) * steps;
    b->stepsPending = false;
}

int runOnce(pg3gpu_batch *b)
{
    if (int st = ensureScratch(b)) return st;
    cudaSetDevice(b->device);
    for (size_t i = 0; i < b->inst.size(); ++i) b->hostInst[i].sample0 = (uint32_t)b->inst[i]->iterations;
    if (int st = bcuda(b, cudaMemcpyAsync(b->dInst, b->hostInst.data(), sizeof(BatchInst) * b->hostInst.size(),
                                          cudaMemcpyHostToDevice, b->stream),
                       "instance table upload"))
        return st;
    if (b->stepsPending) {
        cudaStreamSynchronize(b->stream);
        collectSteps(b);
    }
    if (int st = bcuda(b, cudaEventRecord(b->ev0, b->stream), "event")) return st;
    if (b->tuning.use_graph) {
        if (int st = buildGraph(b)) return st;
        if (int st = bcuda(b, cudaGraphLaunch(b->exec, b->stream), "cudaGraphLaunch")) return st;
        b->stepsPending = true;
    } else {
        const StepShape s = stepShape(b);
        launchInit(b, s, b->stream);
        b->launches += 1;
        // host-driven steps, 8 at a time, until the device reports the run finished
        const uint64_t maxChecks = (uint64_t)s.maxSteps / 8 + 2;
        uint32_t done = 0;
        for (uint64_t c = 0; c < maxChecks && !done; ++c) {
            for (int k = 0; k < 8; ++k) launchStep(b, s, b->stream, 0);
            b->launches += 8ull * stepLaunches(b);
            if (int st = bcuda(b, cudaMemcpyAsync(&done, &b->dCtl->done, sizeof done, cudaMemcpyDeviceToHost, b->stream),
                               "done flag"))
                return st;
            if (int st = bcuda(b, cudaStreamSynchronize(b->stream), "batch step")) return st;
        }
    }
    if (int st = bcuda(b, cudaEventRecord(b->ev1, b->stream), "event")) return st;
    if (int st = bcuda(b, cudaGetLastError(), "batch launch")) return st;
    b->timed = true;
    b->runs += 1;
    for (size_t i = 0; i < b->inst.size(); ++i) b->inst[i]->iterations += b->spp[i];
    return PG3GPU_OK;
}

}  // namespace

extern "C" {

int pg3gpu_batch_destroy(pg3gpu_batch *b)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroyGraph(b);
    if (b->dScratch) cudaFree(b->dScratch);
    cudaFree(b->dViews);
    cudaFree(b->dInst);
    cudaFree(b->dStats);
    cudaFree(b->dErr);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->captureStream) cudaStreamDestroy(b->captureStream);
    for (pg3gpu_ctx *c : b->inst) pg3gpu_destroy(c);
    delete b;
    return PG3GPU_OK;
}

int pg3gpu_batch_create(const pg3gpu_scene *scenes, const pg3gpu_options *opts, const uint32_t *spp, uint32_t n,
                        int device, pg3gpu_batch **out)
{
    if (!out) return bfail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!scenes || !opts || !spp) return bfail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "scenes, opts or spp is NULL");
    if (n == 0 || n > kMaxInst)
        return bfail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "batch needs 1.." + std::to_string(kMaxInst) + " instances");
    pg3gpu_batch *b = new (std::nothrow) pg3gpu_batch;
    if (!b) return bfail(nullptr, PG3GPU_ERR_OUT_OF_MEMORY, "host allocation failed");
    auto bail = [&](int st) {
        g_batchCreateError = b->lastError;
        pg3gpu_batch_destroy(b);
        return st;
    };
    b->device = device;
    for (uint32_t i = 0; i < n; ++i) {   // arguments first, before any device work
        const std::string who = "instance " + std::to_string(i) + ": ";
        if (opts[i].algorithm != PG3GPU_ALG_PATH_TRACING)
            return bail(bfail(b, PG3GPU_ERR_UNSUPPORTED, who + "batches render algorithm 7 (path tracing) only"));
        if (spp[i] == 0) return bail(bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, who + "spp must be positive"));
        if (opts[i].splitting_budget > 1 || opts[i].indirect_clipping > 0.f || opts[i].light_to_bsdf_ratio >= 1.5f)
            return bail(bfail(b, PG3GPU_ERR_UNSUPPORTED, who + "batches do not split paths or clip"));
    }
    int emk = -1;
    for (uint32_t i = 0; i < n; ++i) {
        const std::string who = "instance " + std::to_string(i) + ": ";
        pg3gpu_ctx *c = nullptr;
        const int st = createContext(&scenes[i], &opts[i], device, true, &c);
        if (st) return bail(bfail(b, st, who + pg3gpu_last_error(nullptr)));
        b->inst.push_back(c);
        b->spp.push_back(spp[i]);
        b->kindMask |= c->kindMask;
        if (c->kindMask & (1u << kMatSra))
            return bail(bfail(b, PG3GPU_ERR_UNSUPPORTED, who + "the path tracers cannot render the SRA layered material"));
        if (c->view.bgKind == kBgEnvMap) {
            if (emk >= 0 && emk != c->view.emSampler)
                return bail(bfail(b, PG3GPU_ERR_UNSUPPORTED, who + "all environment-map instances must use one sampler"));
            emk = c->view.emSampler;
        }
        const uint64_t paths = (uint64_t)c->W * c->H * spp[i];
        if (paths > 0xffffffffull) return bail(bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, who + "more than 2^32 paths per run"));
        BatchInst bi{};
        bi.sum = c->dSum;
        bi.sumsq = c->dSumsq;
        bi.firstPath = b->totalPaths;
        bi.npix = c->W * c->H;
        b->hostInst.push_back(bi);
        b->totalPaths += paths;
        b->maxLen = std::max(b->maxLen, c->view.maxPL > 0 ? c->view.maxPL : kMaxPathLengthHard);
    }
    b->emk = emk >= 0 ? emk : kEmCosine;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, device);
    if (int st = bcuda(b, cudaStreamCreateWithFlags(&b->captureStream, cudaStreamNonBlocking), "stream")) return bail(st);
    if (int st = bcuda(b, cudaMalloc(&b->dViews, sizeof(SceneView) * n), "cudaMalloc")) return bail(st);
    if (int st = bcuda(b, cudaMalloc(&b->dInst, sizeof(BatchInst) * n), "cudaMalloc")) return bail(st);
    if (int st = bcuda(b, cudaMalloc(&b->dStats, sizeof(DevStats)), "cudaMalloc")) return bail(st);
    if (int st = bcuda(b, cudaMalloc(&b->dErr, sizeof(unsigned int)), "cudaMalloc")) return bail(st);
    std::vector<SceneView> views(n);
    for (uint32_t i = 0; i < n; ++i) views[i] = b->inst[i]->view;
    if (int st = bcuda(b, cudaMemcpy(b->dViews, views.data(), sizeof(SceneView) * n, cudaMemcpyHostToDevice), "upload"))
        return bail(st);
    if (int st = bcuda(b, cudaMemset(b->dStats, 0, sizeof(DevStats)), "memset")) return bail(st);
    if (int st = bcuda(b, cudaMemset(b->dErr, 0, sizeof(unsigned int)), "memset")) return bail(st);
    if (int st = bcuda(b, cudaEventCreate(&b->ev0), "event")) return bail(st);
    if (int st = bcuda(b, cudaEventCreate(&b->ev1), "event")) return bail(st);
    b->tuning.use_graph = 1;
    if (int st = bcuda(b, cudaDeviceSynchronize(), "setup")) return bail(st);
    *out = b;
    return PG3GPU_OK;
}

int pg3gpu_batch_set_stream(pg3gpu_batch *b, void *stream)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    b->stream = reinterpret_cast<cudaStream_t>(stream);
    return PG3GPU_OK;
}

int pg3gpu_batch_set_tuning(pg3gpu_batch *b, const pg3gpu_batch_tuning *t)
{
    if (!b || !t) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (t->block_size != 0 && t->block_size != 128 && t->block_size != 256)
        return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "block_size must be 0, 128 or 256");
    if (t->capacity > kMaxSlots) return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "capacity above 2^24 slots");
    if (!(t->regen_threshold >= 0.f && t->regen_threshold <= 0.875f))
        return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "regen_threshold must be in [0, 0.875]");
    if (t->blocks_per_sm > 16) return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "blocks_per_sm above 16");
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    collectSteps(b);
    b->tuning = *t;
    destroyGraph(b);
    return PG3GPU_OK;
}

int pg3gpu_batch_get_tuning(pg3gpu_batch *b, pg3gpu_batch_tuning *t)
{
    if (!b || !t) return PG3GPU_ERR_INVALID_ARGUMENT;
    *t = b->tuning;
    t->capacity = (uint32_t)effCapacity(b);
    t->block_size = effBlock(b);
    t->blocks_per_sm = effBlocksPerSm(b);
    t->regen_threshold = effThreshold(b);
    return PG3GPU_OK;
}

int pg3gpu_batch_run(pg3gpu_batch *b)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    return runOnce(b);
}

int pg3gpu_batch_synchronize(pg3gpu_batch *b)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    if (int st = bcuda(b, cudaStreamSynchronize(b->stream), "batch")) return st;
    collectSteps(b);
    unsigned int flag = 0;
    if (int st = bcuda(b, cudaMemcpy(&flag, b->dErr, sizeof flag, cudaMemcpyDeviceToHost), "error flag")) return st;
    for (pg3gpu_ctx *c : b->inst) {
        unsigned int f = 0;
        if (cudaMemcpy(&f, c->dErr, sizeof f, cudaMemcpyDeviceToHost) == cudaSuccess) flag |= f;
    }
    if (flag)
        return bfail(b, PG3GPU_ERR_DEVICE_LIMIT,
                     "kernel limit flag " + std::to_string(flag) + " (1: BVH stack, 2: queue, 4: steerable descent, 8: step limit)");
    return PG3GPU_OK;
}

int pg3gpu_batch_read_framebuffer(pg3gpu_batch *b, uint32_t i, double *mean, double *var, uint64_t *spp)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (i >= b->inst.size()) return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "instance out of range");
    if (int st = pg3gpu_batch_synchronize(b)) return st;
    const int st = pg3gpu_read_framebuffer(b->inst[i], mean, var, spp);
    if (st) return bfail(b, st, pg3gpu_last_error(b->inst[i]));
    return PG3GPU_OK;
}

int pg3gpu_batch_save_image(pg3gpu_batch *b, uint32_t i, const char *path, float gamma)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (i >= b->inst.size()) return bfail(b, PG3GPU_ERR_INVALID_ARGUMENT, "instance out of range");
    if (int st = pg3gpu_batch_synchronize(b)) return st;
    const int st = pg3gpu_save_image(b->inst[i], path, gamma);
    if (st) return bfail(b, st, pg3gpu_last_error(b->inst[i]));
    return PG3GPU_OK;
}

int pg3gpu_batch_clear(pg3gpu_batch *b)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    collectSteps(b);
    for (pg3gpu_ctx *c : b->inst) {
        const size_t bytes = (size_t)c->W * c->H * 3 * sizeof(double);
        if (int st = bcuda(b, cudaMemset(c->dSum, 0, bytes), "clear")) return st;
        if (int st = bcuda(b, cudaMemset(c->dSumsq, 0, bytes), "clear")) return st;
        c->iterations = 0;
    }
    b->runs = 0;
    return PG3GPU_OK;
}

int pg3gpu_batch_autotune(pg3gpu_batch *b, uint32_t maxTrials, pg3gpu_batch_tuning *chosen)
{
    if (!b) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->device);
    pg3gpu_batch_tuning best = b->tuning;
    best.use_graph = 1;
    if (!best.capacity) best.capacity = (uint32_t)effCapacity(b);
    if (!best.block_size) best.block_size = 256;
    if (!(best.regen_threshold > 0.f)) best.regen_threshold = 0.5f;
    double bestMs = 1e300;
    uint32_t trials = 0;
    auto trial = [&](const pg3gpu_batch_tuning &t) -> int {
        if (trials >= maxTrials) return PG3GPU_OK;
        ++trials;
        if (int st = pg3gpu_batch_set_tuning(b, &t)) return st;
        if (int st = runOnce(b)) return st;   // builds the graph and warms up
        if (int st = runOnce(b)) return st;
        if (int st = pg3gpu_batch_synchronize(b)) return st;
        float ms = 0.f;
        if (int st = bcuda(b, cudaEventElapsedTime(&ms, b->ev0, b->ev1), "trial timing")) return st;
        if (ms < bestMs) {
            bestMs = ms;
            best = t;
        }
        return PG3GPU_OK;
    };
    // capacity, then refill threshold, then block shape (coordinate descent)
    const uint64_t capMax = std::min<uint64_t>(kMaxSlots, std::max<uint64_t>(b->totalPaths, 1024));
    for (uint32_t cap : {1u << 20, 1u << 21, 1u << 22, 1u << 23}) {
        if (cap > capMax && cap != (1u << 20)) continue;
        pg3gpu_batch_tuning t = best;
        t.capacity = cap;
        if (int st = trial(t)) return st;
    }
    for (float thr : {0.25f, 0.5f, 0.75f, 0.875f}) {
        pg3gpu_batch_tuning t = best;
        t.regen_threshold = thr;
        if (int st = trial(t)) return st;
    }
    for (uint32_t blk : {128u, 256u}) {
        for (uint32_t bps : {0u, 2u}) {
            pg3gpu_batch_tuning t = best;
            t.block_size = blk;
            t.blocks_per_sm = bps ? bps * (256u / blk) : 0u;
            if (int st = trial(t)) return st;
        }
    }
    if (int st = pg3gpu_batch_set_tuning(b, &best)) return st;
    if (int st = pg3gpu_batch_clear(b)) return st;
    if (chosen) pg3gpu_batch_get_tuning(b, chosen);
    return PG3GPU_OK;
}

int pg3gpu_batch_get_stats(pg3gpu_batch *b, pg3gpu_stats *out)
{
    if (!b || !out) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (int st = pg3gpu_batch_synchronize(b)) return st;
    DevStats d;
    if (int st = bcuda(b, cudaMemcpy(&d, b->dStats, sizeof d, cudaMemcpyDeviceToHost), "stats")) return st;
    std::memset(out, 0, sizeof *out);
    out->paths = d.paths;
    out->extension_rays = d.extRays;
    out->shadow_rays = d.shadowRays;
    out->terminated_by_russian_roulette = d.byRR;
    out->terminated_by_background = d.byBackground;
    out->terminated_by_blocker = d.byBlocker;
    out->terminated_by_max_limit = d.byMax;
    out->terminated_by_safety_limit = d.bySafety;
    float ms = 0.f;
    if (b->timed && cudaEventElapsedTime(&ms, b->ev0, b->ev1) == cudaSuccess) out->last_iteration_ms = ms;
    out->path_kernel_ms = 0.0;
    out->path_kernel_launches = b->runs;
    out->kernel_launches = b->launches;
    return PG3GPU_OK;
}

const char *pg3gpu_batch_last_error(const pg3gpu_batch *b) { return b ? b->lastError.c_str() : g_batchCreateError.c_str(); }

}  // extern "C"
