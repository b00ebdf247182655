// C ABI of the hot path (include/pg3gpu.h): context life cycle, scene upload,
// light-sampling tables, iteration scheduling and framebuffer readback.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pg3gpu.h"
#include "pg3_ctx.h"
#include "pg3_host.h"
#include "pg3_kernels.h"
#include "pg3_scene_view.h"

using namespace pg3;

namespace {

thread_local std::string g_createError;

int fail(pg3gpu_ctx *ctx, int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) ctx->lastError = buf;
    else g_createError = buf;
    return status;
}

}  // namespace

int pg3::ctxError(pg3gpu_ctx *ctx, int status, const std::string &msg) { return fail(ctx, status, "%s", msg.c_str()); }

namespace {

#define PG3_CUDA(ctx, call)                                                                          \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PG3GPU_ERR_OUT_OF_MEMORY : PG3GPU_ERR_CUDA, \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                           \
    } while (0)

template <typename T>
int devAlloc(pg3gpu_ctx *ctx, T **p, size_t count)
{
    void *q = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    PG3_CUDA(ctx, cudaMalloc(&q, bytes));
    ctx->allocs.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PG3GPU_OK;
}

template <typename T>
int upload(pg3gpu_ctx *ctx, T **p, const std::vector<T> &v)
{
    int st = devAlloc(ctx, p, v.size());
    if (st) return st;
    if (!v.empty()) PG3_CUDA(ctx, cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return PG3GPU_OK;
}

// The per-sample outputs and the wavefront queues of a context (hundreds of MB to 4.6 GiB) come
// from a memory pool of the library per device that keeps up to kPoolKeepBytes of freed memory:
// contexts created one after another (a render server, an end-to-end loop of create, render,
// read, destroy) reuse the previous context's buffers instead of a device allocation and free of
// that size each time. Stream-ordered on the context's stream; while that stream is being
// captured into a graph, plain allocations are used.
#ifndef PG3_QUEUE_POOL
#define PG3_QUEUE_POOL 1
#endif
// Framebuffer accumulation of a multi-chunk call overlapped with the next chunk's rendering.
#ifndef PG3_ACC_OVERLAP
#define PG3_ACC_OVERLAP 1
#endif
constexpr uint64_t kPoolKeepBytes = 8ull << 30;
constexpr int kMaxPoolDevices = 64;
cudaMemPool_t g_queuePools[kMaxPoolDevices] = {};
std::mutex g_queuePoolMutex;

cudaMemPool_t queuePool(int device)
{
    if (device < 0 || device >= kMaxPoolDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_queuePoolMutex);
    if (!g_queuePools[device]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        uint64_t keep = kPoolKeepBytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_queuePools[device] = pool;
    }
    return g_queuePools[device];
}

template <typename T>
int bigAlloc(pg3gpu_ctx *ctx, T **p, size_t count)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaMemPool_t pool = PG3_QUEUE_POOL ? queuePool(ctx->device) : nullptr;
    if (pool && cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
        void *q = nullptr;
        const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
        PG3_CUDA(ctx, cudaMallocFromPoolAsync(&q, bytes, pool, ctx->stream));
        ctx->pooled.push_back(q);
        *p = reinterpret_cast<T *>(q);
        return PG3GPU_OK;
    }
    return devAlloc(ctx, p, count);
}

void bigFree(pg3gpu_ctx *ctx, void *p)
{
    if (!p) return;
    auto it = std::find(ctx->pooled.begin(), ctx->pooled.end(), p);
    if (it != ctx->pooled.end()) {
        cudaFreeAsync(p, ctx->stream);
        ctx->pooled.erase(it);
    } else
        ctxFree(ctx, p);
}

int ensureOutputSet(pg3gpu_ctx *ctx, float *(&out)[3], uint64_t &capacity, uint64_t paths)
{
    if (paths <= capacity) return PG3GPU_OK;
    for (auto &p : out) {
        bigFree(ctx, p);
        p = nullptr;
    }
    for (auto &p : out) {
        int st = bigAlloc(ctx, &p, paths);
        if (st) return st;
    }
    capacity = paths;
    return PG3GPU_OK;
}
int ensureOutput(pg3gpu_ctx *ctx, uint64_t paths) { return ensureOutputSet(ctx, ctx->dOut, ctx->outCapacity, paths); }

// Wavefront queues for launches of `paths` paths: max_paths_in_flight slots (default 2^24, the
// slot-index limit: 292 bytes per slot, 4.6 GiB at most), fewer when a launch has fewer paths;
// they only grow. A launch chunk then holds all paths of up to 2^24 samples, so the sparse
// late bounces, where roulette has ended most paths, repeat once per 2^24 paths instead of once
// per 2^22 (+20% on the 512x512 x 256 spp environment-map benchmark).
int ensureWave(pg3gpu_ctx *ctx, uint64_t paths)
{
    const uint64_t cap = ctx->opts.max_paths_in_flight ? ctx->opts.max_paths_in_flight : (1ull << 24);
    const uint64_t want = std::min<uint64_t>(cap, paths);
    if (ctx->dWave && ctx->waveCapacity >= want) return PG3GPU_OK;
    bigFree(ctx, ctx->dWave);
    ctx->dWave = nullptr;
    ctx->waveCapacity = 0;
    char *w = nullptr;
    if (int st = bigAlloc(ctx, &w, wavefrontBytes(want, false))) return st;
    ctx->dWave = w;
    ctx->waveCapacity = want;
    return PG3GPU_OK;
}

// Frame stacks of the recursive estimator: one stack of (max path length or the hard limit)
// frames per thread, at most 2 GiB, so deep roulette paths get fewer resident threads.
int ensureTree(pg3gpu_ctx *ctx)
{
    if (ctx->dTree) return PG3GPU_OK;
    const uint32_t depth = ctx->view.maxPL > 0 ? ctx->view.maxPL : 1200u;
    const uint64_t perThread = (uint64_t)depth * sizeof(TreeFrame);
    uint64_t threads = std::min<uint64_t>((uint64_t)ctx->megaGrid * kMegaBlock, (2ull << 30) / perThread);
    threads = std::max<uint64_t>(kMegaBlock, threads / kMegaBlock * kMegaBlock);
    TreeFrame *t = nullptr;
    if (int st = devAlloc(ctx, &t, threads * depth)) return st;
    ctx->dTree = t;
    ctx->treeDepth = depth;
    ctx->treeGrid = (int)(threads / kMegaBlock);
    return PG3GPU_OK;
}

// Paths per launch chunk: whole sample passes, bounded by max_paths_in_flight.
uint32_t passesPerChunk(const pg3gpu_ctx *ctx, uint32_t spp)
{
    const uint64_t npix = (uint64_t)ctx->W * ctx->H;
    const uint64_t budget = ctx->opts.max_paths_in_flight ? ctx->opts.max_paths_in_flight : (1ull << 24);
    uint64_t k = std::max<uint64_t>(1, budget / npix);
    return (uint32_t)std::min<uint64_t>(k, spp);
}

// Adds the elapsed times of all recorded path-kernel launches (stream must be idle).
void foldTimers(pg3gpu_ctx *ctx)
{
    for (int i = 0; i < ctx->pendingTimers; ++i) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ctx->tStart[i], ctx->tStop[i]) == cudaSuccess) ctx->kernelMs += ms;
    }
    ctx->pendingTimers = 0;
}

// Scene / algorithm combinations the path kernels refuse before any launch (every entry point
// that renders calls this).
int checkRenderable(pg3gpu_ctx *ctx, int algorithm)
{
    if ((ctx->kindMask & (1u << kMatSra)) &&
        (algorithm == PG3GPU_ALG_PATH_TRACING || algorithm == PG3GPU_ALG_PATH_TRACING_NAIVE))
        return fail(ctx, PG3GPU_ERR_UNSUPPORTED,
                    "the SRA layered material has no roulette probability or zero-reflectance test, so the path "
                    "tracers cannot render it (the reference stops with a fatal error, src/materials.hxx:1544-1557)");
    return PG3GPU_OK;
}

// algorithm: 7 runs on the wavefront pipeline (unless the megakernel was chosen), the others
// on the megakernel
// out: the per-sample output set (second: ctx->dOut2)
int renderChunk(pg3gpu_ctx *ctx, int algorithm, uint32_t sample0, uint32_t passes, bool second = false)
{
    if (int st = checkRenderable(ctx, algorithm)) return st;
    const uint32_t npix = ctx->W * ctx->H;
    const uint64_t paths = (uint64_t)passes * npix;
    int st = second ? ensureOutputSet(ctx, ctx->dOut2, ctx->out2Capacity, paths) : ensureOutput(ctx, paths);
    float *const *out = second ? ctx->dOut2 : ctx->dOut;
    const bool tree = algorithm == PG3GPU_ALG_PATH_TRACING && ctx->view.treeMode;
    const bool wave = ctx->useWavefront && algorithm == PG3GPU_ALG_PATH_TRACING && !tree;
    if (!st && wave) st = ensureWave(ctx, paths);
    if (!st && tree) st = ensureTree(ctx);
    if (st) return st;
    if (ctx->pendingTimers == pg3gpu_ctx::kTimerSlots) {
        cudaStreamSynchronize(ctx->stream);
        foldTimers(ctx);
    }
    const int slot = ctx->pendingTimers++;
    cudaEventRecord(ctx->tStart[slot], ctx->stream);
    cudaError_t e;
    uint64_t launches = 1;
    if (wave) {
        launches = 0;
        e = launchWavefront(ctx->view, ctx->kindMask, sample0, paths, npix, out[0], out[1], out[2],
                            ctx->dStats, ctx->dWave, ctx->waveCapacity, ctx->waveGrid, ctx->stream, &launches);
    } else
        e = launchMegakernel(ctx->view, algorithm, sample0, paths, npix, out[0], out[1], out[2],
                             ctx->dStats, tree ? ctx->treeGrid : ctx->megaGrid, ctx->stream, ctx->dTree,
                             ctx->treeDepth);
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "path kernel launch: %s", cudaGetErrorString(e));
    cudaEventRecord(ctx->tStop[slot], ctx->stream);
    ctx->kernelLaunches += 1;
    ctx->allLaunches += launches;
    return PG3GPU_OK;
}

// Calls of at most this many paths in one launch chunk replay a captured render graph: their
// ~90 stage launches cost more than their kernels' work (a 512x512 call of one sample per pixel,
// the reference's RunIteration pattern, is launch bound).
#ifndef PG3_CALL_GRAPH_MAX_PATHS
#define PG3_CALL_GRAPH_MAX_PATHS (1u << 22)
#endif
// The stage launches inside the render graph keep their programmatic dependencies (a stage's
// blocks start while its predecessor drains and wait in griddepcontrol.wait).
#ifndef PG3_CALL_GRAPH_PDL
#define PG3_CALL_GRAPH_PDL 1
#endif

bool callGraphEligible(pg3gpu_ctx *ctx, int algorithm, uint32_t spp)
{
    const uint64_t paths = (uint64_t)ctx->W * ctx->H * spp;
    if (PG3_CALL_GRAPH_MAX_PATHS == 0 || paths > PG3_CALL_GRAPH_MAX_PATHS) return false;
    if (algorithm != PG3GPU_ALG_PATH_TRACING || !ctx->useWavefront || ctx->view.treeMode) return false;
    // roulette-only paths end when the host sees an empty queue: not a fixed launch sequence
    if (ctx->view.maxPL == 0 || passesPerChunk(ctx, spp) != spp) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(ctx->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
    return true;
}

void dropCallGraph(pg3gpu_ctx *ctx)
{
    if (ctx->callGraphExec) cudaGraphExecDestroy(ctx->callGraphExec);
    if (ctx->callGraph) cudaGraphDestroy(ctx->callGraph);
    ctx->callGraphExec = nullptr;
    ctx->callGraph = nullptr;
    ctx->callGraphHead = nullptr;
    ctx->callGraphPasses = 0;
}

// Captures one launch chunk of `passes` samples per pixel (sample indices from the word
// dCallBase on) and its accumulation into the framebuffer.
int captureCallGraph(pg3gpu_ctx *ctx, uint32_t passes)
{
    dropCallGraph(ctx);
    const uint32_t npix = ctx->W * ctx->H;
    const uint64_t paths = (uint64_t)passes * npix;
    if (int st = ensureOutput(ctx, paths)) return st;
    if (int st = ensureWave(ctx, paths)) return st;
    if (!ctx->dCallBase) {
        if (int st = devAlloc(ctx, &ctx->dCallBase, 1)) return st;
    }
    if (!ctx->graphStream) PG3_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->graphStream, cudaStreamNonBlocking));
    // the capture stream must not run ahead of work already queued on the context's stream
    PG3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    PG3_CUDA(ctx, cudaStreamBeginCapture(ctx->graphStream, cudaStreamCaptureModeThreadLocal));
    uint64_t launches = 0;
    cudaError_t e = launchSetWord(ctx->dCallBase, 0u, ctx->graphStream);
    if (e == cudaSuccess)
        e = launchWavefront(ctx->view, ctx->kindMask, 0u, paths, npix, ctx->dOut[0], ctx->dOut[1], ctx->dOut[2],
                            ctx->dStats, ctx->dWave, ctx->waveCapacity, ctx->waveGrid, ctx->graphStream, &launches,
                            nullptr, ctx->dCallBase, PG3_CALL_GRAPH_PDL != 0);
    if (e == cudaSuccess)
        e = launchAccumulate(npix, passes, ctx->dOut[0], ctx->dOut[1], ctx->dOut[2], ctx->dSum, ctx->dSumsq,
                             ctx->graphStream);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(ctx->graphStream, &g);
    if (e == cudaSuccess) e = ee;
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(ctx, PG3GPU_ERR_CUDA, "render graph capture: %s", cudaGetErrorString(e));
    }
    cudaGraphNode_t roots[2];
    size_t nroots = 2;
    e = cudaGraphGetRootNodes(g, roots, &nroots);
    if (e == cudaSuccess && nroots != 1) e = cudaErrorInvalidValue;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return fail(ctx, PG3GPU_ERR_CUDA, "render graph: %s", cudaGetErrorString(e));
    }
    ctx->callGraph = g;
    ctx->callGraphExec = exec;
    ctx->callGraphHead = roots[0];
    ctx->callGraphPasses = passes;
    ctx->callGraphLaunches = launches + 2;   // + the head node and the accumulation
    std::memcpy(&ctx->callGraphView, &ctx->view, sizeof(SceneView));   // bytes, as runCallGraph compares them
    const void *bufs[6] = {ctx->dOut[0], ctx->dOut[1], ctx->dOut[2], ctx->dWave, ctx->dSum, ctx->dStats};
    std::memcpy(ctx->callGraphBufs, bufs, sizeof bufs);
    return PG3GPU_OK;
}

// One call through the render graph (captured on first use, and again when the passes, the
// scene view or a buffer changed).
int runCallGraph(pg3gpu_ctx *ctx, uint32_t iteration, uint32_t spp)
{
    const void *bufs[6] = {ctx->dOut[0], ctx->dOut[1], ctx->dOut[2], ctx->dWave, ctx->dSum, ctx->dStats};
    if (!ctx->callGraphExec || ctx->callGraphPasses != spp ||
        std::memcmp(&ctx->callGraphView, &ctx->view, sizeof(SceneView)) != 0 ||
        std::memcmp(ctx->callGraphBufs, bufs, sizeof bufs) != 0) {
        if (int st = captureCallGraph(ctx, spp)) return st;
    }
    cudaKernelNodeParams p = {};
    uint32_t *dst = ctx->dCallBase;
    uint32_t value = iteration;
    void *args[2] = {&dst, &value};
    p.func = const_cast<void *>(setWordKernelFunction());
    p.gridDim = dim3(1);
    p.blockDim = dim3(1);
    p.sharedMemBytes = 0;
    p.kernelParams = args;
    p.extra = nullptr;
    PG3_CUDA(ctx, cudaGraphExecKernelNodeSetParams(ctx->callGraphExec, ctx->callGraphHead, &p));
    if (ctx->pendingTimers == pg3gpu_ctx::kTimerSlots) {
        cudaStreamSynchronize(ctx->stream);
        foldTimers(ctx);
    }
    const int slot = ctx->pendingTimers++;   // the path-kernel timer spans the whole replay
    PG3_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    PG3_CUDA(ctx, cudaEventRecord(ctx->tStart[slot], ctx->stream));
    PG3_CUDA(ctx, cudaGraphLaunch(ctx->callGraphExec, ctx->stream));
    PG3_CUDA(ctx, cudaEventRecord(ctx->tStop[slot], ctx->stream));
    PG3_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->timed = true;
    ctx->iterations += spp;
    ctx->kernelLaunches += 1;
    ctx->allLaunches += ctx->callGraphLaunches;
    return PG3GPU_OK;
}

}  // namespace

extern "C" {

void pg3gpu_default_options(pg3gpu_options *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->algorithm = PG3GPU_ALG_PATH_TRACING;
    o->min_path_length = 1;
    o->max_path_length = 0;
    o->rr_min_path_length = 0;
    o->indirect_clipping = 0.f;
    o->splitting_budget = 1;
    o->splitting_level = 1.f;
    o->light_to_bsdf_ratio = 1.f;
    o->em_sampler = PG3GPU_EM_CDF;
    o->traversal = PG3GPU_TRAVERSAL_AUTO;
    o->pipeline = PG3GPU_PIPELINE_AUTO;
    o->steer_subdiv_level = 3;
    o->steer_weights = PG3GPU_STEER_WEIGHTS_PROJECTED;
    o->steer_max_subdiv_level = 0;
    o->steer_max_approx_error = 5.f;
    o->seed = 1234;
}

const char *pg3gpu_status_string(int s)
{
    switch (s) {
    case PG3GPU_OK: return "ok";
    case PG3GPU_ERR_INVALID_ARGUMENT: return "invalid argument";
    case PG3GPU_ERR_UNSUPPORTED: return "unsupported";
    case PG3GPU_ERR_CUDA: return "CUDA error";
    case PG3GPU_ERR_OUT_OF_MEMORY: return "out of device memory";
    case PG3GPU_ERR_DEVICE_LIMIT: return "device limit reached";
    default: return "unknown status";
    }
}

const char *pg3gpu_version(void) { return "pg3gpu 0.1 sm_103a"; }

const char *pg3gpu_last_error(const pg3gpu_ctx *ctx) { return ctx ? ctx->lastError.c_str() : g_createError.c_str(); }

int pg3gpu_destroy(pg3gpu_ctx *ctx)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->accStream) {
        cudaStreamSynchronize(ctx->accStream);
        cudaStreamDestroy(ctx->accStream);
    }
    for (cudaEvent_t ev : {ctx->evRendered[0], ctx->evRendered[1], ctx->evAccumulated[0], ctx->evAccumulated[1],
                           ctx->evAccJoin})
        if (ev) cudaEventDestroy(ev);
    if (ctx->graphStream) cudaStreamSynchronize(ctx->graphStream);
    if (ctx->callGraphExec) cudaGraphExecDestroy(ctx->callGraphExec);
    if (ctx->callGraph) cudaGraphDestroy(ctx->callGraph);
    if (ctx->graphStream) cudaStreamDestroy(ctx->graphStream);
    if (!ctx->pooled.empty()) {
        for (void *p : ctx->pooled) cudaFreeAsync(p, ctx->stream);   // back to the library's pool
        cudaStreamSynchronize(ctx->stream);
    }
    for (void *p : ctx->allocs) cudaFree(p);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (int i = 0; i < pg3gpu_ctx::kTimerSlots; ++i) {
        if (ctx->tStart[i]) cudaEventDestroy(ctx->tStart[i]);
        if (ctx->tStop[i]) cudaEventDestroy(ctx->tStop[i]);
    }
    delete ctx;
    return PG3GPU_OK;
}

}  // extern "C"

namespace {

int floatBitsAsInt(float f)
{
    int i;
    std::memcpy(&i, &f, sizeof i);
    return i;
}

// The 4-wide BVH of a binary LBVH (root = node 0): every wide node takes its binary node's
// children, with each inner child replaced by that child's own two children, so a wide node has
// up to 4 children and the tree half the binary tree's levels. Wide nodes are numbered breadth
// first (root 0). Returns false if a child id is out of range or a node is reached twice.
bool collapseBvh4(const std::vector<BvhNode> &bin, std::vector<BvhNode4> &out)
{
    const int n = (int)bin.size();
    out.clear();
    if (n < 1) return false;
    std::vector<int> queue{0};
    std::vector<char> seen((size_t)n, 0);
    seen[0] = 1;
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const BvhNode &b = bin[(size_t)queue[qi]];
        int id[4];
        float4 lo[4], hi[4];
        int cnt = 0;
        const float4 los[2] = {b.lo_l, b.lo_r}, his[2] = {b.hi_l, b.hi_r};
        for (int side = 0; side < 2; ++side) {
            const int c = floatBitsAsInt(los[side].w);
            if (c >= 0) {
                if (c >= n) return false;
                const BvhNode &g = bin[(size_t)c];
                const float4 glo[2] = {g.lo_l, g.lo_r}, ghi[2] = {g.hi_l, g.hi_r};
                for (int gs = 0; gs < 2; ++gs) {
                    id[cnt] = floatBitsAsInt(glo[gs].w);
                    lo[cnt] = glo[gs];
                    hi[cnt] = ghi[gs];
                    ++cnt;
                }
            } else {
                id[cnt] = c;
                lo[cnt] = los[side];
                hi[cnt] = his[side];
                ++cnt;
            }
        }
        BvhNode4 w;
        const float big = 3.0e38f;
        float *lx = &w.lox.x, *hx = &w.hix.x, *ly = &w.loy.x, *hy = &w.hiy.x, *lz = &w.loz.x, *hz = &w.hiz.x;
        int *ch = &w.child.x;
        for (int k = 0; k < 4; ++k) {
            if (k < cnt) {
                lx[k] = lo[k].x; ly[k] = lo[k].y; lz[k] = lo[k].z;
                hx[k] = hi[k].x; hy[k] = hi[k].y; hz[k] = hi[k].z;
                if (id[k] >= 0) {
                    if (id[k] >= n || seen[(size_t)id[k]]) return false;
                    seen[(size_t)id[k]] = 1;
                    ch[k] = (int)queue.size();
                    queue.push_back(id[k]);
                } else
                    ch[k] = id[k];
            } else {
                lx[k] = ly[k] = lz[k] = big;
                hx[k] = hy[k] = hz[k] = -big;
                ch[k] = INT_MIN;
            }
        }
        w.pad = make_float4(0.f, 0.f, 0.f, 0.f);
        out.push_back(w);
    }
    return true;
}

}  // namespace

int pg3::uploadSteer(pg3gpu_ctx *ctx, std::shared_ptr<const SteerGeom> gp, const float *vwHost)
{
    if (!gp) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "steerable tables: no geometry");
    const SteerGeom &g = *gp;
    const uint32_t nLeaf = g.numLeaves();
    const bool uniformOk = !g.adaptive && nLeaf == (20ull << (2 * g.level)) && g.leafGrid == (4u << g.level) &&
                           g.leafCells.size() == 6ull * g.leafGrid * g.leafGrid &&
                           g.startCells.size() == 6ull * kSteerUniformStartGrid * kSteerUniformStartGrid;
    const bool adaptiveOk = g.adaptive && g.qtree.size() >= 5 && g.leafGrid == 0 &&
                            g.startCells.size() == 6ull * kSteerStartGrid * kSteerStartGrid;
    if ((!uniformOk && !adaptiveOk) || g.leafTri.size() != nLeaf || g.leafPlane.size() != nLeaf ||
        g.leafEdge.size() != 3ull * nLeaf || g.leafArea.size() != nLeaf || g.layerStart.size() < 2 ||
        g.layerStart.size() > kSteerMaxLayers + 1 || g.tri.size() < 20 || g.levelOffset.size() < 2)
        return fail(ctx, PG3GPU_ERR_CUDA, "steerable tables: unexpected leaf count, grid or tree depth");
    // the descent takes a node's children as consecutive ids from its first child (pg3_steer.cuh)
    for (uint32_t n = 0; n < g.numNodes(); ++n) {
        const int first = g.nodeChild[8 * (size_t)n];
        for (int i = 0; i < 8; ++i) {
            const int id = g.nodeChild[8 * (size_t)n + i];
            if (id != INT_MIN && (i >= 6 || id != (first >= 0 ? first + i : first - i)))
                return fail(ctx, PG3GPU_ERR_CUDA, "steerable tables: a tree node's children are not consecutive");
            if (id == INT_MIN && i + 1 < 8 && g.nodeChild[8 * (size_t)n + i + 1] != INT_MIN)
                return fail(ctx, PG3GPU_ERR_CUDA, "steerable tables: a tree node's children are not consecutive");
        }
    }
    // the previous tables of this context (an adaptive file replaces the triangulation)
    for (void *p : ctx->steerAllocs) ctxFree(ctx, p);
    ctx->steerAllocs.clear();
    const size_t mark = ctx->allocs.size();
    auto keep = [&](int st) {
        ctx->steerAllocs.insert(ctx->steerAllocs.end(), ctx->allocs.begin() + (std::ptrdiff_t)mark, ctx->allocs.end());
        return st;
    };
    SceneView &v = ctx->view;
    SteerView sv{};
    int st;
    if ((st = upload(ctx, (float4 **)&sv.vdir, g.vdir))) return keep(st);
    if ((st = upload(ctx, (int4 **)&sv.tri, g.tri))) return keep(st);
    if ((st = upload(ctx, (int **)&sv.nodeChild, g.nodeChild))) return keep(st);
    // leaf planes, then (pg3_steer.cuh) edge normals, leaf-locator cells, whole-sphere weights
    std::vector<float4> aux = g.leafPlane;
    aux.insert(aux.end(), g.leafEdge.begin(), g.leafEdge.end());
    for (const uint4 &c : g.leafCells) {
        float4 f;
        std::memcpy(&f, &c, sizeof f);
        aux.push_back(f);
    }
    const size_t rootAt = aux.size();
    aux.resize(rootAt + 3, make_float4(0.f, 0.f, 0.f, 0.f));
    if ((st = upload(ctx, (float4 **)&sv.leafPlane, aux))) return keep(st);
    int4 *leafTri = nullptr;
    if ((st = upload(ctx, &leafTri, g.leafTri))) return keep(st);
    if ((st = upload(ctx, (int4 **)&sv.faceCells, g.faceCells))) return keep(st);
    if (g.adaptive && (st = upload(ctx, (int4 **)&sv.qtree, g.qtree))) return keep(st);
    if (!g.startCells.empty() && (st = upload(ctx, (int **)&sv.startCells, g.startCells))) return keep(st);
    float *rootW = reinterpret_cast<float *>(const_cast<float4 *>(sv.leafPlane) + rootAt);
    sv.numLeaves = nLeaf;
    sv.leafGrid = g.leafGrid;
    sv.level = g.level;
    for (uint32_t l = 0; !g.adaptive && l + 1 < g.levelOffset.size(); ++l)
        if (g.levelOffset[l] != 20u * (((1u << (2 * l)) - 1u) / 3u))
            return fail(ctx, PG3GPU_ERR_CUDA, "steerable tables: unexpected level layout");
    sv.root = g.root;
    SteerWeightArgs &a = ctx->steerArgs;
    a = SteerWeightArgs{};
    a.em = v.em;
    a.emW = v.emW;
    a.emH = v.emH;
    a.vdir = sv.vdir;
    a.numVertices = (uint32_t)g.vdir.size();
    a.leafTri = leafTri;
    a.numLeaves = nLeaf;
    if ((st = upload(ctx, (float **)&a.leafArea, g.leafArea))) return keep(st);
    a.nodeChild = sv.nodeChild;
    a.numLayers = (uint32_t)g.layerStart.size() - 1;
    for (uint32_t l = 0; l <= a.numLayers; ++l) a.layerStart[l] = g.layerStart[l];
    if ((st = devAlloc(ctx, &a.vw, 12 * (size_t)a.numVertices))) return keep(st);
    if ((st = devAlloc(ctx, &a.vlum, (size_t)a.numVertices))) return keep(st);
    if ((st = devAlloc(ctx, &a.leafRec, 5 * (size_t)nLeaf))) return keep(st);
    a.projected = (ctx->opts.steer_weights == PG3GPU_STEER_WEIGHTS_PROJECTED) ? 1 : 0;
    unsigned char *proj = nullptr;
    if (a.projected && (st = devAlloc(ctx, &proj, projScratchBytes(a.numVertices)))) return keep(st);
    a.projScratch = proj;
    if ((st = devAlloc(ctx, &a.leafW, 9 * (size_t)nLeaf))) return keep(st);
    if ((st = devAlloc(ctx, &a.nodeW, 4 * (size_t)kSteerNodeVec4 * g.numNodes()))) return keep(st);
    a.rootW = rootW;
    sv.leafRec = a.leafRec;
    sv.nodeW = a.nodeW;
    a.locator = sv;      // geometry and locator tables (vw / nodeW are outputs of this build)
    keep(PG3GPU_OK);
    cudaError_t e;
    if (vwHost) {
        e = cudaMemcpy(a.vw, vwHost, 12 * sizeof(float) * (size_t)a.numVertices, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launchSteerTreeWeights(a, nullptr);
    } else
        e = launchSteerWeights(a, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "steerable build: %s", cudaGetErrorString(e));
    v.steer = sv;
    v.bgShL = a.rootW;   // the background's picking estimate: the sampler's whole integral
    v.emSampler = g.adaptive ? kEmSteerableAdaptive : kEmSteerable;
    ctx->steerGeom = gp;
    ctx->hasSteer = true;
    return PG3GPU_OK;
}

// forBatch: a scene instance of a batch (pg3_batch.cu) -- no launch queues, outputs or timers
int pg3::createContext(const pg3gpu_scene *scene, const pg3gpu_options *opts, int device, bool forBatch,
                       pg3gpu_ctx **out)
{
    if (!out) return fail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (!scene || !opts) return fail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "scene or options is NULL");

    HostScene hs;
    std::string err;
    int st = prepareScene(*scene, *opts, hs, err);
    if (st != PG3GPU_OK) return fail(nullptr, st, "%s", err.c_str());

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, PG3GPU_ERR_CUDA, "no CUDA device visible");
    if (device < 0 || device >= ndev) return fail(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "device %d out of range", device);

    pg3gpu_ctx *ctx = new (std::nothrow) pg3gpu_ctx;
    if (!ctx) return fail(nullptr, PG3GPU_ERR_OUT_OF_MEMORY, "host allocation failed");
    ctx->device = device;
    ctx->opts = *opts;
    ctx->W = scene->camera.width;
    ctx->H = scene->camera.height;
    ctx->nmat = scene->num_materials;
    ctx->kindMask = hs.kindMask;
    ctx->numPointLights = hs.numPointLights;
    auto bail = [&](int s) {
        g_createError = ctx->lastError;
        pg3gpu_destroy(ctx);
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(fail(ctx, PG3GPU_ERR_CUDA, "cudaSetDevice failed"));
    if (!forBatch) resolveNoallocScratch(device);

    SceneView &v = ctx->view;
    v = hs.view;   // camera, counts, options
    if ((st = upload(ctx, (float4 **)&v.tri, hs.tri))) return bail(st);
    if ((st = upload(ctx, (int **)&v.triMat, hs.triMat))) return bail(st);
    if ((st = upload(ctx, (float4 **)&v.sph, hs.sph))) return bail(st);
    if ((st = upload(ctx, (int **)&v.sphMat, hs.sphMat))) return bail(st);
    if ((st = upload(ctx, (DevMaterial **)&v.mats, hs.mats))) return bail(st);
    if ((st = upload(ctx, (int **)&v.mat2light, hs.mat2light))) return bail(st);
    if ((st = upload(ctx, (DevAreaLight **)&v.lights, hs.lights))) return bail(st);
    if (hs.emTexels) {
        // the caller's RGB texels to the device (a quarter less to copy than float4) and widened
        // there; the staging copy is freed once the kernel has run
        float4 *em = nullptr;
        float *rgb = nullptr;
        if ((st = devAlloc(ctx, &em, hs.emTexels))) return bail(st);
        if (cudaMalloc(&rgb, 3 * sizeof(float) * hs.emTexels) != cudaSuccess)
            return bail(fail(ctx, PG3GPU_ERR_OUT_OF_MEMORY, "environment map staging allocation failed"));
        cudaError_t e = cudaMemcpy(rgb, hs.emRgb, 3 * sizeof(float) * hs.emTexels, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = launchEmFromRgb(rgb, (uint32_t)hs.emTexels, em, nullptr);
        const cudaError_t ef = cudaFree(rgb);   // (waits for the kernel)
        if (e == cudaSuccess) e = ef;
        if (e != cudaSuccess) return bail(fail(ctx, PG3GPU_ERR_CUDA, "environment map upload: %s", cudaGetErrorString(e)));
        v.em = em;
    }
    if ((st = upload(ctx, (float **)&v.emMarg, hs.emMarg))) return bail(st);
    if ((st = upload(ctx, (float **)&v.emCond, hs.emCond))) return bail(st);
    {
        // padded to 12 floats: the device reads the 9 coefficients as three float4 (dot9)
        std::vector<float> sh = hs.bgShL;
        if (!sh.empty()) sh.resize(12, 0.f);
        if ((st = upload(ctx, (float **)&v.bgShL, sh))) return bail(st);
    }
    if (hs.hasSteer) {
        // geometry from the host build; the map-dependent weights are built on the device
        if ((st = uploadSteer(ctx, hs.steer, nullptr))) return bail(st);
    }
    if ((st = devAlloc(ctx, &ctx->dErr, 1))) return bail(st);
    if (cudaMemset(ctx->dErr, 0, sizeof(unsigned int)) != cudaSuccess) return bail(fail(ctx, PG3GPU_ERR_CUDA, "memset"));
    v.errorFlag = ctx->dErr;

    // acceleration structure
    const uint32_t nprim = v.ntri + v.nsph;
    if (nprim >= 2) {
        BvhNode *nodes;
        void *scratch;
        if ((st = devAlloc(ctx, &nodes, nprim - 1))) return bail(st);
        if ((st = devAlloc(ctx, (char **)&scratch, lbvhScratchBytes(nprim)))) return bail(st);
        if ((st = devAlloc(ctx, &ctx->dBvhCodes, nprim))) return bail(st);
        if ((st = devAlloc(ctx, &ctx->dBvhIds, nprim))) return bail(st);
        cudaError_t e = buildLbvh(v, nodes, scratch, ctx->dBvhCodes, ctx->dBvhIds, nullptr);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) return bail(fail(ctx, PG3GPU_ERR_CUDA, "LBVH build: %s", cudaGetErrorString(e)));
        v.bvh = nodes;
        v.bvhRoot = 0;
        ctx->dBvhBinary = nodes;
    }
    const int trav = opts->traversal;
    if (trav < PG3GPU_TRAVERSAL_AUTO || trav > PG3GPU_TRAVERSAL_BVH4)
        return bail(fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "unknown traversal %d", trav));
    // AUTO takes the binary LBVH above 32 primitives (the 4-wide tree measured 3% slower on the
    // 40968-triangle mesh); batch instances traverse the binary LBVH (the batch's query kernels
    // carry no wide traversal)
    const bool bvh = nprim >= 2 && (trav == PG3GPU_TRAVERSAL_BVH || trav == PG3GPU_TRAVERSAL_BVH4 ||
                                    (trav == PG3GPU_TRAVERSAL_AUTO && nprim > 32));
    const bool wide = bvh && !forBatch && trav == PG3GPU_TRAVERSAL_BVH4;
    v.useBvh = wide ? 2 : bvh ? 1 : 0;
    if (wide) {
        std::vector<BvhNode> bin(nprim - 1);
        if (cudaMemcpy(bin.data(), ctx->dBvhBinary, sizeof(BvhNode) * bin.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
            return bail(fail(ctx, PG3GPU_ERR_CUDA, "reading the LBVH"));
        std::vector<BvhNode4> w;
        if (!collapseBvh4(bin, w)) return bail(fail(ctx, PG3GPU_ERR_CUDA, "LBVH: malformed tree"));
        BvhNode4 *dw = nullptr;
        if ((st = upload(ctx, &dw, w))) return bail(st);
        v.bvh = reinterpret_cast<const BvhNode *>(dw);
    }

    if ((st = devAlloc(ctx, &ctx->dSum, (size_t)ctx->W * ctx->H * 3))) return bail(st);
    if ((st = devAlloc(ctx, &ctx->dSumsq, (size_t)ctx->W * ctx->H * 3))) return bail(st);
    if ((st = devAlloc(ctx, &ctx->dStats, 1))) return bail(st);
    if (cudaMemset(ctx->dSum, 0, sizeof(double) * ctx->W * ctx->H * 3) != cudaSuccess ||
        cudaMemset(ctx->dSumsq, 0, sizeof(double) * ctx->W * ctx->H * 3) != cudaSuccess ||
        cudaMemset(ctx->dStats, 0, sizeof(DevStats)) != cudaSuccess)
        return bail(fail(ctx, PG3GPU_ERR_CUDA, "memset"));

    int sms = 0, perSm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (megakernelOccupancy(opts->algorithm, &perSm) != cudaSuccess || perSm < 1)
        perSm = 1;
    ctx->megaGrid = sms * perSm;
    // the wavefront pipeline is the default for the NEE path tracer (3x the megakernel on the
    // benchmark scenes); the BSDF-only tracer always runs as a megakernel
    ctx->useWavefront = (opts->pipeline == PG3GPU_PIPELINE_WAVEFRONT || opts->pipeline == PG3GPU_PIPELINE_AUTO);
    ctx->waveGrid = sms * (1024 / PG3_WAVE_BLOCK);   // queues are allocated by the first launch (ensureWave)
    if (!forBatch) {
        if (cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess)
            return bail(fail(ctx, PG3GPU_ERR_CUDA, "event create"));
        for (int i = 0; i < pg3gpu_ctx::kTimerSlots; ++i)
            if (cudaEventCreate(&ctx->tStart[i]) != cudaSuccess || cudaEventCreate(&ctx->tStop[i]) != cudaSuccess)
                return bail(fail(ctx, PG3GPU_ERR_CUDA, "event create"));
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(ctx, PG3GPU_ERR_CUDA, "setup sync"));
    *out = ctx;
    return PG3GPU_OK;
}

extern "C" {

int pg3gpu_create(const pg3gpu_scene *scene, const pg3gpu_options *opts, int device, pg3gpu_ctx **out)
{
    return createContext(scene, opts, device, false, out);
}

int pg3gpu_set_stream(pg3gpu_ctx *ctx, void *stream)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    ctx->stream = reinterpret_cast<cudaStream_t>(stream);
    return PG3GPU_OK;
}

int pg3gpu_run_iteration(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (algorithm < PG3GPU_ALG_EYE_LIGHT || algorithm > PG3GPU_ALG_PATH_TRACING)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "unknown algorithm %d", (int)algorithm);
    if (spp == 0) return PG3GPU_OK;
    cudaSetDevice(ctx->device);
    if (callGraphEligible(ctx, algorithm, spp)) {
        if (int st = checkRenderable(ctx, algorithm)) return st;
        return runCallGraph(ctx, iteration, spp);
    }
    const uint32_t npix = ctx->W * ctx->H;
    const uint32_t per = passesPerChunk(ctx, spp);
    PG3_CUDA(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
    // A call of several chunks accumulates each chunk on a side stream while the next one renders
    // into the other output set; chunks are accumulated in order (one side stream), an output set
    // is rendered into again only after its accumulation, and the context's stream joins the side
    // stream at the end. Not while the stream is being captured.
    bool overlap = PG3_ACC_OVERLAP && spp > per;
    if (overlap) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        overlap = cudaStreamIsCapturing(ctx->stream, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
    }
    if (overlap && !ctx->accStream) {
        PG3_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->accStream, cudaStreamNonBlocking));
        for (int k = 0; k < 2; ++k) {
            PG3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evRendered[k], cudaEventDisableTiming));
            PG3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evAccumulated[k], cudaEventDisableTiming));
        }
        PG3_CUDA(ctx, cudaEventCreateWithFlags(&ctx->evAccJoin, cudaEventDisableTiming));
    }
    uint32_t chunk = 0;
    for (uint32_t done = 0; done < spp; done += per, ++chunk) {
        const uint32_t passes = std::min(per, spp - done);
        const int set = overlap ? (int)(chunk & 1) : 0;
        if (overlap && chunk >= 2) PG3_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->evAccumulated[set], 0));
        int st = renderChunk(ctx, algorithm, iteration + done, passes, set == 1);
        if (st) return st;
        float *const *out = set ? ctx->dOut2 : ctx->dOut;
        cudaStream_t accSt = ctx->stream;
        if (overlap) {
            PG3_CUDA(ctx, cudaEventRecord(ctx->evRendered[set], ctx->stream));
            PG3_CUDA(ctx, cudaStreamWaitEvent(ctx->accStream, ctx->evRendered[set], 0));
            accSt = ctx->accStream;
        }
        cudaError_t e = launchAccumulate(npix, passes, out[0], out[1], out[2], ctx->dSum, ctx->dSumsq, accSt);
        if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "accumulate: %s", cudaGetErrorString(e));
        if (overlap) PG3_CUDA(ctx, cudaEventRecord(ctx->evAccumulated[set], ctx->accStream));
        ctx->allLaunches += 1;
    }
    if (overlap) {
        PG3_CUDA(ctx, cudaEventRecord(ctx->evAccJoin, ctx->accStream));
        PG3_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->evAccJoin, 0));
    }
    PG3_CUDA(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
    ctx->timed = true;
    ctx->iterations += spp;
    return PG3GPU_OK;
}

int pg3gpu_synchronize(pg3gpu_ctx *ctx)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    PG3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    foldTimers(ctx);
    unsigned int flag = 0;
    PG3_CUDA(ctx, cudaMemcpy(&flag, ctx->dErr, sizeof flag, cudaMemcpyDeviceToHost));
    if (flag)
        return fail(ctx, PG3GPU_ERR_DEVICE_LIMIT,
                    "kernel limit flag 0x%x (1: BVH stack, 2: queue, 4: steerable descent, 16: estimator tree)", flag);
    return PG3GPU_OK;
}

int pg3gpu_render_samples(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp, float *out)
{
    if (!ctx || !out) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (algorithm < PG3GPU_ALG_EYE_LIGHT || algorithm > PG3GPU_ALG_PATH_TRACING)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "unknown algorithm %d", (int)algorithm);
    cudaSetDevice(ctx->device);
    const uint32_t npix = ctx->W * ctx->H;
    const uint32_t per = passesPerChunk(ctx, spp);
    std::vector<float> tmp[3];
    for (uint32_t done = 0; done < spp; done += per) {
        const uint32_t passes = std::min(per, spp - done);
        int st = renderChunk(ctx, algorithm, iteration + done, passes);
        if (st) return st;
        const size_t n = (size_t)passes * npix;
        for (int c = 0; c < 3; ++c) {
            tmp[c].resize(n);
            PG3_CUDA(ctx, cudaMemcpyAsync(tmp[c].data(), ctx->dOut[c], n * sizeof(float), cudaMemcpyDeviceToHost,
                                          ctx->stream));
        }
        PG3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        float *dst = out + (size_t)done * npix * 3;
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < 3; ++c) dst[i * 3 + c] = tmp[c][i];
    }
    return pg3gpu_synchronize(ctx);
}

int pg3gpu_read_framebuffer(pg3gpu_ctx *ctx, double *mean, double *var, uint64_t *iters)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    int st = pg3gpu_synchronize(ctx);
    if (st) return st;
    const size_t n = (size_t)ctx->W * ctx->H * 3;
    std::vector<double> s(n), q(var ? n : 0);
    PG3_CUDA(ctx, cudaMemcpy(s.data(), ctx->dSum, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (var) PG3_CUDA(ctx, cudaMemcpy(q.data(), ctx->dSumsq, n * sizeof(double), cudaMemcpyDeviceToHost));
    const double it = (double)ctx->iterations;
    for (size_t i = 0; i < n; ++i) {
        const double m = it > 0 ? s[i] / it : 0.0;   // GetFramebuffer scaling (src/renderer.hxx:255-262)
        if (mean) mean[i] = m;
        if (var) var[i] = it > 1 ? std::max(0.0, (q[i] - it * m * m) / (it - 1)) : 0.0;
    }
    if (iters) *iters = ctx->iterations;
    return PG3GPU_OK;
}

int pg3gpu_write_image(const double *rgb, uint32_t width, uint32_t height, const char *path, float gamma)
{
    std::string err;
    const int st = writeImage(rgb, width, height, path, gamma, err);
    return st ? fail(nullptr, st, "%s", err.c_str()) : PG3GPU_OK;
}

int pg3gpu_save_image(pg3gpu_ctx *ctx, const char *path, float gamma)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    std::vector<double> mean((size_t)ctx->W * ctx->H * 3);
    if (int st = pg3gpu_read_framebuffer(ctx, mean.data(), nullptr, nullptr)) return st;
    std::string err;
    const int st = writeImage(mean.data(), ctx->W, ctx->H, path, gamma, err);
    return st ? fail(ctx, st, "%s", err.c_str()) : PG3GPU_OK;
}

int pg3gpu_clear_framebuffer(pg3gpu_ctx *ctx)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    const size_t n = (size_t)ctx->W * ctx->H * 3 * sizeof(double);
    PG3_CUDA(ctx, cudaMemsetAsync(ctx->dSum, 0, n, ctx->stream));
    PG3_CUDA(ctx, cudaMemsetAsync(ctx->dSumsq, 0, n, ctx->stream));
    ctx->iterations = 0;
    return PG3GPU_OK;
}

uint64_t pg3gpu_iterations(const pg3gpu_ctx *ctx) { return ctx ? ctx->iterations : 0; }

int pg3gpu_get_stats(pg3gpu_ctx *ctx, pg3gpu_stats *out)
{
    if (!ctx || !out) return PG3GPU_ERR_INVALID_ARGUMENT;
    int st = pg3gpu_synchronize(ctx);
    if (st) return st;
    DevStats d;
    PG3_CUDA(ctx, cudaMemcpy(&d, ctx->dStats, sizeof d, cudaMemcpyDeviceToHost));
    out->paths = d.paths;
    out->extension_rays = d.extRays;
    out->shadow_rays = d.shadowRays;
    out->terminated_by_russian_roulette = d.byRR;
    out->terminated_by_background = d.byBackground;
    out->terminated_by_blocker = d.byBlocker;
    out->terminated_by_max_limit = d.byMax;
    out->terminated_by_safety_limit = d.bySafety;
    float ms = 0.f;
    if (ctx->timed && cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1) == cudaSuccess) out->last_iteration_ms = ms;
    else out->last_iteration_ms = 0.0;
    out->path_kernel_ms = ctx->kernelMs;
    out->path_kernel_launches = ctx->kernelLaunches;
    out->kernel_launches = ctx->allLaunches;
    for (int b = 0; b < kLenBins; ++b) out->length_histogram[b] = d.lenHist[b];
    out->min_path_length = d.minLenC ? ~d.minLenC : 0u;
    out->max_path_length = d.maxLen;
    return PG3GPU_OK;
}

int pg3gpu_reset_stats(pg3gpu_ctx *ctx)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    PG3_CUDA(ctx, cudaMemsetAsync(ctx->dStats, 0, sizeof(DevStats), ctx->stream));
    PG3_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    foldTimers(ctx);
    ctx->kernelMs = 0.0;
    ctx->kernelLaunches = 0;
    ctx->allLaunches = 0;
    return PG3GPU_OK;
}

int pg3gpu_device_framebuffer(pg3gpu_ctx *ctx, const double **sum, const double **sumsq)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (sum) *sum = ctx->dSum;
    if (sumsq) *sumsq = ctx->dSumsq;
    return PG3GPU_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Rendering without device allocations (no counterpart in the reference).
//
// For callers that may not allocate device memory once they are running -- a plugin inside
// a host application or engine whose device memory belongs to that host's own allocator, or
// a real-time loop with a fixed memory budget that must not fail for lack of memory half-way
// through a session. The per-sample radiance of a launch
// chunk lives in this file-scope array instead of a cudaMalloc'd buffer; every GPU on which a
// context is created holds it (12 MiB) from that first context until the process exits.
// ------------------------------------------------------------------------------------------
namespace {

constexpr uint32_t kNoAllocMaxPaths = PG3GPU_NOALLOC_MAX_PATHS;
static __device__ __align__(256) float g_noallocRadiance[3 * (size_t)kNoAllocMaxPaths];

constexpr int kNoAllocMaxDevices = 64;
float *g_noallocAddress[kNoAllocMaxDevices] = {};
std::string g_noallocError[kNoAllocMaxDevices];
std::mutex g_noallocMutex;

}  // namespace

// Looks up the scratch array's device address on `device` (which the caller has made current)
// once per device, when the first context on that device is created. In host code the array's
// name is a host-side stand-in, not a device address. This file has no kernels, so under lazy
// module loading the array's module -- and its 12 MiB -- is loaded by this lookup: doing it at
// context creation keeps the allocation-free call itself free of any module load or allocation.
// A failed lookup does not fail the context (the regular entry points do not need the array);
// the allocation-free call then reports the recorded reason.
void pg3::resolveNoallocScratch(int device)
{
    if (device < 0 || device >= kNoAllocMaxDevices) return;
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (g_noallocAddress[device]) return;
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocRadiance);
    if (e != cudaSuccess || !p) {
        g_noallocError[device] = std::string("cudaGetSymbolAddress of the scratch area: ") + cudaGetErrorString(e);
        cudaGetLastError();   // not sticky: clear it so the context's next call does not see it
        return;
    }
    g_noallocAddress[device] = static_cast<float *>(p);
}

namespace {

// The cached device address of the scratch array on ctx's device (looked up at context
// creation; no CUDA call here).
int noallocScratch(pg3gpu_ctx *ctx, float **out)
{
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return fail(ctx, PG3GPU_ERR_UNSUPPORTED, "device %d: no scratch slot", ctx->device);
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocAddress[ctx->device])
        return fail(ctx, PG3GPU_ERR_CUDA, "no scratch area on device %d: %s", ctx->device,
                    g_noallocError[ctx->device].empty() ? "not looked up" : g_noallocError[ctx->device].c_str());
    *out = g_noallocAddress[ctx->device];
    return PG3GPU_OK;
}

}  // namespace

extern "C" int pg3gpu_run_iteration_noalloc(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp,
                                            double *sum_rgb, double *sumsq_rgb)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (!sum_rgb || !sumsq_rgb) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "sum_rgb and sumsq_rgb are required");
    if (algorithm < PG3GPU_ALG_EYE_LIGHT || algorithm > PG3GPU_ALG_PATH_TRACING)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "unknown algorithm %d", (int)algorithm);
    const uint32_t npix = ctx->W * ctx->H;
    if (npix > kNoAllocMaxPaths)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT,
                    "image of %u pixels exceeds the %u-path scratch area of pg3gpu_run_iteration_noalloc", npix,
                    kNoAllocMaxPaths);
    if (algorithm == PG3GPU_ALG_PATH_TRACING && ctx->view.treeMode)
        return fail(ctx, PG3GPU_ERR_UNSUPPORTED,
                    "splitting / clipping keep frame stacks in device memory: use pg3gpu_run_iteration");
    if (int st = checkRenderable(ctx, algorithm)) return st;
    if (spp == 0) return PG3GPU_OK;
    PG3_CUDA(ctx, cudaSetDevice(ctx->device));
    float *scratch = nullptr;
    int st = noallocScratch(ctx, &scratch);
    if (st) return st;
    // Every scratch element the accumulation reads is written by the path kernel of the same
    // chunk first, so nothing in the (shared, persistent) scratch has to start at zero.
    float *r = scratch, *g = scratch + kNoAllocMaxPaths, *b = scratch + 2 * (size_t)kNoAllocMaxPaths;
    const uint32_t per = std::min(spp, kNoAllocMaxPaths / npix);
    for (uint32_t done = 0; done < spp; done += per) {
        const uint32_t passes = std::min(per, spp - done);
        cudaError_t e = launchMegakernel(ctx->view, algorithm, iteration + done, (uint64_t)passes * npix, npix, r, g, b,
                                         ctx->dStats, ctx->megaGrid, ctx->stream);
        if (e == cudaSuccess) e = launchAccumulate(npix, passes, r, g, b, sum_rgb, sumsq_rgb, ctx->stream);
        if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "allocation-free launch: %s", cudaGetErrorString(e));
    }
    return PG3GPU_OK;
}

// ------------------------------------------------------------------------------------------
// Sampler probes (test entry points; host arrays in and out, temporary device buffers)
// ------------------------------------------------------------------------------------------
namespace {

struct DevTemp {
    std::vector<void *> ptrs;
    ~DevTemp() { for (void *p : ptrs) cudaFree(p); }
    float *in(const float *h, size_t n, cudaError_t &e)
    {
        void *p = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(float));
        if (e == cudaSuccess) { ptrs.push_back(p); if (h) e = cudaMemcpy(p, h, n * sizeof(float), cudaMemcpyHostToDevice); }
        return (float *)p;
    }
};

int probeChecks(pg3gpu_ctx *ctx, uint32_t n)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (n == 0 || n > (1u << 26)) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "probe count must be in 1..2^26");
    cudaSetDevice(ctx->device);
    return PG3GPU_OK;
}

}  // namespace

extern "C" int pg3gpu_probe_bsdf(pg3gpu_ctx *ctx, int32_t material, uint32_t n, const float *wol, uint32_t seed,
                                 float *wil, float *pdf_sampled, float *pdf_eval, float *att_sampled, float *att_eval)
{
    int st = probeChecks(ctx, n);
    if (st) return st;
    if (material < 0 || (uint32_t)material >= ctx->nmat) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "material id");
    if (!wol || !wil || !pdf_sampled || !pdf_eval || !att_sampled || !att_eval)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "NULL probe array");
    cudaError_t e = cudaSuccess;
    DevTemp t;
    float *dWo = t.in(wol, 3 * (size_t)n, e), *dWi = t.in(nullptr, 3 * (size_t)n, e);
    float *dPs = t.in(nullptr, n, e), *dPe = t.in(nullptr, n, e);
    float *dAs = t.in(nullptr, 3 * (size_t)n, e), *dAe = t.in(nullptr, 3 * (size_t)n, e);
    if (e == cudaSuccess) e = launchProbeBsdf(ctx->view, material, n, dWo, seed, dWi, dPs, dPe, dAs, dAe, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(wil, dWi, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pdf_sampled, dPs, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pdf_eval, dPe, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(att_sampled, dAs, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(att_eval, dAe, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "bsdf probe: %s", cudaGetErrorString(e));
    return PG3GPU_OK;
}

extern "C" int pg3gpu_probe_bsdf_pdf(pg3gpu_ctx *ctx, int32_t material, uint32_t n, const float *wol, const float *wil,
                                     float *pdf, float *att)
{
    int st = probeChecks(ctx, n);
    if (st) return st;
    if (material < 0 || (uint32_t)material >= ctx->nmat) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "material id");
    if (!wol || !wil || !pdf) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "NULL probe array");
    cudaError_t e = cudaSuccess;
    DevTemp t;
    float *dWo = t.in(wol, 3 * (size_t)n, e), *dWi = t.in(wil, 3 * (size_t)n, e), *dP = t.in(nullptr, n, e);
    float *dA = att ? t.in(nullptr, n, e) : nullptr;
    if (e == cudaSuccess) e = launchProbeBsdfPdf(ctx->view, material, n, dWo, dWi, dP, dA, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(pdf, dP, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && att) e = cudaMemcpy(att, dA, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "bsdf pdf probe: %s", cudaGetErrorString(e));
    return PG3GPU_OK;
}

extern "C" int pg3gpu_probe_light(pg3gpu_ctx *ctx, int32_t light, uint32_t n, const float *points,
                                  const float *normals, uint32_t seed, float *dirs, float *pdf_sampled,
                                  float *pdf_eval, float *radiance_cos)
{
    int st = probeChecks(ctx, n);
    if (st) return st;
    if (light < 0 || (uint32_t)light >= ctx->view.lightCount) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "light id");
    if (!points || !normals || !dirs || !pdf_sampled || !pdf_eval || !radiance_cos)
        return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "NULL probe array");
    cudaError_t e = cudaSuccess;
    DevTemp t;
    float *dP = t.in(points, 3 * (size_t)n, e), *dN = t.in(normals, 3 * (size_t)n, e);
    float *dD = t.in(nullptr, 3 * (size_t)n, e), *dPs = t.in(nullptr, n, e), *dPe = t.in(nullptr, n, e);
    float *dR = t.in(nullptr, 3 * (size_t)n, e);
    if (e == cudaSuccess) e = launchProbeLight(ctx->view, light, n, dP, dN, seed, dD, dPs, dPe, dR, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(dirs, dD, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pdf_sampled, dPs, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pdf_eval, dPe, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(radiance_cos, dR, 12 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "light probe: %s", cudaGetErrorString(e));
    return pg3gpu_synchronize(ctx);
}

extern "C" int pg3gpu_probe_light_pdf(pg3gpu_ctx *ctx, int32_t light, uint32_t n, const float *points,
                                      const float *normals, const float *dirs, float *pdf)
{
    int st = probeChecks(ctx, n);
    if (st) return st;
    if (light < 0 || (uint32_t)light >= ctx->view.lightCount) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "light id");
    if (!points || !normals || !dirs || !pdf) return fail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "NULL probe array");
    cudaError_t e = cudaSuccess;
    DevTemp t;
    float *dP = t.in(points, 3 * (size_t)n, e), *dN = t.in(normals, 3 * (size_t)n, e);
    float *dD = t.in(dirs, 3 * (size_t)n, e), *dO = t.in(nullptr, n, e);
    if (e == cudaSuccess) e = launchProbeLightPdf(ctx->view, light, n, dP, dN, dD, dO, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(pdf, dO, 4 * (size_t)n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(ctx, PG3GPU_ERR_CUDA, "light pdf probe: %s", cudaGetErrorString(e));
    return PG3GPU_OK;
}

// LBVH export (test entry point): sorted Morton codes, primitive ids and the node array.
extern "C" int pg3gpu_export_bvh(pg3gpu_ctx *ctx, uint32_t *num_prims, uint32_t *codes, uint32_t *ids, float *nodes)
{
    if (!ctx || !num_prims) return PG3GPU_ERR_INVALID_ARGUMENT;
    const uint32_t n = ctx->view.ntri + ctx->view.nsph;
    *num_prims = n;
    if (n < 2 || (!codes && !ids && !nodes)) return PG3GPU_OK;
    PG3_CUDA(ctx, cudaSetDevice(ctx->device));
    if (codes) PG3_CUDA(ctx, cudaMemcpy(codes, ctx->dBvhCodes, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    if (ids) PG3_CUDA(ctx, cudaMemcpy(ids, ctx->dBvhIds, 4 * (size_t)n, cudaMemcpyDeviceToHost));
    if (nodes) PG3_CUDA(ctx, cudaMemcpy(nodes, ctx->dBvhBinary, sizeof(BvhNode) * (size_t)(n - 1), cudaMemcpyDeviceToHost));
    return PG3GPU_OK;
}
