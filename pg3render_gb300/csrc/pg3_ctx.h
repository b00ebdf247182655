// Internal: the context behind the opaque pg3gpu_ctx handle of include/pg3gpu.h, shared by
// the translation units of the C ABI (pg3_api.cu, pg3_diff.cu, pg3_batch.cu).
#pragma once

#include <algorithm>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pg3gpu.h"
#include "pg3_kernels.h"
#include "pg3_scene_view.h"
#include "pg3_steerable.h"

struct pg3gpu_ctx {
    using SceneView = pg3::SceneView;
    using DevStats = pg3::DevStats;
    using TreeFrame = pg3::TreeFrame;
    int device = 0;
    cudaStream_t stream = nullptr;
    pg3gpu_options opts{};
    SceneView view{};
    std::vector<void *> allocs;
    std::vector<void *> pooled;          // allocations from the library's queue pool (pg3_api.cu)
    uint32_t W = 0, H = 0;
    uint32_t nmat = 0;
    uint32_t kindMask = 0;               // material kinds of the scene (bit per kind)
    uint32_t numPointLights = 0;
    uint32_t *dBvhCodes = nullptr, *dBvhIds = nullptr;   // sorted Morton codes / primitive ids of the LBVH
    const pg3::BvhNode *dBvhBinary = nullptr;             // its binary nodes (view.bvh may hold the 4-wide tree)
    double *dSum = nullptr, *dSumsq = nullptr;
    float *dOut[3] = {nullptr, nullptr, nullptr};
    uint64_t outCapacity = 0;            // paths per launch chunk
    // a second set of per-sample outputs and a side stream: a call of several chunks accumulates
    // chunk k into the framebuffer while chunk k + 1 renders (pg3gpu_run_iteration)
    float *dOut2[3] = {nullptr, nullptr, nullptr};
    uint64_t out2Capacity = 0;
    cudaStream_t accStream = nullptr;
    cudaEvent_t evRendered[2] = {nullptr, nullptr}, evAccumulated[2] = {nullptr, nullptr}, evAccJoin = nullptr;
    void *dWave = nullptr;               // wavefront queues
    uint64_t waveCapacity = 0;
    DevStats *dStats = nullptr;
    unsigned int *dErr = nullptr;
    uint64_t iterations = 0;
    int megaGrid = 0, waveGrid = 0;
    bool useWavefront = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    // per-launch timing of the path kernel: event pairs recorded around each launch,
    // folded into kernelMs when the stream is synchronised
    static constexpr int kTimerSlots = 64;
    cudaEvent_t tStart[kTimerSlots] = {}, tStop[kTimerSlots] = {};
    int pendingTimers = 0;
    double kernelMs = 0.0;
    uint64_t kernelLaunches = 0, allLaunches = 0;
    std::string lastError;

    // render graph of small calls (pg3gpu_run_iteration of one launch chunk): the whole chunk --
    // queues reset, camera rays, every bounce's stage kernels, accumulation -- captured once and
    // replayed per call with the call's first sample index set in its head node
    cudaStream_t graphStream = nullptr;
    cudaGraph_t callGraph = nullptr;
    cudaGraphExec_t callGraphExec = nullptr;
    cudaGraphNode_t callGraphHead = nullptr;
    uint32_t callGraphPasses = 0;
    uint64_t callGraphLaunches = 0;      // kernel launches one replay makes
    uint32_t *dCallBase = nullptr;       // device word: the replay's first sample index
    SceneView callGraphView{};           // the scene view the graph was captured with
    const void *callGraphBufs[6] = {};   // and its buffers (a change of either re-captures it)

    // recursive estimator (splitting / clipping): frame stacks of the megakernel's threads
    TreeFrame *dTree = nullptr;
    uint32_t treeDepth = 0;
    int treeGrid = 0;

    // differentiable rendering (pg3_diff.cu)
    float *dTot[3] = {nullptr, nullptr, nullptr};   // primal radiance of every path of the last forward
    float *dAdj[3] = {nullptr, nullptr, nullptr};   // radiance accumulators of the adjoint replay
    uint64_t totCapacity = 0;
    void *dWaveGrad = nullptr;                      // queues with gradient records
    uint64_t waveGradCapacity = 0;
    float *dRowInt = nullptr;                       // environment-map CDF build: per-row integrals
    bool hasSteer = false;                          // steerable sampler: its device build inputs/outputs
    pg3::SteerWeightArgs steerArgs{};
    std::shared_ptr<const pg3::SteerGeom> steerGeom;   // its geometry (host copy)
    std::vector<void *> steerAllocs;                // its device tables (replaced by an adaptive file)
    uint32_t diffIteration = 0, diffSpp = 0;        // samples the stored radiance belongs to
    const uint32_t *dSampleOffset = nullptr;        // caller's device word added to sample indices
    bool diffValid = false;
};

namespace pg3 {

// Records msg as the context's last error (or the thread's create error when ctx is null)
// and returns status.
int ctxError(pg3gpu_ctx *ctx, int status, const std::string &msg);

// pg3gpu_create; forBatch leaves out the launch queues, per-path outputs and timers.
int createContext(const pg3gpu_scene *scene, const pg3gpu_options *opts, int device, bool forBatch,
                  pg3gpu_ctx **out);

// Uploads a steerable sampler's geometry (replacing any earlier one of the context) and builds its
// weights on the device: from the context's map, or from vwHost (12 floats per vertex) when given.
int uploadSteer(pg3gpu_ctx *ctx, std::shared_ptr<const SteerGeom> geom, const float *vwHost);

// Looks up, once per device, the device address of the allocation-free entry point's scratch
// array (pg3_api.cu); `device` must be current.
void resolveNoallocScratch(int device);

inline int cudaStatus(pg3gpu_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return PG3GPU_OK;
    return ctxError(ctx, e == cudaErrorMemoryAllocation ? PG3GPU_ERR_OUT_OF_MEMORY : PG3GPU_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

// Device allocation owned by the context (freed by pg3gpu_destroy).
template <typename T>
int ctxAlloc(pg3gpu_ctx *ctx, T **p, size_t count)
{
    void *q = nullptr;
    const size_t bytes = std::max<size_t>(count * sizeof(T), 16);
    if (int st = cudaStatus(ctx, cudaMalloc(&q, bytes), "cudaMalloc")) return st;
    ctx->allocs.push_back(q);
    *p = reinterpret_cast<T *>(q);
    return PG3GPU_OK;
}

inline void ctxFree(pg3gpu_ctx *ctx, void *p)
{
    if (!p) return;
    cudaFree(p);
    ctx->allocs.erase(std::remove(ctx->allocs.begin(), ctx->allocs.end(), p), ctx->allocs.end());
}

}  // namespace pg3
