// Megakernel pipeline: one thread carries one camera path from the camera to
// its last vertex, then writes its radiance to the per-sample buffer.
//
// Launch shape: a persistent grid (SM count x resident blocks per SM) striding
// over path indices; consecutive threads take consecutive pixels of the same
// sample pass, so neighbouring lanes start with nearly identical primary rays.
#include "pg3_estimator.cuh"
#include "pg3_kernels.h"

namespace pg3 {

PG3_DI void flushCounters(DevStats *st, const PathCounters &c, uint32_t paths)
{
    const unsigned mask = __activemask();
    const uint32_t vals[8] = {paths, c.ext, c.shadow, c.rr, c.bg, c.blocker, c.maxl, c.safety};
    unsigned long long *dst = &st->paths;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t s = __reduce_add_sync(mask, vals[i]);
        if ((threadIdx.x & 31) == (__ffs(mask) - 1) && s) atomicAdd(dst + i, (unsigned long long)s);
    }
}

// KIND: 0 NEE+MIS path tracer (algorithm 7), 1 naive path tracer (6), 2 one-hit estimators (0-5),
// 3 the recursive estimator with splitting / clipping (algorithm 7; `tree` holds treeDepth
// frames per thread of the grid)
template <int KIND>
__global__ void __launch_bounds__(kMegaBlock) megakernel(const __grid_constant__ SceneView S, int alg,
                                                         uint32_t sample0, uint64_t numPaths, uint32_t npix,
                                                         float *__restrict__ outR, float *__restrict__ outG,
                                                         float *__restrict__ outB, DevStats *stats, TreeFrame *tree,
                                                         uint32_t treeDepth)
{
    TreeFrame *myStack = (KIND == 3) ? tree + (size_t)(blockIdx.x * blockDim.x + threadIdx.x) * treeDepth : nullptr;
    PathCounters pc;
    uint32_t done = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < numPaths; i += stride) {
        const uint32_t pixel = (uint32_t)(i % npix);
        const uint32_t sample = sample0 + (uint32_t)(i / npix);
        const float3 L = (KIND == 1)   ? tracePathNaive(S, pixel, sample, pc)
                         : (KIND == 2) ? traceDirect(S, alg, pixel, sample, pc)
                         : (KIND == 3) ? traceTree(S, pixel, sample, pc, myStack, treeDepth)
                                       : tracePath(S, pixel, sample, pc);
        outR[i] = L.x;
        outG[i] = L.y;
        outB[i] = L.z;
        ++done;
    }
    flushCounters(stats, pc, done);
}

// Adds `passes` samples per pixel from the per-sample buffer into the fp64
// framebuffer accumulators (sum and sum of squares).
__global__ void __launch_bounds__(256) accumulateKernel(uint32_t npix, uint32_t passes, const float *__restrict__ inR,
                                                         const float *__restrict__ inG, const float *__restrict__ inB,
                                                         double *__restrict__ sum, double *__restrict__ sumsq)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    // every sample is added in fp64, as the reference's framebuffer adds each iteration's
    // radiance (src/frame_buffer.hxx:30-77): the sum of identical samples stays exact
    double s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    for (uint32_t k = 0; k < passes; ++k) {
        const size_t idx = (size_t)k * npix + p;
        const double v[3] = {inR[idx], inG[idx], inB[idx]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            s[c] += v[c];
            q[c] = fma(v[c], v[c], q[c]);
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        sum[(size_t)p * 3 + c] += s[c];
        sumsq[(size_t)p * 3 + c] += q[c];
    }
}

__global__ void setWordKernel(uint32_t *dst, uint32_t value) { *dst = value; }

cudaError_t launchSetWord(uint32_t *dst, uint32_t value, cudaStream_t stream)
{
    setWordKernel<<<1, 1, 0, stream>>>(dst, value);
    return cudaGetLastError();
}

const void *setWordKernelFunction() { return reinterpret_cast<const void *>(setWordKernel); }

// RGB texels (3 floats each, as the caller passes them) to the float4 texels the kernels read.
__global__ void emFromRgbKernel(const float *rgb, uint32_t n, float4 *em)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        em[i] = make_float4(rgb[3 * (size_t)i], rgb[3 * (size_t)i + 1], rgb[3 * (size_t)i + 2], 0.f);
}

cudaError_t launchEmFromRgb(const float *rgb, uint32_t n, float4 *em, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 4096);
    emFromRgbKernel<<<blocks, 256, 0, stream>>>(rgb, n, em);
    return cudaGetLastError();
}

cudaError_t launchMegakernel(const SceneView &S, int algorithm, uint32_t sample0, uint64_t numPaths, uint32_t npix,
                             float *outR, float *outG, float *outB, DevStats *stats, int gridBlocks,
                             cudaStream_t stream, TreeFrame *tree, uint32_t treeDepth)
{
    if (algorithm == 7 && S.treeMode) {
        if (!tree || treeDepth == 0) return cudaErrorInvalidValue;
        megakernel<3><<<gridBlocks, kMegaBlock, 0, stream>>>(S, algorithm, sample0, numPaths, npix, outR, outG, outB,
                                                            stats, tree, treeDepth);
    } else if (algorithm == 6)
        megakernel<1><<<gridBlocks, kMegaBlock, 0, stream>>>(S, algorithm, sample0, numPaths, npix, outR, outG, outB, stats,
                                                            nullptr, 0);
    else if (algorithm == 7)
        megakernel<0><<<gridBlocks, kMegaBlock, 0, stream>>>(S, algorithm, sample0, numPaths, npix, outR, outG, outB, stats,
                                                            nullptr, 0);
    else
        megakernel<2><<<gridBlocks, kMegaBlock, 0, stream>>>(S, algorithm, sample0, numPaths, npix, outR, outG, outB, stats,
                                                            nullptr, 0);
    return cudaGetLastError();
}

cudaError_t megakernelOccupancy(int algorithm, int *blocksPerSm)
{
    if (algorithm == 6) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, megakernel<1>, kMegaBlock, 0);
    if (algorithm == 7) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, megakernel<0>, kMegaBlock, 0);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocksPerSm, megakernel<2>, kMegaBlock, 0);
}

cudaError_t launchAccumulate(uint32_t npix, uint32_t passes, const float *r, const float *g, const float *b,
                             double *sum, double *sumsq, cudaStream_t stream)
{
    accumulateKernel<<<(npix + 255) / 256, 256, 0, stream>>>(npix, passes, r, g, b, sum, sumsq);
    return cudaGetLastError();
}

}  // namespace pg3
