// Host-callable launchers of the device kernels (one translation unit each).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "pg3_scene_view.h"

namespace pg3 {

constexpr int kMegaBlock = 128;

// Threads per block of the wavefront stage kernels (a build option for occupancy sweeps).
#ifndef PG3_WAVE_BLOCK
#define PG3_WAVE_BLOCK 256
#endif

// pg3_megakernel.cu
// algorithm: an id of src/config.hxx:23-34 (0-7)
// tree / treeDepth: frames of the recursive estimator (algorithm 7 with S.treeMode), treeDepth
// per thread of the grid (gridBlocks x kMegaBlock threads)
cudaError_t launchMegakernel(const SceneView &S, int algorithm, uint32_t sample0, uint64_t numPaths, uint32_t npix,
                             float *outR, float *outG, float *outB, DevStats *stats, int gridBlocks,
                             cudaStream_t stream, TreeFrame *tree = nullptr, uint32_t treeDepth = 0);
cudaError_t megakernelOccupancy(int algorithm, int *blocksPerSm);
cudaError_t launchAccumulate(uint32_t npix, uint32_t passes, const float *r, const float *g, const float *b,
                             double *sum, double *sumsq, cudaStream_t stream);
// One thread stores `value` to *dst (the head node of a captured render graph, whose parameter
// each replay sets to the call's first sample index).
cudaError_t launchSetWord(uint32_t *dst, uint32_t value, cudaStream_t stream);
// n RGB texels (3 floats each) to float4 texels (alpha 0)
cudaError_t launchEmFromRgb(const float *rgb, uint32_t n, float4 *em, cudaStream_t stream);
const void *setWordKernelFunction();

// pg3_lbvh.cu
size_t lbvhScratchBytes(uint32_t numPrims);
cudaError_t buildLbvh(const SceneView &S, BvhNode *nodes, void *scratch, uint32_t *sortedCodesOut,
                      uint32_t *sortedIdsOut, cudaStream_t stream);

// pg3_wavefront.cu
// kindMask: bit k set when the scene has a material of kind k (shade kernels of absent kinds are
// not launched); grad: null renders; otherwise a primal replay (grad->adjoint == 0) or the
// adjoint pass
size_t wavefrontBytes(uint64_t capacity, bool grad);
cudaError_t launchWavefront(const SceneView &S, uint32_t kindMask, uint32_t sample0, uint64_t numPaths, uint32_t npix,
                            float *outR, float *outG, float *outB, DevStats *stats, void *scratch,
                            uint64_t capacity, int gridBlocks, cudaStream_t stream, uint64_t *launches,
                            const GradArgs *grad = nullptr, const uint32_t *sampleOffset = nullptr,
                            bool pdlInCapture = false);

// pg3_steer_build.cu: the steerable sampler's map-dependent tables from the device texels
constexpr uint32_t kSteerMaxLayers = 16;
struct SteerWeightArgs {
    const float4 *em;
    uint32_t emW, emH;
    const float4 *vdir;                          // geometry (pg3_steerable.cpp)
    uint32_t numVertices;
    const int4 *leafTri;
    const float *leafArea;
    uint32_t numLeaves;
    const int *nodeChild;
    uint32_t layerStart[kSteerMaxLayers + 1];    // tree layers bottom-up, node ranges
    uint32_t numLayers;
    float *vw, *leafW, *nodeW, *rootW;           // outputs (12 / 9 / 56 floats per item, 9)
    float2 *vlum;                                // output: per vertex (L(d_v), L(-d_v)) (pg3_steer.cuh)
    float4 *leafRec;                             // output: per leaf 5 float4 (SteerView::leafRec)
    // projected vertex luminance (PG3GPU_STEER_WEIGHTS_PROJECTED): the map projected onto the
    // triangulation's piecewise-linear hat functions; scratch of projScratchBytes(numVertices)
    // bytes and the leaf locator (the geometry part of the scene's SteerView)
    int projected;
    void *projScratch;
    SteerView locator;
};
size_t projScratchBytes(uint32_t numVertices);
cudaError_t launchSteerWeights(const SteerWeightArgs &args, cudaStream_t stream);
// The leaf, node and whole-sphere weights from vertex weights already in args.vw (read from a
// file), through their luminance.
cudaError_t launchSteerTreeWeights(const SteerWeightArgs &args, cudaStream_t stream);

// pg3_probe.cu (sampler probes for tests)
cudaError_t launchProbeBsdf(const SceneView &S, int mat, uint32_t n, const float *wol, uint32_t seed, float *wil,
                            float *pdfS, float *pdfE, float *attS, float *attE, cudaStream_t st);
cudaError_t launchProbeBsdfPdf(const SceneView &S, int mat, uint32_t n, const float *wol, const float *wil, float *pdf,
                               float *att, cudaStream_t st);
cudaError_t launchProbeLight(const SceneView &S, int light, uint32_t n, const float *pts, const float *nrms,
                             uint32_t seed, float *dirs, float *pdfS, float *pdfE, float *rad, cudaStream_t st);
cudaError_t launchProbeLightPdf(const SceneView &S, int light, uint32_t n, const float *pts, const float *nrms,
                                const float *dirs, float *pdf, cudaStream_t st);

}  // namespace pg3
