// Differentiable rendering entry points of the C ABI (pg3gpu_set_params, pg3gpu_get_params,
// pg3gpu_diff_forward, pg3gpu_diff_adjoint; no counterpart in the reference): parameter
// updates on the device, the environment-map CDF rebuilt on the device, the forward pass that
// keeps each path's radiance, and the path-replay adjoint (stage code in pg3_wave.cuh).
#include <algorithm>
#include <cstring>
#include <vector>

#include "pg3_ctx.h"
#include "pg3_device.cuh"
#include "pg3_kernels.h"

using namespace pg3;

namespace {

constexpr uint32_t kMaxDiffMaterials = 2048;    // 16 bytes of shared memory per material per block
constexpr uint32_t kMaxCdfSide = 8192;          // one environment-map row in shared memory
constexpr int kCdfBlock = 256;

// Materials from (albedo rgb, alpha) per material; sampling data follow unless keep
// (the same rules as the scene setup: src/materials.hxx:262-266, 297-305, 791-806).
__global__ void setMaterialsKernel(DevMaterial *mats, uint32_t n, const float *p, int keep)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    DevMaterial m = mats[i];
    const float4 v = make_float4(p[4 * i], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]);
    if (m.kind == kMatLambert) {
        m.r = fmaxf(v.x, 0.f);
        m.g = fmaxf(v.y, 0.f);
        m.b = fmaxf(v.z, 0.f);
        m.zeroRefl = (m.r == 0.f && m.g == 0.f && m.b == 0.f) ? 1 : 0;
        if (!keep) {
            const float mx = fmaxf(m.r, fmaxf(m.g, m.b));
            const float q = fminf(fmaxf(0.15f * luminance(make_float3(m.r, m.g, m.b)) + 0.85f * mx, 0.f), 1.f);
            m.rrProb = fminf(fmaxf(q, 0.0f), 0.997f);
        }
    } else {
        m.alpha = fminf(fmaxf(v.w, 0.001f), 1.0f);
        if (!keep) m.alphaS = m.alpha;
    }
    mats[i] = m;
}

__global__ void setEnvKernel(float4 *em, uint32_t n, const float *t)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    em[i] = make_float4(fmaxf(t[3 * i], 0.f), fmaxf(t[3 * i + 1], 0.f), fmaxf(t[3 * i + 2], 0.f), 0.f);
}

// In-place inclusive prefix sum of a[0..n) in shared memory by one block: each thread sums a
// contiguous run, the run totals are scanned across warps, then each run is rescanned.
__device__ void blockInclusiveScan(float *a, uint32_t n)
{
    __shared__ float warpTotals[32];
    const uint32_t T = blockDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, nw = (T + 31) / 32;
    const uint32_t per = (n + T - 1) / T;
    const uint32_t b = min(n, t * per), e = min(n, b + per);
    float run = 0.f;
    for (uint32_t i = b; i < e; ++i) run += a[i];
    float x = run;
    for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, x, o);
        if ((int)lane >= o) x += y;
    }
    if (lane == 31) warpTotals[warp] = x;
    __syncthreads();
    if (warp == 0) {
        float v = lane < nw ? warpTotals[lane] : 0.f;
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(0xffffffffu, v, o);
            if ((int)lane >= o) v += y;
        }
        warpTotals[lane] = v;
    }
    __syncthreads();
    float acc = x - run + (warp > 0 ? warpTotals[warp - 1] : 0.f);
    for (uint32_t i = b; i < e; ++i) {
        acc += a[i];
        a[i] = acc;
    }
    __syncthreads();
}

// Luminance of texel (x, y) with the reference's wrap (NormalizeImgCoords, src/em_image.hxx:269-302).
__device__ float emLum(const float4 *em, int W, int H, int x, int y)
{
    int rx = x, ry = y;
    if (y >= H) { rx = x + W / 2; ry = H - 1; }
    else if (y < 0) { rx = x + W / 2; ry = 0; }
    int m = rx % W;
    if (m < 0) m += W;
    const float4 v = em[(size_t)ry * W + m];
    return luminance(make_float3(v.x, v.y, v.z));
}

// ComputeCdf (src/distribution.hxx:45-74) of one row of the sampler's function: the tent-filtered
// luminance times sin(theta_mid) (src/em_simple_spherical_sampler.hxx:117-152, src/em_image.hxx:152-183).
__global__ void __launch_bounds__(kCdfBlock) cdfRowsKernel(const float4 *em, uint32_t W, uint32_t H, float *cond,
                                                           float *rowInt)
{
    extern __shared__ float f[];
    const uint32_t r = blockIdx.x;
    const float s = sinf(kPiF * (r + 0.5f) / H);
    const float w0 = 1.f / 24.f, w1 = 2.f / 3.f;
    for (uint32_t c = threadIdx.x; c < W; c += blockDim.x) {
        const int x = (int)c, y = (int)r, iW = (int)W, iH = (int)H;
        float avg = emLum(em, iW, iH, x, y) * w1;
        avg += (emLum(em, iW, iH, x - 1, y - 1) + emLum(em, iW, iH, x - 1, y) + emLum(em, iW, iH, x - 1, y + 1) +
                emLum(em, iW, iH, x, y - 1) + emLum(em, iW, iH, x, y + 1) + emLum(em, iW, iH, x + 1, y - 1) +
                emLum(em, iW, iH, x + 1, y) + emLum(em, iW, iH, x + 1, y + 1)) *
               w0;
        f[c] = s * avg / (float)W;
    }
    __syncthreads();
    blockInclusiveScan(f, W);
    const float integral = f[W - 1];
    float *row = cond + (size_t)r * (W + 1);
    if (threadIdx.x == 0) {
        row[0] = 0.f;
        rowInt[r] = integral;
    }
    for (uint32_t c = threadIdx.x; c < W; c += blockDim.x)
        row[c + 1] = (integral == 0.f) ? (float)(c + 1) / W : f[c] / integral;
}

__global__ void __launch_bounds__(kCdfBlock) cdfMarginalKernel(const float *rowInt, uint32_t H, float *marg)
{
    extern __shared__ float f[];
    for (uint32_t r = threadIdx.x; r < H; r += blockDim.x) f[r] = rowInt[r] / (float)H;
    __syncthreads();
    blockInclusiveScan(f, H);
    const float integral = f[H - 1];
    if (threadIdx.x == 0) marg[0] = 0.f;
    for (uint32_t r = threadIdx.x; r < H; r += blockDim.x)
        marg[r + 1] = (integral == 0.f) ? (float)(r + 1) / H : f[r] / integral;
}

// Mean over the spp samples of each pixel (path index = sample * npix + pixel).
__global__ void meanImageKernel(uint32_t npix, uint32_t spp, const float *r, const float *g, const float *b,
                                float *img)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (uint32_t k = 0; k < spp; ++k) {
        const size_t i = (size_t)k * npix + p;
        s0 += r[i];
        s1 += g[i];
        s2 += b[i];
    }
    img[3 * (size_t)p] = (float)(s0 / spp);
    img[3 * (size_t)p + 1] = (float)(s1 / spp);
    img[3 * (size_t)p + 2] = (float)(s2 / spp);
}

int diffChecks(pg3gpu_ctx *ctx)
{
    if (ctx->opts.algorithm != PG3GPU_ALG_PATH_TRACING)
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "differentiable rendering needs algorithm 7 (path tracing)");
    if (!ctx->useWavefront)
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "differentiable rendering needs the wavefront pipeline");
    if (ctx->view.treeMode)
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "differentiable rendering does not split paths or clip");
    if (ctx->nmat > kMaxDiffMaterials)
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "differentiable rendering supports at most 2048 materials");
    if (ctx->kindMask & ~((1u << kMatLambert) | (1u << kMatGgxConductor) | (1u << kMatGgxDielectric)))
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED,
                        "differentiable rendering supports Lambert and GGX materials only (no Phong or smooth materials)");
    if (ctx->numPointLights)
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "differentiable rendering does not support point lights");
    return PG3GPU_OK;
}

int ensureDiffBuffers(pg3gpu_ctx *ctx, uint64_t paths)
{
    if (paths > ctx->totCapacity || !ctx->dTot[0]) {
        for (int c = 0; c < 3; ++c) {
            ctxFree(ctx, ctx->dTot[c]);
            ctxFree(ctx, ctx->dAdj[c]);
            ctx->dTot[c] = ctx->dAdj[c] = nullptr;
        }
        ctx->totCapacity = 0;
        for (int c = 0; c < 3; ++c) {
            if (int st = ctxAlloc(ctx, &ctx->dTot[c], paths)) return st;
            if (int st = ctxAlloc(ctx, &ctx->dAdj[c], paths)) return st;
        }
        ctx->totCapacity = paths;
    }
    const uint64_t cap = std::min<uint64_t>(paths, ctx->opts.max_paths_in_flight ? ctx->opts.max_paths_in_flight
                                                                                 : (1ull << 22));
    if (!ctx->dWaveGrad || ctx->waveGradCapacity < cap) {
        ctxFree(ctx, ctx->dWaveGrad);
        ctx->dWaveGrad = nullptr;
        char *w = nullptr;
        if (int st = ctxAlloc(ctx, &w, wavefrontBytes(cap, true))) return st;
        ctx->dWaveGrad = w;
        ctx->waveGradCapacity = cap;
    }
    return PG3GPU_OK;
}

}  // namespace

extern "C" int pg3gpu_set_params(pg3gpu_ctx *ctx, const float *mp, const float *et, uint32_t flags)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    const bool dev = (flags & PG3GPU_PARAMS_DEVICE) != 0, keep = (flags & PG3GPU_PARAMS_KEEP_SAMPLING) != 0;
    if (flags & ~(PG3GPU_PARAMS_DEVICE | PG3GPU_PARAMS_KEEP_SAMPLING))
        return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "unknown flags");
    const SceneView &v = ctx->view;
    const bool hasEm = v.bgKind == kBgEnvMap;
    if (et && !hasEm) return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "the scene has no environment map");
    const bool rebuild = et && !keep;
    if (rebuild && (v.emW > kMaxCdfSide || v.emH > kMaxCdfSide))
        return ctxError(ctx, PG3GPU_ERR_UNSUPPORTED, "device CDF rebuild supports maps up to 8192 texels a side");
    if (int st = cudaStatus(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return st;
    const uint32_t ntex = v.emW * v.emH;
    std::vector<void *> temps;
    auto stage = [&](const float *h, size_t n, const float **out) -> int {
        if (!h || dev) {
            *out = h;
            return PG3GPU_OK;
        }
        void *p = nullptr;
        if (int st = cudaStatus(ctx, cudaMalloc(&p, n * sizeof(float)), "cudaMalloc")) return st;
        temps.push_back(p);
        *out = static_cast<const float *>(p);
        return cudaStatus(ctx, cudaMemcpy(p, h, n * sizeof(float), cudaMemcpyHostToDevice), "parameter upload");
    };
    const float *dm = nullptr, *de = nullptr;
    int st = stage(mp, 4 * (size_t)ctx->nmat, &dm);
    if (!st) st = stage(et, 3 * (size_t)ntex, &de);
    if (!st && dm)
        setMaterialsKernel<<<(ctx->nmat + 127) / 128, 128, 0, ctx->stream>>>(const_cast<DevMaterial *>(v.mats),
                                                                            ctx->nmat, dm, keep ? 1 : 0);
    if (!st && de) {
        setEnvKernel<<<(ntex + 255) / 256, 256, 0, ctx->stream>>>(const_cast<float4 *>(v.em), ntex, de);
        if (rebuild && v.emSampler == kEmCdf) {   // CDF tables exist for the CDF sampler only
            if (!ctx->dRowInt) st = ctxAlloc(ctx, &ctx->dRowInt, v.emH);
            if (!st) {
                cdfRowsKernel<<<v.emH, kCdfBlock, v.emW * sizeof(float), ctx->stream>>>(
                    v.em, v.emW, v.emH, const_cast<float *>(v.emCond), ctx->dRowInt);
                cdfMarginalKernel<<<1, kCdfBlock, v.emH * sizeof(float), ctx->stream>>>(
                    ctx->dRowInt, v.emH, const_cast<float *>(v.emMarg));
            }
        }
        // the steerable sampler's weights (and with them the background's picking estimate)
        if (rebuild && !st && ctx->hasSteer)
            st = cudaStatus(ctx, launchSteerWeights(ctx->steerArgs, ctx->stream), "steerable build");
    }
    if (!st) st = cudaStatus(ctx, cudaGetLastError(), "parameter update");
    if (!temps.empty()) {
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        for (void *p : temps) cudaFree(p);
        if (!st) st = cudaStatus(ctx, e, "parameter update");
    }
    ctx->diffValid = false;
    return st;
}

extern "C" int pg3gpu_get_params(pg3gpu_ctx *ctx, float *mp, float *et)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (int st = cudaStatus(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return st;
    if (int st = cudaStatus(ctx, cudaStreamSynchronize(ctx->stream), "synchronize")) return st;
    const SceneView &v = ctx->view;
    if (mp) {
        std::vector<DevMaterial> m(ctx->nmat);
        if (int st = cudaStatus(ctx, cudaMemcpy(m.data(), v.mats, sizeof(DevMaterial) * m.size(), cudaMemcpyDeviceToHost),
                                "read materials"))
            return st;
        for (uint32_t i = 0; i < ctx->nmat; ++i) {
            const bool lam = m[i].kind == kMatLambert;
            mp[4 * i] = lam ? m[i].r : 0.f;
            mp[4 * i + 1] = lam ? m[i].g : 0.f;
            mp[4 * i + 2] = lam ? m[i].b : 0.f;
            mp[4 * i + 3] = lam ? 0.f : m[i].alpha;
        }
    }
    if (et) {
        if (v.bgKind != kBgEnvMap) return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "the scene has no environment map");
        std::vector<float4> t((size_t)v.emW * v.emH);
        if (int st = cudaStatus(ctx, cudaMemcpy(t.data(), v.em, sizeof(float4) * t.size(), cudaMemcpyDeviceToHost),
                                "read environment map"))
            return st;
        for (size_t i = 0; i < t.size(); ++i) {
            et[3 * i] = t[i].x;
            et[3 * i + 1] = t[i].y;
            et[3 * i + 2] = t[i].z;
        }
    }
    return PG3GPU_OK;
}

extern "C" int pg3gpu_diff_forward(pg3gpu_ctx *ctx, uint32_t iteration, uint32_t spp, float *image)
{
    if (!ctx || !image) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (spp == 0) return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "spp must be positive");
    if (int st = diffChecks(ctx)) return st;
    const uint32_t npix = ctx->W * ctx->H;
    const uint64_t paths = (uint64_t)npix * spp;
    if (paths > 0xffffffffull) return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "more than 2^32 paths");
    if (int st = cudaStatus(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return st;
    if (int st = ensureDiffBuffers(ctx, paths)) return st;
    GradArgs G{};
    G.adjoint = 0;
    G.sampleOffset = ctx->dSampleOffset;
    uint64_t launches = 0;
    cudaError_t e = launchWavefront(ctx->view, ctx->kindMask, iteration, paths, npix, ctx->dTot[0], ctx->dTot[1], ctx->dTot[2],
                                    ctx->dStats, ctx->dWaveGrad, ctx->waveGradCapacity, ctx->waveGrid, ctx->stream,
                                    &launches, &G);
    if (e == cudaSuccess) {
        meanImageKernel<<<(npix + 255) / 256, 256, 0, ctx->stream>>>(npix, spp, ctx->dTot[0], ctx->dTot[1],
                                                                      ctx->dTot[2], image);
        e = cudaGetLastError();
    }
    if (int st = cudaStatus(ctx, e, "differentiable forward")) return st;
    ctx->allLaunches += launches + 1;
    ctx->diffIteration = iteration;
    ctx->diffSpp = spp;
    ctx->diffValid = true;
    return PG3GPU_OK;
}

extern "C" int pg3gpu_diff_adjoint(pg3gpu_ctx *ctx, const float *dLdI, float *gMat, float *gEm)
{
    if (!ctx || !dLdI || !gMat) return PG3GPU_ERR_INVALID_ARGUMENT;
    if (int st = diffChecks(ctx)) return st;
    if (!ctx->diffValid)
        return ctxError(ctx, PG3GPU_ERR_INVALID_ARGUMENT,
                        "no forward to replay: call pg3gpu_diff_forward after the last parameter change");
    if (int st = cudaStatus(ctx, cudaSetDevice(ctx->device), "cudaSetDevice")) return st;
    const uint32_t npix = ctx->W * ctx->H;
    const uint64_t paths = (uint64_t)npix * ctx->diffSpp;
    GradArgs G{};
    G.dLdI = dLdI;
    G.invSpp = 1.f / (float)ctx->diffSpp;
    G.totR = ctx->dTot[0];
    G.totG = ctx->dTot[1];
    G.totB = ctx->dTot[2];
    G.gMat = gMat;
    G.gEm = (ctx->view.bgKind == kBgEnvMap) ? gEm : nullptr;
    G.adjoint = 1;
    G.sampleOffset = ctx->dSampleOffset;
    uint64_t launches = 0;
    const cudaError_t e = launchWavefront(ctx->view, ctx->kindMask, ctx->diffIteration, paths, npix, ctx->dAdj[0],
                                          ctx->dAdj[1], ctx->dAdj[2], ctx->dStats, ctx->dWaveGrad,
                                          ctx->waveGradCapacity, ctx->waveGrid, ctx->stream, &launches, &G);
    if (int st = cudaStatus(ctx, e, "adjoint")) return st;
    ctx->allLaunches += launches;
    return PG3GPU_OK;
}

extern "C" int pg3gpu_set_sample_offset(pg3gpu_ctx *ctx, const uint32_t *offset)
{
    if (!ctx) return PG3GPU_ERR_INVALID_ARGUMENT;
    ctx->dSampleOffset = offset;
    ctx->diffValid = false;
    return PG3GPU_OK;
}
