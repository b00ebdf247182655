// Sampler probes: the BSDF and light samplers of the path kernels run on their own,
// one sample per thread, so that tests can compare each sample's returned pdf with
// the pdf the evaluation path computes for the same direction, and histogram the
// directions against the evaluated density (chi-square).
#include "pg3_estimator.cuh"
#include "pg3_kernels.h"

namespace pg3 {

namespace {

__global__ void probeBsdfKernel(const __grid_constant__ SceneView S, int matId, uint32_t n, const float *wol,
                                uint32_t seed, float *wil, float *pdfS, float *pdfE, float *attS, float *attE)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const DevMaterial m = S.mats[matId];
    const float3 wo = make_float3(wol[3 * i], wol[3 * i + 1], wol[3 * i + 2]);
    const Rand4 r = philox(i, seed, 0xB5DFu, 1u, S.seedLo, S.seedHi);
    BsdfRec s;
    sampleBsdf(m, wo, r.b, r.c, r.d, s);
    BsdfRec e;
    evalBsdf(m, s.wil, wo, e);
    wil[3 * i] = s.wil.x; wil[3 * i + 1] = s.wil.y; wil[3 * i + 2] = s.wil.z;
    pdfS[i] = s.pdfW * s.compProb;
    pdfE[i] = e.pdfW * e.compProb;
    attS[3 * i] = s.att.x; attS[3 * i + 1] = s.att.y; attS[3 * i + 2] = s.att.z;
    attE[3 * i] = e.att.x; attE[3 * i + 1] = e.att.y; attE[3 * i + 2] = e.att.z;
}

__global__ void probeBsdfPdfKernel(const __grid_constant__ SceneView S, int matId, uint32_t n, const float *wol,
                                   const float *wil, float *pdf, float *att)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    BsdfRec e;
    evalBsdf(S.mats[matId], make_float3(wil[3 * i], wil[3 * i + 1], wil[3 * i + 2]),
             make_float3(wol[3 * i], wol[3 * i + 1], wol[3 * i + 2]), e);
    pdf[i] = e.pdfW * e.compProb;
    if (att) att[i] = maxc(e.att);
}

// Pdf of reaching the light along (pt, dir), as the emitter-hit MIS computes it.
__device__ float lightPdfAlong(const SceneView &S, int light, float3 pt, float3 nrm, float3 dir)
{
    if (light == S.bgLightId) {
        float pdf = 0.f;
        bgEmission(S, dir, true, frameFromZ(nrm), pdf);
        return pdf;
    }
    const DevAreaLight &L = S.lights[light];
    if (isPointLight(L)) return infF();   // a point light is reached by light sampling only
    const float3 p0 = xyz(L.p0_invArea), e1 = xyz(L.e1_r), e2 = xyz(L.e2_g);
    float t = 1e36f;
    const float3 nrmT = normalize(cross(e1, e2));
    if (!hitTriangle(make_float4(p0.x, p0.y, p0.z, nrmT.x), make_float4(p0.x + e1.x, p0.y + e1.y, p0.z + e1.z, nrmT.y),
                     make_float4(p0.x + e2.x, p0.y + e2.y, p0.z + e2.z, nrmT.z), pt, dir, 0.f, t))
        return 0.f;
    float pdf = 0.f;
    areaEmission(L, pt + dir * t, 1.f, pt, pdf);
    return pdf;
}

__global__ void probeLightKernel(const __grid_constant__ SceneView S, int light, uint32_t n, const float *pts,
                                 const float *nrms, uint32_t seed, float *dirs, float *pdfS, float *pdfE, float *rad)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float3 pt = make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    const float3 nrm = make_float3(nrms[3 * i], nrms[3 * i + 1], nrms[3 * i + 2]);
    const Frame f = frameFromZ(nrm);
    const Rand4 r = philox(i, seed, 0x11A7u, 0u, S.seedLo, S.seedHi);
    float3 wig, smp;
    float pdf = 0.f, dist;
    if (light == S.bgLightId) bgSample(S, f, r.b, r.c, r.d, wig, pdf, smp);
    else tableSample(S.lights[light], pt, nrm, r.b, r.c, wig, dist, smp, pdf);
    dirs[3 * i] = wig.x; dirs[3 * i + 1] = wig.y; dirs[3 * i + 2] = wig.z;
    pdfS[i] = pdf;
    pdfE[i] = lightPdfAlong(S, light, pt, nrm, wig);
    rad[3 * i] = smp.x; rad[3 * i + 1] = smp.y; rad[3 * i + 2] = smp.z;
}

__global__ void probeLightPdfKernel(const __grid_constant__ SceneView S, int light, uint32_t n, const float *pts,
                                    const float *nrms, const float *dirs, float *pdf)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pdf[i] = lightPdfAlong(S, light, make_float3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]),
                           make_float3(nrms[3 * i], nrms[3 * i + 1], nrms[3 * i + 2]),
                           make_float3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
}

}  // namespace

cudaError_t launchProbeBsdf(const SceneView &S, int mat, uint32_t n, const float *wol, uint32_t seed, float *wil,
                            float *pdfS, float *pdfE, float *attS, float *attE, cudaStream_t st)
{
    probeBsdfKernel<<<(n + 127) / 128, 128, 0, st>>>(S, mat, n, wol, seed, wil, pdfS, pdfE, attS, attE);
    return cudaGetLastError();
}
cudaError_t launchProbeBsdfPdf(const SceneView &S, int mat, uint32_t n, const float *wol, const float *wil, float *pdf,
                               float *att, cudaStream_t st)
{
    probeBsdfPdfKernel<<<(n + 127) / 128, 128, 0, st>>>(S, mat, n, wol, wil, pdf, att);
    return cudaGetLastError();
}
cudaError_t launchProbeLight(const SceneView &S, int light, uint32_t n, const float *pts, const float *nrms,
                             uint32_t seed, float *dirs, float *pdfS, float *pdfE, float *rad, cudaStream_t st)
{
    probeLightKernel<<<(n + 127) / 128, 128, 0, st>>>(S, light, n, pts, nrms, seed, dirs, pdfS, pdfE, rad);
    return cudaGetLastError();
}
cudaError_t launchProbeLightPdf(const SceneView &S, int light, uint32_t n, const float *pts, const float *nrms,
                                const float *dirs, float *pdf, cudaStream_t st)
{
    probeLightPdfKernel<<<(n + 127) / 128, 128, 0, st>>>(S, light, n, pts, nrms, dirs, pdf);
    return cudaGetLastError();
}

}  // namespace pg3
