// Device build of the steerable sampler's map-dependent tables (the geometry comes from the
// host, pg3_steerable.cpp): vertex weights, leaf weights, the 6-ary tree's node weights and the
// whole-sphere integral. It runs at context creation and whenever the environment map changes
// (differentiable rendering), so neither waits for a host pass over the map.
//
// vertex weight   vw[v][k]  = Y_k(d_v) * L(d_v)         (src/em_steerable_sampler.hxx:181-202, 3084-3095)
// leaf weight     lw[t][k]  = area_t * mean of its three vertex weights           (:1277-1296)
// node weight     nodeW[n][k][c] = the summed weight of child c                    (:3755-3793)
// whole sphere    rootW[k]  = sum over all leaves of lw[t][k]
// with Y the 9 real SH basis functions (Ramamoorthi & Hanrahan 2001) and L the luminance of
// the map's bilinear (tent) lookup in the vertex direction (src/em_image.hxx:95-143): the
// reference's point sample (PG3GPU_STEER_WEIGHTS_POINT). With PG3GPU_STEER_WEIGHTS_PROJECTED,
// L is instead the projection of the map's luminance onto the vertex's hat function phi_v (1 at
// the vertex, 0 at the other vertices, linear over each leaf's plane):
//   L_v = sum over texels t of lum_t dOmega_t phi_v(d_t) / sum over texels of dOmega_t phi_v(d_t)
// so that the piecewise-linear approximation keeps the energy of features smaller than a
// triangle (a sun between vertices), which point samples miss; the sampler's density and pdf
// stay exactly the ones of pg3_steer.cuh, only the vertex values change. A vertex whose hat
// function covers no texel centre keeps its point sample.
// Layouts for vector loads: a vertex's 9 weights padded to 12 floats (three float4), a node's
// weights coefficient-major over its 6 children, packed (54 floats padded to 14 float4).
// The sampler reads a vertex's value as L(d_v) times c(n) . Y(d_v), evaluated from the vertex
// direction (pg3_steer.cuh), so besides the weights the build writes per vertex the pair
// (L(d_v), L(-d_v)) (vlum; the antipode's luminance for the mirrored term of a uniform level),
// and the leaf weights are summed from L(d_v) Y(d_v) with the same float arithmetic as the vertex
// weights. Weights read from a file (launchSteerTreeWeights) enter through their luminance
// L = w_0 / Y_0; the reference's files hold weights of that form (tests/test_emssd.py).
#include <algorithm>
#include <climits>

#include "pg3_kernels.h"
#include "pg3_steer.cuh"

namespace pg3 {

namespace {

__device__ float texelLum(const float4 *em, uint32_t W, uint32_t H, int x, int y)
{
    // NormalizeImgCoords (src/em_image.hxx:269-302)
    int rx = x, ry = y;
    if (y >= (int)H) { rx = x + (int)W / 2; ry = (int)H - 1; }
    else if (y < 0) { rx = x + (int)W / 2; ry = 0; }
    int m = rx % (int)W;
    if (m < 0) m += (int)W;
    const float4 p = em[(size_t)ry * W + (size_t)m];
    return 0.212671f * p.x + 0.715160f * p.y + 0.072169f * p.z;
}

// Projection of the texels' luminance onto the hat functions of the leaf that contains each
// texel centre: acc[v] += lum dOmega phi_v, mass[v] += dOmega phi_v, summed in 64-bit fixed point
// so that the sums, and every render after them, do not depend on the order of the atomics.
// Scales: a term is at most maxLum * maxOmega (lum) or maxOmega (mass), a vertex sums at most
// W * H terms, so scale = 1e18 / (W * H * bound) keeps each sum below 2^63 with a resolution of
// 1e-12 of the largest term.
struct ProjScratch {
    unsigned long long *acc, *mass;   // nv each
    unsigned int *maxLumBits;         // max texel luminance (non-negative float bits)
};

__device__ float texelLumAt(const float4 *em, uint32_t i)
{
    const float4 p = em[i];
    return fmaxf(0.212671f * p.x + 0.715160f * p.y + 0.072169f * p.z, 0.f);
}

__global__ void maxLumKernel(const float4 *em, uint32_t n, unsigned int *maxLumBits)
{
    float m = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = fmaxf(m, texelLumAt(em, i));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxLumBits, __float_as_uint(m));   // non-negative: bits order as values
}

__device__ double projScale(uint32_t W, uint32_t H, double bound)
{
    return 1e18 / ((double)W * (double)H * fmax(bound, 1e-30));
}

__global__ void projectLumKernel(const float4 *em, uint32_t W, uint32_t H, SteerView T, const int4 *leafTri,
                                 ProjScratch P)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W * H) return;
    const uint32_t x = i % W, y = i / W;
    const float kPi = 3.14159265358979f;
    // inverse of the lat-long mapping of vertexWeightsKernel (u = 0.5 - atan2(y, x) / 2pi, v = theta / pi)
    const float theta = ((float)y + 0.5f) * (kPi / (float)H);
    const float phi = (((float)x + 0.5f) / (float)W - 0.5f) * (2.f * kPi);
    const float st = sinf(theta);
    const float3 d = make_float3(st * cosf(phi), -st * sinf(phi), cosf(theta));
    const double maxOmega = (2.0 * 3.14159265358979 / W) * (3.14159265358979 / H);
    const float dOmega = (2.f * kPi / (float)W) * (kPi / (float)H) * st;
    const float lum = texelLumAt(em, i);
    const int leaf = T.qtree ? steerLocateAdaptive(T, d) : steerLocate(T, d);
    if (leaf < 0 || (uint32_t)leaf >= T.numLeaves) return;
    const int4 tri = leafTri[leaf];
    const float3 A = xyz(T.vdir[tri.x]), B = xyz(T.vdir[tri.y]), C = xyz(T.vdir[tri.z]);
    const float3 n = cross(B - A, C - A);
    const float nn = dot(n, n);
    const float dn = dot(n, d);
    if (!(nn > 0.f) || !(dn > 0.f)) return;
    const float3 q = d * (dot(n, A) / dn);          // d meets the leaf's plane
    float b[3];
    b[0] = fmaxf(dot(cross(B - q, C - q), n) / nn, 0.f);
    b[1] = fmaxf(dot(cross(C - q, A - q), n) / nn, 0.f);
    b[2] = fmaxf(1.f - b[0] - b[1], 0.f);
    const float bs = b[0] + b[1] + b[2];
    if (!(bs > 0.f)) return;
    const double maxLum = (double)__uint_as_float(*P.maxLumBits);
    const double sA = projScale(W, H, maxLum * maxOmega), sM = projScale(W, H, maxOmega);
    const int v[3] = {tri.x, tri.y, tri.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double w = (double)dOmega * (double)(b[k] / bs);
        atomicAdd(&P.acc[v[k]], (unsigned long long)(w * (double)lum * sA + 0.5));
        atomicAdd(&P.mass[v[k]], (unsigned long long)(w * sM + 0.5));
    }
}

// L Y_k(d) for the 9 real SH basis functions (the vertex weight of luminance L at direction d)
__device__ void shWeights(float L, float4 d, float *o)
{
    const float x = d.x, y = d.y, z = d.z;
    o[0] = L * 0.282095f;
    o[1] = L * 0.488603f * y;
    o[2] = L * 0.488603f * z;
    o[3] = L * 0.488603f * x;
    o[4] = L * 1.092548f * x * y;
    o[5] = L * 1.092548f * y * z;
    o[6] = L * 0.315392f * (3.f * z * z - 1.f);
    o[7] = L * 1.092548f * x * z;
    o[8] = L * 0.546274f * (x * x - y * y);
}

__global__ void vertexWeightsKernel(const float4 *em, uint32_t W, uint32_t H, const float4 *vdir, uint32_t nv,
                                    ProjScratch proj, int useProj, float *vw, float2 *vlum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const float4 d = vdir[i];
    const float kPi = 3.14159265358979f;
    const float phi = -atan2f(d.y, d.x);
    const float theta = acosf(fminf(fmaxf(d.z, -1.f), 1.f));
    const float u = fminf(fmaxf(0.5f + phi * 0.5f * (1.f / kPi), 0.f), 1.f);
    const float v = fminf(fmaxf(theta * (1.f / kPi), 0.f), 1.f);
    const float xf = u * (float)W, yf = v * (float)H;
    const int cx = (int)(xf + 0.5f), cy = (int)(yf + 0.5f);
    const int x0 = cx - 1, y0 = cy - 1;
    const float xl = xf - ((float)x0 + 0.5f), yl = yf - ((float)y0 + 0.5f);
    const float top = (1.f - xl) * texelLum(em, W, H, x0, y0) + xl * texelLum(em, W, H, cx, y0);
    const float bot = (1.f - xl) * texelLum(em, W, H, x0, cy) + xl * texelLum(em, W, H, cx, cy);
    float L = (1.f - yl) * top + yl * bot;
    if (useProj && proj.mass[i] > 0ull) {
        const double maxOmega = (2.0 * 3.14159265358979 / W) * (3.14159265358979 / H);
        const double maxLum = (double)__uint_as_float(*proj.maxLumBits);
        const double a = (double)proj.acc[i] / projScale(W, H, maxLum * maxOmega);
        const double m = (double)proj.mass[i] / projScale(W, H, maxOmega);
        L = (float)(a / m);
    }
    float *o = vw + 12 * (size_t)i;
    shWeights(L, d, o);
    o[9] = o[10] = o[11] = 0.f;
    vlum[i].x = L;
}

// The luminance of weights read from a file: w_0 = L Y_0.
__global__ void lumFromWeightsKernel(const float *vw, uint32_t nv, float2 *vlum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) vlum[i].x = vw[12 * (size_t)i] / 0.282095f;
}

// Leaf records: the corners with their luminance, the antipodes' luminance, the plane.
__global__ void leafRecordKernel(const int4 *leafTri, const float4 *vdir, const float2 *vlum, const float4 *leafPlane,
                                 uint32_t nLeaf, float4 *rec)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nLeaf) return;
    const int4 t = leafTri[i];
    const float2 la = vlum[t.x], lb = vlum[t.y], lc = vlum[t.z];
    const float4 A = vdir[t.x], B = vdir[t.y], C = vdir[t.z];
    float4 *r = rec + 5 * (size_t)i;
    r[0] = make_float4(A.x, A.y, A.z, la.x);
    r[1] = make_float4(B.x, B.y, B.z, lb.x);
    r[2] = make_float4(C.x, C.y, C.z, lc.x);
    r[3] = make_float4(la.y, lb.y, lc.y, 0.f);
    r[4] = leafPlane[i];
}

// The antipode's luminance (uniform levels: vdir.w holds the antipodal vertex; adaptive: -1).
__global__ void antipodeLumKernel(const float4 *vdir, uint32_t nv, float2 *vlum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nv) return;
    const int a = __float_as_int(vdir[i].w);
    vlum[i].y = (a >= 0 && (uint32_t)a < nv) ? vlum[a].x : 0.f;
}

__global__ void leafWeightsKernel(const int4 *leafTri, const float *leafArea, uint32_t nLeaf, const float4 *vdir,
                                  const float2 *vlum, float *lw)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nLeaf) return;
    const int4 t = leafTri[i];
    const float a = leafArea[i] * (1.f / 3.f);
    float wa[9], wb[9], wc[9];
    shWeights(vlum[t.x].x, vdir[t.x], wa);
    shWeights(vlum[t.y].x, vdir[t.y], wb);
    shWeights(vlum[t.z].x, vdir[t.z], wc);
#pragma unroll
    for (int k = 0; k < 9; ++k) lw[9 * (size_t)i + k] = a * (wa[k] + wb[k] + wc[k]);
}

constexpr int kNodeFloats = 4 * kSteerNodeVec4;   // a tree node's weights (pg3_steer.cuh)

// One tree layer: every child slot of nodes [n0, n1) gets its child's summed weight (a leaf's
// weight, or the sum of a lower node's child slots, written by the previous launch).
__global__ void treeLayerKernel(const int *nodeChild, uint32_t n0, uint32_t n1, const float *lw, float *nodeW)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= 8 * (n1 - n0)) return;
    const uint32_t n = n0 + j / 8, c = j % 8;
    if (c >= 6) return;   // slots 6 and 7 are never used (6-ary tree)
    const int ch = nodeChild[8 * (size_t)n + c];
    float w[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[k] = 0.f;
    if (ch != INT_MIN) {
        if (ch < 0) {
#pragma unroll
            for (int k = 0; k < 9; ++k) w[k] = lw[9 * (size_t)(~ch) + k];
        } else {
            for (int cc = 0; cc < 6; ++cc)
#pragma unroll
                for (int k = 0; k < 9; ++k) w[k] += nodeW[kNodeFloats * (size_t)ch + 6 * k + cc];
        }
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) nodeW[kNodeFloats * (size_t)n + 6 * k + c] = w[k];
    if (c == 0) {
        // the record's tail: the first child and the number of children (the tree is built over
        // consecutive items, so the children are first, first + 1, ... or ~first, ~first - 1, ...)
        int count = 0;
        for (int cc = 0; cc < 6; ++cc) count += nodeChild[8 * (size_t)n + cc] != INT_MIN;
        nodeW[kNodeFloats * (size_t)n + 54] = __int_as_float(ch);
        nodeW[kNodeFloats * (size_t)n + 55] = __int_as_float(count);
    }
}

// Whole-sphere weights: one block, fp64 partial sums over all leaves.
__global__ void rootWeightsKernel(const float *lw, uint32_t nLeaf, float *rootW)
{
    __shared__ double part[9][256];
    double acc[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) acc[k] = 0.0;
    for (uint32_t i = threadIdx.x; i < nLeaf; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < 9; ++k) acc[k] += lw[9 * (size_t)i + k];
#pragma unroll
    for (int k = 0; k < 9; ++k) part[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (uint32_t s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
#pragma unroll
            for (int k = 0; k < 9; ++k) part[k][threadIdx.x] += part[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 9) rootW[threadIdx.x] = (float)part[threadIdx.x][0];
}

}  // namespace

size_t projScratchBytes(uint32_t numVertices) { return 16 * (size_t)numVertices + 16; }

namespace {
// The antipodes' luminance, the leaf, node and whole-sphere weights from the vertex luminance.
cudaError_t treeWeights(const SteerWeightArgs &a, cudaStream_t st);
}  // namespace

cudaError_t launchSteerWeights(const SteerWeightArgs &a, cudaStream_t st)
{
    if (!a.em || !a.vdir || !a.vw || (a.projected && !a.projScratch)) return cudaErrorInvalidValue;
    // projScratch: acc[nv], mass[nv] (64-bit), the max-luminance word; passed to the kernels by
    // value (no host-side record, so the build can be captured into a CUDA graph)
    ProjScratch P{};
    if (a.projected) {
        P.acc = reinterpret_cast<unsigned long long *>(a.projScratch);
        P.mass = P.acc + a.numVertices;
        P.maxLumBits = reinterpret_cast<unsigned int *>(P.mass + a.numVertices);
        const cudaError_t e = cudaMemsetAsync(a.projScratch, 0, projScratchBytes(a.numVertices), st);
        if (e != cudaSuccess) return e;
        const uint32_t texels = a.emW * a.emH;
        maxLumKernel<<<std::min<uint32_t>((texels + 255) / 256, 1024), 256, 0, st>>>(a.em, texels, P.maxLumBits);
        projectLumKernel<<<(texels + 255) / 256, 256, 0, st>>>(a.em, a.emW, a.emH, a.locator, a.leafTri, P);
    }
    vertexWeightsKernel<<<(a.numVertices + 127) / 128, 128, 0, st>>>(a.em, a.emW, a.emH, a.vdir, a.numVertices,
                                                                     P, a.projected, a.vw, a.vlum);
    return treeWeights(a, st);
}

cudaError_t launchSteerTreeWeights(const SteerWeightArgs &a, cudaStream_t st)
{
    if (!a.vw || !a.vlum) return cudaErrorInvalidValue;
    lumFromWeightsKernel<<<(a.numVertices + 127) / 128, 128, 0, st>>>(a.vw, a.numVertices, a.vlum);
    return treeWeights(a, st);
}

namespace {
cudaError_t treeWeights(const SteerWeightArgs &a, cudaStream_t st)
{
    if (!a.leafTri || !a.leafArea || !a.nodeChild || !a.vdir || !a.vlum || !a.leafRec || !a.locator.leafPlane ||
        !a.leafW || !a.nodeW || !a.rootW || a.numLayers == 0 || a.numLayers > kSteerMaxLayers)
        return cudaErrorInvalidValue;
    antipodeLumKernel<<<(a.numVertices + 127) / 128, 128, 0, st>>>(a.vdir, a.numVertices, a.vlum);
    leafRecordKernel<<<(a.numLeaves + 127) / 128, 128, 0, st>>>(a.leafTri, a.vdir, a.vlum, a.locator.leafPlane,
                                                               a.numLeaves, a.leafRec);
    leafWeightsKernel<<<(a.numLeaves + 127) / 128, 128, 0, st>>>(a.leafTri, a.leafArea, a.numLeaves, a.vdir, a.vlum,
                                                                a.leafW);
    for (uint32_t l = 0; l < a.numLayers; ++l) {
        const uint32_t n0 = a.layerStart[l], n1 = a.layerStart[l + 1];
        if (n1 <= n0) return cudaErrorInvalidValue;
        treeLayerKernel<<<(8 * (n1 - n0) + 127) / 128, 128, 0, st>>>(a.nodeChild, n0, n1, a.leafW, a.nodeW);
    }
    rootWeightsKernel<<<1, 256, 0, st>>>(a.leafW, a.numLeaves, a.rootW);
    return cudaGetLastError();
}
}  // namespace

}  // namespace pg3
