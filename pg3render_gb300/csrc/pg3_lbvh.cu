// Linear BVH built on the device (the reference has no acceleration structure:
// it loops over all primitives, src/scene_graph.hxx:33-82).
//
//  1. primBounds:   per-primitive AABB and centroid (triangles: vertex min/max;
//                   spheres: centre -/+ radius), centroid = (lo + hi) / 2.
//  2. mortonCodes:  30-bit codes of the centroids quantised to 10 bits per axis
//                   inside the centroid bounds.
//  3. radix sort:   stable LSD sort of (code, primitive id), 4 passes of 8 bits
//                   (block histogram, digit-major exclusive scan, stable scatter).
//  4. karras:       one internal node per sorted position (Karras, "Maximizing
//                   Parallelism in the Construction of BVHs, Octrees, and k-d
//                   Trees", HPG 2012), with equal codes ordered by position.
//  5. refit:        leaves to root; each parent is finished by whichever of its
//                   two children arrives second (atomic counter per node).
// Every floating-point step uses explicitly rounded intrinsics (no contraction),
// and min/max are exact, so the result is bit-identical to a CPU build of the
// same steps (checked against oracle's lbvh build in the tests).
#include <cstdint>

#include "pg3_device.cuh"
#include "pg3_kernels.h"

namespace pg3 {

namespace {

constexpr int kSortBlock = 256;   // elements per radix tile (one per thread)

__device__ __forceinline__ uint32_t expandBits10(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void primBounds(SceneView S, float4 *lo, float4 *hi, float4 *cen)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = S.ntri + S.nsph;
    if (i >= n) return;
    float3 a, b;
    if (i < S.ntri) {
        const float4 p0 = S.tri[3 * i], p1 = S.tri[3 * i + 1], p2 = S.tri[3 * i + 2];
        a = make_float3(fminf(fminf(p0.x, p1.x), p2.x), fminf(fminf(p0.y, p1.y), p2.y), fminf(fminf(p0.z, p1.z), p2.z));
        b = make_float3(fmaxf(fmaxf(p0.x, p1.x), p2.x), fmaxf(fmaxf(p0.y, p1.y), p2.y), fmaxf(fmaxf(p0.z, p1.z), p2.z));
    } else {
        const float4 s = S.sph[i - S.ntri];
        a = make_float3(__fsub_rn(s.x, s.w), __fsub_rn(s.y, s.w), __fsub_rn(s.z, s.w));
        b = make_float3(__fadd_rn(s.x, s.w), __fadd_rn(s.y, s.w), __fadd_rn(s.z, s.w));
    }
    lo[i] = make_float4(a.x, a.y, a.z, 0.f);
    hi[i] = make_float4(b.x, b.y, b.z, 0.f);
    cen[i] = make_float4(__fmul_rn(__fadd_rn(a.x, b.x), 0.5f), __fmul_rn(__fadd_rn(a.y, b.y), 0.5f),
                         __fmul_rn(__fadd_rn(a.z, b.z), 0.5f), 0.f);
}

// Centroid bounds by one block (n is a primitive count; a single block streams it).
__global__ void centroidBounds(const float4 *cen, uint32_t n, float4 *out)
{
    __shared__ float sm[6][256];
    float lx = 3.4e38f, ly = 3.4e38f, lz = 3.4e38f, hx = -3.4e38f, hy = -3.4e38f, hz = -3.4e38f;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const float4 c = cen[i];
        lx = fminf(lx, c.x); ly = fminf(ly, c.y); lz = fminf(lz, c.z);
        hx = fmaxf(hx, c.x); hy = fmaxf(hy, c.y); hz = fmaxf(hz, c.z);
    }
    sm[0][threadIdx.x] = lx; sm[1][threadIdx.x] = ly; sm[2][threadIdx.x] = lz;
    sm[3][threadIdx.x] = hx; sm[4][threadIdx.x] = hy; sm[5][threadIdx.x] = hz;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            for (int k = 0; k < 3; ++k) sm[k][threadIdx.x] = fminf(sm[k][threadIdx.x], sm[k][threadIdx.x + s]);
            for (int k = 3; k < 6; ++k) sm[k][threadIdx.x] = fmaxf(sm[k][threadIdx.x], sm[k][threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = make_float4(sm[0][0], sm[1][0], sm[2][0], 0.f);
        out[1] = make_float4(sm[3][0], sm[4][0], sm[5][0], 0.f);
    }
}

__device__ __forceinline__ uint32_t quantise(float c, float lo, float hi)
{
    const float ext = __fsub_rn(hi, lo);
    if (!(ext > 0.f)) return 0u;
    const float t = __fmul_rn(__fdiv_rn(__fsub_rn(c, lo), ext), 1024.0f);
    const int q = (int)floorf(t);
    return (uint32_t)min(max(q, 0), 1023);
}

__global__ void mortonCodes(const float4 *cen, const float4 *bounds, uint32_t n, uint32_t *codes, uint32_t *ids)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 c = cen[i], lo = bounds[0], hi = bounds[1];
    const uint32_t x = quantise(c.x, lo.x, hi.x), y = quantise(c.y, lo.y, hi.y), z = quantise(c.z, lo.z, hi.z);
    codes[i] = (expandBits10(x) << 2) | (expandBits10(y) << 1) | expandBits10(z);
    ids[i] = i;
}

// Per-block digit histogram, digit-major: counts[digit * numBlocks + block].
__global__ void radixHistogram(const uint32_t *keys, uint32_t n, int shift, uint32_t *counts)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * kSortBlock + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    __syncthreads();
    counts[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of `m` counts by one block of 1024 threads (chunked).
__global__ void exclusiveScan(uint32_t *data, uint32_t m)
{
    __shared__ uint32_t sh[1024];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < m; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = (i < m) ? data[i] : 0u;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const uint32_t t = (threadIdx.x >= (uint32_t)off) ? sh[threadIdx.x - off] : 0u;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < m) data[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
}

// Stable scatter: rank = scanned block offset + earlier warps' count of the digit
// in this tile + same-digit lanes below this lane.
__global__ void radixScatter(const uint32_t *keysIn, const uint32_t *valsIn, uint32_t n, int shift,
                             const uint32_t *offsets, uint32_t *keysOut, uint32_t *valsOut)
{
    __shared__ uint32_t warpHist[kSortBlock / 32][256];
    for (int k = threadIdx.x; k < (kSortBlock / 32) * 256; k += blockDim.x) (&warpHist[0][0])[k] = 0;
    __syncthreads();
    const uint32_t i = blockIdx.x * kSortBlock + threadIdx.x;
    const bool valid = i < n;
    const uint32_t key = valid ? keysIn[i] : 0u;
    const uint32_t d = valid ? (key >> shift) & 255u : 256u + (threadIdx.x & 31);   // invalid lanes never match
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t below = __popc(peers & ((1u << lane) - 1u));
    if (valid && below == 0) warpHist[warp][d] = __popc(peers);
    __syncthreads();
    if (threadIdx.x < 256) {
        uint32_t run = 0;
        for (int w = 0; w < kSortBlock / 32; ++w) {
            const uint32_t t = warpHist[w][threadIdx.x];
            warpHist[w][threadIdx.x] = run;
            run += t;
        }
    }
    __syncthreads();
    if (valid) {
        const uint32_t pos = offsets[d * gridDim.x + blockIdx.x] + warpHist[warp][d] + below;
        keysOut[pos] = key;
        valsOut[pos] = valsIn[i];
    }
}

__device__ __forceinline__ int delta(const uint32_t *codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// Karras 2012, Fig. 4: internal node i covers a contiguous range of sorted leaves.
__global__ void karras(const uint32_t *codes, const uint32_t *sortedIds, int n, int *leftChild, int *rightChild,
                       int *parentOfNode, int *parentOfLeaf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(codes, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    const int gamma = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    // children: leaves are encoded as ~primitive id, inner nodes by index
    int lc, rc;
    if (first == gamma) { lc = ~(int)sortedIds[gamma]; parentOfLeaf[gamma] = i; }
    else { lc = gamma; parentOfNode[gamma] = i; }
    if (last == gamma + 1) { rc = ~(int)sortedIds[gamma + 1]; parentOfLeaf[gamma + 1] = i; }
    else { rc = gamma + 1; parentOfNode[gamma + 1] = i; }
    leftChild[i] = lc;
    rightChild[i] = rc;
    if (i == 0) parentOfNode[0] = -1;
}

__global__ void refit(const float4 *primLo, const float4 *primHi, const uint32_t *sortedIds, int n,
                      const int *leftChild, const int *rightChild, const int *parentOfNode, const int *parentOfLeaf,
                      BvhNode *nodes, float4 *nodeLo, float4 *nodeHi, unsigned int *arrivals)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int parent = parentOfLeaf[k];
    // the path to the root has fewer than n inner nodes; the bound guards a malformed tree
    for (int depth = 0; parent >= 0 && parent < n - 1 && depth < n; ++depth) {
        __threadfence();
        const unsigned old = atomicAdd(&arrivals[parent], 1u);
        if (old == 0) return;   // the sibling finishes this parent
        __threadfence();
        const int lc = leftChild[parent], rc = rightChild[parent];
        float4 llo, lhi, rlo, rhi;
        if (lc < 0) { llo = primLo[~lc]; lhi = primHi[~lc]; }
        else { llo = __ldcg(&nodeLo[lc]); lhi = __ldcg(&nodeHi[lc]); }
        if (rc < 0) { rlo = primLo[~rc]; rhi = primHi[~rc]; }
        else { rlo = __ldcg(&nodeLo[rc]); rhi = __ldcg(&nodeHi[rc]); }
        BvhNode nd;
        nd.lo_l = make_float4(llo.x, llo.y, llo.z, __int_as_float(lc));
        nd.hi_l = make_float4(lhi.x, lhi.y, lhi.z, 0.f);
        nd.lo_r = make_float4(rlo.x, rlo.y, rlo.z, __int_as_float(rc));
        nd.hi_r = make_float4(rhi.x, rhi.y, rhi.z, 0.f);
        nodes[parent] = nd;
        __stcg(&nodeLo[parent], make_float4(fminf(llo.x, rlo.x), fminf(llo.y, rlo.y), fminf(llo.z, rlo.z), 0.f));
        __stcg(&nodeHi[parent], make_float4(fmaxf(lhi.x, rhi.x), fmaxf(lhi.y, rhi.y), fmaxf(lhi.z, rhi.z), 0.f));
        parent = parentOfNode[parent];
    }
}

}  // namespace

// Each array of the scratch carve starts on a 256-byte boundary (see buildLbvh).
static size_t carveSize(size_t bytes) { return (bytes + 255) & ~size_t(255); }

size_t lbvhScratchBytes(uint32_t n)
{
    const size_t nb = (n + kSortBlock - 1) / kSortBlock;
    return 3 * carveSize(16 * (size_t)n)    // lo, hi, centroid
           + carveSize(32)                  // bounds
           + 4 * carveSize(4 * (size_t)n)   // keys/vals x2
           + carveSize(4 * 256 * nb)        // counts
           + 4 * carveSize(4 * (size_t)n)   // left, right, parentOfNode, parentOfLeaf
           + 2 * carveSize(16 * (size_t)n)  // node lo/hi
           + carveSize(4 * (size_t)n);      // arrivals
}

// Builds the node array for n >= 2 primitives. `scratch` holds lbvhScratchBytes(n) bytes;
// `sortedCodes`/`sortedIds` (n entries each, may be null) receive the sorted keys for checks.
cudaError_t buildLbvh(const SceneView &S, BvhNode *nodes, void *scratch, uint32_t *sortedCodesOut,
                      uint32_t *sortedIdsOut, cudaStream_t stream)
{
    const uint32_t n = S.ntri + S.nsph;
    if (n < 2) return cudaSuccess;
    const uint32_t nb = (n + kSortBlock - 1) / kSortBlock;
    char *p = reinterpret_cast<char *>(scratch);
    auto take = [&](size_t bytes) {
        char *r = p;
        p += (bytes + 255) & ~size_t(255);
        return r;
    };
    float4 *lo = (float4 *)take(16 * (size_t)n), *hi = (float4 *)take(16 * (size_t)n);
    float4 *cen = (float4 *)take(16 * (size_t)n), *bounds = (float4 *)take(32);
    uint32_t *k0 = (uint32_t *)take(4 * (size_t)n), *v0 = (uint32_t *)take(4 * (size_t)n);
    uint32_t *k1 = (uint32_t *)take(4 * (size_t)n), *v1 = (uint32_t *)take(4 * (size_t)n);
    uint32_t *counts = (uint32_t *)take(4 * 256 * (size_t)nb);
    int *lc = (int *)take(4 * (size_t)n), *rc = (int *)take(4 * (size_t)n);
    int *pn = (int *)take(4 * (size_t)n), *pl = (int *)take(4 * (size_t)n);
    float4 *nlo = (float4 *)take(16 * (size_t)n), *nhi = (float4 *)take(16 * (size_t)n);
    unsigned int *arr = (unsigned int *)take(4 * (size_t)n);

    const int tb = 256, gb = (int)((n + tb - 1) / tb);
    primBounds<<<gb, tb, 0, stream>>>(S, lo, hi, cen);
    centroidBounds<<<1, 256, 0, stream>>>(cen, n, bounds);
    mortonCodes<<<gb, tb, 0, stream>>>(cen, bounds, n, k0, v0);
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = pass * 8;
        radixHistogram<<<nb, kSortBlock, 0, stream>>>(k0, n, shift, counts);
        exclusiveScan<<<1, 1024, 0, stream>>>(counts, 256u * nb);
        radixScatter<<<nb, kSortBlock, 0, stream>>>(k0, v0, n, shift, counts, k1, v1);
        uint32_t *t = k0; k0 = k1; k1 = t;
        t = v0; v0 = v1; v1 = t;
    }
    cudaMemsetAsync(arr, 0, 4 * (size_t)n, stream);
    karras<<<(n - 1 + tb - 1) / tb, tb, 0, stream>>>(k0, v0, (int)n, lc, rc, pn, pl);
    refit<<<gb, tb, 0, stream>>>(lo, hi, v0, (int)n, lc, rc, pn, pl, nodes, nlo, nhi, arr);
    if (sortedCodesOut) cudaMemcpyAsync(sortedCodesOut, k0, 4 * (size_t)n, cudaMemcpyDeviceToDevice, stream);
    if (sortedIdsOut) cudaMemcpyAsync(sortedIdsOut, v0, 4 * (size_t)n, cudaMemcpyDeviceToDevice, stream);
    return cudaGetLastError();
}

}  // namespace pg3
