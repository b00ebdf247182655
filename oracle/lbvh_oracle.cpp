// CPU build of the linear BVH (test infrastructure only): the same steps as the
// device build in pg3render_gb300/csrc/pg3_lbvh.cu, in scalar C++ with the same
// rounded float operations (compiled with -ffp-contract=off), so that the tests
// can require the device tree to be bit-identical:
//   primitive boxes (triangles: vertex min/max; spheres: centre -/+ radius),
//   centroids (lo + hi) * 0.5, centroid bounds, 10-bit quantisation per axis,
//   30-bit Morton codes, stable sort by code, Karras (HPG 2012) hierarchy with
//   equal codes ordered by position, bottom-up box refit.
// The reference renderer has no acceleration structure (src/scene_graph.hxx:33-82).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

namespace {

uint32_t expandBits10(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

uint32_t quantise(float c, float lo, float hi)
{
    const float ext = hi - lo;
    if (!(ext > 0.f)) return 0u;
    const float t = ((c - lo) / ext) * 1024.0f;
    const int q = (int)std::floor(t);
    return (uint32_t)std::min(std::max(q, 0), 1023);
}

int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

int delta(const std::vector<uint32_t> &codes, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + clz32((uint32_t)i ^ (uint32_t)j);
    return clz32(a ^ b);
}

}  // namespace

extern "C" {

// tris: ntri x 9 floats; sph: nsph x 4 floats (centre, radius). Outputs for n = ntri + nsph >= 2:
// codes[n], ids[n] (sorted), nodes[(n-1) * 16] floats laid out like the device BvhNode
// (left lo xyz + id bits, left hi xyz + 0, right lo xyz + id bits, right hi xyz + 0).
int pg3o_lbvh(const float *tris, int ntri, const float *sph, int nsph, uint32_t *codesOut, uint32_t *idsOut,
              float *nodesOut)
{
    const int n = ntri + nsph;
    if (n < 2) return 1;
    std::vector<float> lo(3 * n), hi(3 * n), cen(3 * n);
    for (int i = 0; i < n; ++i) {
        float a[3], b[3];
        if (i < ntri) {
            const float *p = tris + 9 * i;
            for (int k = 0; k < 3; ++k) {
                a[k] = std::fmin(std::fmin(p[k], p[3 + k]), p[6 + k]);
                b[k] = std::fmax(std::fmax(p[k], p[3 + k]), p[6 + k]);
            }
        } else {
            const float *s = sph + 4 * (i - ntri);
            for (int k = 0; k < 3; ++k) { a[k] = s[k] - s[3]; b[k] = s[k] + s[3]; }
        }
        for (int k = 0; k < 3; ++k) {
            lo[3 * i + k] = a[k];
            hi[3 * i + k] = b[k];
            cen[3 * i + k] = (a[k] + b[k]) * 0.5f;
        }
    }
    float clo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, chi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            clo[k] = std::fmin(clo[k], cen[3 * i + k]);
            chi[k] = std::fmax(chi[k], cen[3 * i + k]);
        }
    std::vector<uint32_t> code(n);
    for (int i = 0; i < n; ++i) {
        const uint32_t x = quantise(cen[3 * i], clo[0], chi[0]);
        const uint32_t y = quantise(cen[3 * i + 1], clo[1], chi[1]);
        const uint32_t z = quantise(cen[3 * i + 2], clo[2], chi[2]);
        code[i] = (expandBits10(x) << 2) | (expandBits10(y) << 1) | expandBits10(z);
    }
    std::vector<uint32_t> ids(n);
    std::iota(ids.begin(), ids.end(), 0u);
    std::stable_sort(ids.begin(), ids.end(), [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });
    std::vector<uint32_t> sc(n);
    for (int i = 0; i < n; ++i) sc[i] = code[ids[i]];

    std::vector<int> lc(n - 1), rc(n - 1), parentNode(n - 1, -1), parentLeaf(n, -1);
    for (int i = 0; i < n - 1; ++i) {
        const int d = (delta(sc, n, i, i + 1) - delta(sc, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta(sc, n, i, i - d);
        int lmax = 2;
        while (delta(sc, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(sc, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = delta(sc, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (delta(sc, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int gamma = i + s * d + std::min(d, 0);
        const int first = std::min(i, j), last = std::max(i, j);
        if (first == gamma) { lc[i] = ~(int)ids[gamma]; parentLeaf[gamma] = i; }
        else { lc[i] = gamma; parentNode[gamma] = i; }
        if (last == gamma + 1) { rc[i] = ~(int)ids[gamma + 1]; parentLeaf[gamma + 1] = i; }
        else { rc[i] = gamma + 1; parentNode[gamma + 1] = i; }
    }
    // refit: post-order (children before parents) over the tree from the root 0
    std::vector<float> nlo(3 * (n - 1)), nhi(3 * (n - 1));
    std::vector<int> order;
    std::vector<int> stack = {0};
    while (!stack.empty()) {
        const int v = stack.back();
        stack.pop_back();
        order.push_back(v);
        if (lc[v] >= 0) stack.push_back(lc[v]);
        if (rc[v] >= 0) stack.push_back(rc[v]);
    }
    for (auto it = order.rbegin(); it != order.rend(); ++it) {
        const int v = *it;
        float bl[6], br[6];
        auto box = [&](int c, float *o) {
            const float *L = (c < 0) ? &lo[3 * (~c)] : &nlo[3 * c];
            const float *H = (c < 0) ? &hi[3 * (~c)] : &nhi[3 * c];
            for (int k = 0; k < 3; ++k) { o[k] = L[k]; o[3 + k] = H[k]; }
        };
        box(lc[v], bl);
        box(rc[v], br);
        float *out = nodesOut + 16 * (size_t)v;
        int li = lc[v], ri = rc[v];
        out[0] = bl[0]; out[1] = bl[1]; out[2] = bl[2]; std::memcpy(&out[3], &li, 4);
        out[4] = bl[3]; out[5] = bl[4]; out[6] = bl[5]; out[7] = 0.f;
        out[8] = br[0]; out[9] = br[1]; out[10] = br[2]; std::memcpy(&out[11], &ri, 4);
        out[12] = br[3]; out[13] = br[4]; out[14] = br[5]; out[15] = 0.f;
        for (int k = 0; k < 3; ++k) {
            nlo[3 * v + k] = std::fmin(bl[k], br[k]);
            nhi[3 * v + k] = std::fmax(bl[3 + k], br[3 + k]);
        }
    }
    for (int i = 0; i < n; ++i) { codesOut[i] = sc[i]; idsOut[i] = ids[i]; }
    return 0;
}

}  // extern "C"
