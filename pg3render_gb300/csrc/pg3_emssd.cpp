// Steerable-sampler data files: the reference's ".emssd" format, version 2.1
// (EnvironmentMapSteerableSampler::SaveToDisk / LoadFromDisk, src/em_steerable_sampler.hxx:1648-2058).
//
// Layout (little-endian, as the reference writes its variables' bytes, utils.hxx:295-345):
//   the header text "Environment Map Steerable Sampler Data, format ver. 2.1\n" with its zero byte;
//   build parameters: float max approximation error, uint32 min and max subdivision level,
//     uint32 max triangle samples per dimension, float max triangle span, float oversampling
//     factor, uint32 maximum children of a triangle-set node (6);
//   vertices: uint32 count, then per vertex its direction (3 floats) and its weight, the 9 SH
//     basis values scaled by the map's luminance in that direction (9 floats);
//   the tree: uint32 counts of set nodes and triangle nodes, then the nodes depth first, each
//     opening with a uint32 flag (1 triangle node): a set node has a uint32 child count and its
//     children; a triangle node its uint32 subdivision level and 3 uint32 vertex indices.
//
// Writing stores the context's triangulation (uniform or adaptive: each leaf with its level, the
// vertices shared, its 6-ary tree) with its build parameters. Reading accepts any file whose leaves
// are triangles of the icosahedron's 4-way subdivision covering the sphere, in any vertex numbering
// or tree order (the reference stores a vertex once per triangle that creates it): a file with
// exactly the context's uniform level replaces only the vertex weights; any other file (an
// adaptive triangulation, the reference's default build, or another level) replaces the context's
// triangulation with the file's. Either way the leaf, node and whole-sphere weights are rebuilt on
// the device; a later change of the map (pg3gpu_set_params) recomputes the weights from it.
#include <algorithm>
#include <array>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "pg3_ctx.h"
#include "pg3_host.h"
#include "pg3_steerable.h"

namespace pg3 {

namespace {

constexpr char kHeader[] = "Environment Map Steerable Sampler Data, format ver. 2.1\n";
constexpr uint32_t kSetChildren = 6;          // MAX_TRIANGLE_SET_CHILDREN
constexpr uint32_t kMaxFileVertices = 1u << 24;
constexpr uint32_t kMaxFileNodes = 1u << 24;

struct Writer {
    std::vector<unsigned char> b;
    void bytes(const void *p, size_t n)
    {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        b.insert(b.end(), c, c + n);
    }
    void u32(uint32_t v)
    {
        for (int i = 0; i < 4; ++i) b.push_back((unsigned char)((v >> (8 * i)) & 0xffu));
    }
    void f32(float v)
    {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        u32(u);
    }
};

struct Reader {
    const std::vector<unsigned char> &b;
    size_t o = 0;
    bool ok = true;
    explicit Reader(const std::vector<unsigned char> &buf) : b(buf) {}
    uint32_t u32()
    {
        if (o + 4 > b.size()) { ok = false; return 0; }
        uint32_t v = 0;
        for (int i = 0; i < 4; ++i) v |= (uint32_t)b[o + i] << (8 * i);
        o += 4;
        return v;
    }
    float f32()
    {
        const uint32_t u = u32();
        float v;
        std::memcpy(&v, &u, 4);
        return v;
    }
};

int ctxFail(pg3gpu_ctx *ctx, int status, const std::string &msg) { return ctxError(ctx, status, msg); }

const SteerGeom *contextGeometry(pg3gpu_ctx *ctx, std::string &err)
{
    if (!ctx->hasSteer || !ctx->steerGeom) {
        err = "the context has no steerable sampler (environment map with em_sampler PG3GPU_EM_STEERABLE)";
        return nullptr;
    }
    return ctx->steerGeom.get();
}

// Depth-first writer of the 6-ary tree (nodeChild: >= 0 node, < 0 ~leaf, INT_MIN none).
void writeNode(Writer &w, const SteerGeom &g, int item, bool isLeaf)
{
    if (isLeaf) {
        const int4 t = g.leafTri[(uint32_t)item];
        w.u32(1u);
        w.u32((uint32_t)t.w);   // the leaf's subdivision level
        w.u32((uint32_t)t.x);
        w.u32((uint32_t)t.y);
        w.u32((uint32_t)t.z);
        return;
    }
    uint32_t n = 0;
    while (n < kSetChildren && g.nodeChild[8 * (size_t)item + n] != INT_MIN) ++n;
    w.u32(0u);
    w.u32(n);
    for (uint32_t c = 0; c < n; ++c) {
        const int ch = g.nodeChild[8 * (size_t)item + c];
        if (ch >= 0) writeNode(w, g, ch, false);
        else writeNode(w, g, ~ch, true);
    }
}

struct FileLeaf {
    uint32_t level, v[3];
};

// Depth-first reader; counts nodes, collects leaves. Depth is bounded by the node count.
bool readNode(Reader &r, uint32_t nv, std::vector<FileLeaf> &leaves, uint32_t &sets, uint32_t depth)
{
    if (depth > 64 || leaves.size() + sets > kMaxFileNodes) return false;
    const uint32_t isTri = r.u32();
    if (!r.ok || isTri > 1u) return false;
    if (isTri) {
        FileLeaf l;
        l.level = r.u32();
        for (int k = 0; k < 3; ++k) l.v[k] = r.u32();
        if (!r.ok || l.v[0] >= nv || l.v[1] >= nv || l.v[2] >= nv) return false;
        leaves.push_back(l);
        return true;
    }
    ++sets;
    const uint32_t n = r.u32();
    if (!r.ok || n == 0 || n > kSetChildren) return false;
    for (uint32_t c = 0; c < n; ++c)
        if (!readNode(r, nv, leaves, sets, depth + 1)) return false;
    return true;
}

// Our vertex of each file direction (-1: none within tolerance): a hash grid over the directions.
std::vector<int> matchVertices(const SteerGeom &g, const std::vector<float> &fileDirs)
{
    const double q = 1e-3;
    auto key = [](long long i, long long j, long long k) { return (i * 73856093LL) ^ (j * 19349663LL) ^ (k * 83492791LL); };
    std::unordered_multimap<long long, int> grid;
    grid.reserve(g.vdir.size() * 2);
    for (size_t v = 0; v < g.vdir.size(); ++v) {
        const float4 d = g.vdir[v];
        grid.emplace(key((long long)std::floor(d.x / q), (long long)std::floor(d.y / q), (long long)std::floor(d.z / q)),
                     (int)v);
    }
    const size_t n = fileDirs.size() / 3;
    std::vector<int> out(n, -1);
    for (size_t i = 0; i < n; ++i) {
        const double x = fileDirs[3 * i], y = fileDirs[3 * i + 1], z = fileDirs[3 * i + 2];
        const long long ci = (long long)std::floor(x / q), cj = (long long)std::floor(y / q), ck = (long long)std::floor(z / q);
        double best = 1e-5;
        for (int di = -1; di <= 1; ++di)
            for (int dj = -1; dj <= 1; ++dj)
                for (int dk = -1; dk <= 1; ++dk) {
                    auto range = grid.equal_range(key(ci + di, cj + dj, ck + dk));
                    for (auto it = range.first; it != range.second; ++it) {
                        const float4 d = g.vdir[(size_t)it->second];
                        const double e = std::fabs(d.x - x) + std::fabs(d.y - y) + std::fabs(d.z - z);
                        if (e < best) { best = e; out[i] = it->second; }
                    }
                }
    }
    return out;
}

bool readFile(const char *path, std::vector<unsigned char> &b)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    unsigned char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    return !err;
}

}  // namespace

}  // namespace pg3

using namespace pg3;

int pg3gpu_save_steerable(pg3gpu_ctx *ctx, const char *path, float max_approx_error)
{
    if (!ctx || !path) return PG3GPU_ERR_INVALID_ARGUMENT;
    std::string err;
    const SteerGeom *gp = contextGeometry(ctx, err);
    if (!gp) return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "save_steerable: " + err);
    const SteerGeom &g = *gp;
    const SteerWeightArgs &a = ctx->steerArgs;
    cudaSetDevice(ctx->device);
    std::vector<float> vw(12 * (size_t)a.numVertices);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess ||
        cudaMemcpy(vw.data(), a.vw, vw.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
        return ctxFail(ctx, PG3GPU_ERR_CUDA, "save_steerable: reading the vertex weights failed");
    Writer w;
    w.bytes(kHeader, sizeof kHeader);   // with the terminating zero
    w.f32(g.adaptive ? g.maxApproxError : max_approx_error);
    w.u32(g.minLevel);                  // uniform: minimum = maximum subdivision level
    w.u32(g.maxLevel);
    w.u32(50u);                         // the reference's defaults of its debugging parameters
    w.f32(1.1f);                        // (BuildParameters, src/em_steerable_sampler.hxx:30-57)
    w.f32(0.7f);
    w.u32(kSetChildren);
    w.u32((uint32_t)g.vdir.size());
    for (size_t v = 0; v < g.vdir.size(); ++v) {
        w.f32(g.vdir[v].x);
        w.f32(g.vdir[v].y);
        w.f32(g.vdir[v].z);
        for (int k = 0; k < 9; ++k) w.f32(vw[12 * v + k]);
    }
    w.u32(g.numNodes());
    w.u32(g.numLeaves());
    writeNode(w, g, g.root, false);
    FILE *f = std::fopen(path, "wb");
    if (!f) return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, std::string("save_steerable: cannot open ") + path);
    const bool ok = std::fwrite(w.b.data(), 1, w.b.size(), f) == w.b.size();
    if (std::fclose(f) != 0 || !ok)
        return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, std::string("save_steerable: cannot write ") + path);
    return PG3GPU_OK;
}

int pg3gpu_load_steerable(pg3gpu_ctx *ctx, const char *path)
{
    if (!ctx || !path) return PG3GPU_ERR_INVALID_ARGUMENT;
    std::string err;
    const SteerGeom *gp = contextGeometry(ctx, err);
    if (!gp) return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, "load_steerable: " + err);
    const SteerGeom &g = *gp;
    std::vector<unsigned char> b;
    if (!readFile(path, b)) return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, std::string("load_steerable: cannot read ") + path);
    auto bad = [&](const std::string &why) {
        return ctxFail(ctx, PG3GPU_ERR_INVALID_ARGUMENT, std::string("load_steerable: ") + path + ": " + why);
    };
    if (b.size() < sizeof kHeader || std::memcmp(b.data(), kHeader, sizeof kHeader) != 0)
        return bad("not a steerable sampler data file of format 2.1");
    Reader r(b);
    r.o = sizeof kHeader;
    const float fileError = r.f32();
    const uint32_t minLevel = r.u32(), maxLevel = r.u32();
    r.u32();
    r.f32();
    r.f32();
    const uint32_t children = r.u32();
    if (!r.ok) return bad("truncated parameters");
    if (children != kSetChildren) return bad("tree nodes of " + std::to_string(children) + " children (6 expected)");
    const uint32_t nv = r.u32();
    if (!r.ok || nv == 0 || nv > kMaxFileVertices || r.o + (size_t)nv * 48 > b.size()) return bad("bad vertex count");
    std::vector<float> dirs(3 * (size_t)nv), weights(9 * (size_t)nv);
    for (uint32_t v = 0; v < nv; ++v) {
        for (int k = 0; k < 3; ++k) dirs[3 * (size_t)v + k] = r.f32();
        for (int k = 0; k < 9; ++k) weights[9 * (size_t)v + k] = r.f32();
    }
    const uint32_t nSets = r.u32(), nTris = r.u32();
    if (!r.ok) return bad("truncated tree counts");
    std::vector<FileLeaf> leaves;
    uint32_t sets = 0;
    if (!readNode(r, nv, leaves, sets, 0)) return bad("malformed tree");
    if (sets != nSets || leaves.size() != nTris) return bad("tree node counts disagree with the header");
    if (r.o != b.size()) return bad("trailing bytes after the tree");
    bool sameLevel = !g.adaptive && leaves.size() == g.numLeaves();
    for (const FileLeaf &l : leaves) sameLevel = sameLevel && l.level == g.level;
    std::shared_ptr<SteerGeom> fileGeom;   // the file's own triangulation, when it is not the context's
    if (sameLevel) {
        // file vertices -> ours; every leaf of the file must be one of ours, each exactly once
        const std::vector<int> map = matchVertices(g, dirs);
        std::map<std::array<int, 3>, uint32_t> ours;
        for (uint32_t t = 0; t < g.numLeaves(); ++t) {
            const int4 v = g.leafTri[t];
            std::array<int, 3> k = {v.x, v.y, v.z};
            std::sort(k.begin(), k.end());
            ours[k] = t;
        }
        std::vector<char> seen(g.numLeaves(), 0);
        for (const FileLeaf &l : leaves) {
            std::array<int, 3> k;
            for (int j = 0; j < 3; ++j) {
                k[j] = map[l.v[j]];
                if (k[j] < 0) return bad("a vertex direction is not one of the level's vertices");
            }
            std::sort(k.begin(), k.end());
            auto it = ours.find(k);
            if (it == ours.end() || seen[it->second]) return bad("a leaf triangle is not one of the level's triangles");
            seen[it->second] = 1;
        }
    } else {
        std::vector<std::array<float, 9>> corners(leaves.size());
        std::vector<uint32_t> levels(leaves.size());
        for (size_t i = 0; i < leaves.size(); ++i) {
            for (int j = 0; j < 3; ++j)
                for (int k = 0; k < 3; ++k) corners[i][3 * j + k] = dirs[3 * (size_t)leaves[i].v[j] + k];
            levels[i] = leaves[i].level;
        }
        std::string gerr;
        fileGeom = steerGeometryFromLeaves(corners, levels, minLevel, maxLevel, fileError, gerr);
        if (!fileGeom) return bad(gerr);
    }
    const SteerGeom &tg = fileGeom ? *fileGeom : g;   // the triangulation the weights belong to
    const std::vector<int> map = matchVertices(tg, dirs);
    // weights of our vertices from the file's (a vertex stored several times carries one value)
    std::vector<float> vw(12 * tg.vdir.size(), 0.f);
    std::vector<char> have(tg.vdir.size(), 0);
    for (uint32_t i = 0; i < nv; ++i) {
        const int v = map[i];
        if (v < 0) continue;
        for (int k = 0; k < 9; ++k) {
            const float x = weights[9 * (size_t)i + k];
            if (!std::isfinite(x)) return bad("non-finite vertex weight");
            if (have[(size_t)v] && std::fabs(vw[12 * (size_t)v + k] - x) > 1e-6f * (1.f + std::fabs(x)))
                return bad("copies of one vertex carry different weights");
            vw[12 * (size_t)v + k] = x;
        }
        have[(size_t)v] = 1;
    }
    for (size_t v = 0; v < have.size(); ++v)
        if (!have[v]) return bad("a vertex of the triangulation has no weight in the file");
    if (fileGeom) {
        cudaSetDevice(ctx->device);
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess)
            return ctxFail(ctx, PG3GPU_ERR_CUDA, "load_steerable: synchronising the context's stream failed");
        return uploadSteer(ctx, fileGeom, vw.data());
    }
    const SteerWeightArgs &a = ctx->steerArgs;
    cudaSetDevice(ctx->device);
    if (cudaMemcpyAsync(a.vw, vw.data(), vw.size() * sizeof(float), cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
        return ctxFail(ctx, PG3GPU_ERR_CUDA, "load_steerable: uploading the vertex weights failed");
    const cudaError_t e = launchSteerTreeWeights(a, ctx->stream);
    if (e == cudaSuccess && cudaStreamSynchronize(ctx->stream) == cudaSuccess) return PG3GPU_OK;
    return ctxFail(ctx, PG3GPU_ERR_CUDA, std::string("load_steerable: rebuilding the tree weights: ") + cudaGetErrorString(e));
}

int pg3gpu_steer_triangulate(const float *rgb, uint32_t width, uint32_t height, uint32_t min_level,
                             uint32_t max_level, float max_error, uint32_t *num_leaves, uint32_t *levels,
                             float *corners)
{
    if (!rgb || !num_leaves) return PG3GPU_ERR_INVALID_ARGUMENT;
    std::string err;
    const std::shared_ptr<SteerGeom> g = steerAdaptiveGeometry(rgb, width, height, min_level, max_level, max_error, err);
    if (!g) return ctxError(nullptr, PG3GPU_ERR_INVALID_ARGUMENT, "steer_triangulate: " + err);
    *num_leaves = g->numLeaves();
    for (uint32_t i = 0; i < g->numLeaves(); ++i) {
        const int4 t = g->leafTri[i];
        if (levels) levels[i] = (uint32_t)t.w;
        if (corners) {
            const int v[3] = {t.x, t.y, t.z};
            for (int j = 0; j < 3; ++j) {
                corners[9 * (size_t)i + 3 * j] = g->vdir[(size_t)v[j]].x;
                corners[9 * (size_t)i + 3 * j + 1] = g->vdir[(size_t)v[j]].y;
                corners[9 * (size_t)i + 3 * j + 2] = g->vdir[(size_t)v[j]].z;
            }
        }
    }
    return PG3GPU_OK;
}
