// CPU check of the steerable sampler's point-location tables (csrc/pg3_steerable.cpp).
//
// The device locates the leaf triangle that contains a direction (csrc/pg3_steer.cuh): uniform
// levels through a start cell that names the leaf when one leaf holds the whole cell, else the
// leaf-locator cell's candidate list tested by edge planes; adaptive triangulations through a
// start cell that names the deepest triangle holding the whole cell, then the quadtree of
// subdivided triangles (from the level-0 face where the cell spans faces). This program repeats
// those steps in float on the host tables, the way the device code does them, and checks for
// random directions and for directions within a few ulps of the start cells' borders that
//   * the start cells give the same leaf as the path without them,
//   * the candidate lists give the leaf that a brute-force test over all leaves gives.
// usage: steer_locator_check uniform <max level> <directions>
//        steer_locator_check adaptive <rgb float32 file> <W> <H> <min> <max> <error> <directions>
// Prints one line per case and exits 0 when nothing disagrees.
#include "pg3_steerable.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

using namespace pg3;

namespace {

struct V3 {
    float x, y, z;
};
V3 mk(float x, float y, float z) { return {x, y, z}; }
float dotf(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 crossf(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 vdir(const SteerGeom &g, int v) { return mk(g.vdir[v].x, g.vdir[v].y, g.vdir[v].z); }
V3 xyz(float4 e) { return mk(e.x, e.y, e.z); }

int cubeFace(V3 w, float &u, float &v)
{
    const float ax = std::fabs(w.x), ay = std::fabs(w.y), az = std::fabs(w.z);
    int a;
    float wa, wb, wc;
    if (ax >= ay && ax >= az) { a = 0; wa = w.x; wb = w.y; wc = w.z; }
    else if (ay >= az) { a = 1; wa = w.y; wb = w.z; wc = w.x; }
    else { a = 2; wa = w.z; wb = w.x; wc = w.y; }
    const float inv = 1.f / std::fabs(wa);
    u = wb * inv;
    v = wc * inv;
    return 2 * a + (wa < 0.f ? 1 : 0);
}

int cubeCell(int face, float u, float v, int G)
{
    const int iu = std::min(std::max((int)((u + 1.f) * (0.5f * G)), 0), G - 1);
    const int iv = std::min(std::max((int)((v + 1.f) * (0.5f * G)), 0), G - 1);
    return (face * G + iv) * G + iu;
}

float minEdge(const float4 *E, V3 w)
{
    return std::fmin(std::fmin(dotf(w, xyz(E[0])), dotf(w, xyz(E[1]))), dotf(w, xyz(E[2])));
}

float faceMinEdge(const SteerGeom &g, int f, V3 w)
{
    const int4 t = g.tri[f];
    const V3 a = vdir(g, t.x), b = vdir(g, t.y), c = vdir(g, t.z);
    return std::fmin(std::fmin(dotf(w, crossf(a, b)), dotf(w, crossf(b, c))), dotf(w, crossf(c, a)));
}

int locateFace(const SteerGeom &g, V3 w)
{
    float fu, fv;
    const int cell = cubeCell(cubeFace(w, fu, fv), fu, fv, kSteerCells);
    const int4 ca = g.faceCells[2 * cell], cb = g.faceCells[2 * cell + 1];
    const int cs[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
    int best = cs[0] >= 0 ? cs[0] : 0;
    float bestMin = -1e30f;
    for (int i = 0; i < 8 && cs[i] >= 0; ++i) {
        const float m = faceMinEdge(g, cs[i], w);
        if (m > bestMin) { bestMin = m; best = cs[i]; }
    }
    if (bestMin < -1e-6f)
        for (int f = 0; f < 20; ++f) {
            const float m = faceMinEdge(g, f, w);
            if (m > bestMin) { bestMin = m; best = f; }
        }
    return best;
}

int child(V3 w, V3 ab, V3 bc, V3 ca)
{
    if (dotf(w, crossf(ab, ca)) >= 0.f) return 0;
    if (dotf(w, crossf(bc, ab)) >= 0.f) return 1;
    if (dotf(w, crossf(ca, bc)) >= 0.f) return 2;
    return 3;
}

// uniform levels: the face, then one of four children per level
int locateUniformHierarchy(const SteerGeom &g, V3 w)
{
    int local = locateFace(g, w);
    for (uint32_t l = 0; l < g.level; ++l) {
        const int4 mid = g.tri[g.levelOffset[l + 1] + 4 * local + 3];
        local = 4 * local + child(w, vdir(g, mid.x), vdir(g, mid.y), vdir(g, mid.z));
    }
    return local;
}

int locateUniform(const SteerGeom &g, V3 w, bool useStart)
{
    float fu, fv;
    const int face = cubeFace(w, fu, fv);
    if (useStart && !g.startCells.empty()) {
        const int s = g.startCells[cubeCell(face, fu, fv, (int)kSteerUniformStartGrid)];
        if (s != INT_MIN) return ~s;
    }
    const uint4 cell = g.leafCells[cubeCell(face, fu, fv, (int)g.leafGrid)];
    if (cell.x != 0xfffefffeu) {
        const uint32_t words[4] = {cell.x, cell.y, cell.z, cell.w};
        int best = -1;
        float bestMin = -1e30f;
        for (int k = 0; k < 8; ++k) {
            const uint32_t id = (words[k >> 1] >> ((k & 1) * 16)) & 0xffffu;
            if (id == 0xffffu) break;
            const float m = minEdge(&g.leafEdge[3 * (size_t)id], w);
            if (m > bestMin) { bestMin = m; best = (int)id; }
            if (m >= 0.f) break;
        }
        if (best >= 0 && bestMin >= -1e-6f) return best;
    }
    return locateUniformHierarchy(g, w);
}

int locateAdaptive(const SteerGeom &g, V3 w, bool useStart)
{
    int code = INT_MIN;
    if (useStart) {
        float fu, fv;
        const int cf = cubeFace(w, fu, fv);
        code = g.startCells[cubeCell(cf, fu, fv, (int)kSteerStartGrid)];
    }
    if (code == INT_MIN) {
        const int f = locateFace(g, w);
        const int4 fc = g.qtree[f >> 2];
        code = (f & 3) == 0 ? fc.x : (f & 3) == 1 ? fc.y : (f & 3) == 2 ? fc.z : fc.w;
    }
    for (uint32_t depth = 0; depth <= kSteerMaxAdaptiveLevel && code >= 0; ++depth) {
        const int4 mid = g.qtree[5 + 2 * code], ch = g.qtree[5 + 2 * code + 1];
        const int c = child(w, vdir(g, mid.x), vdir(g, mid.y), vdir(g, mid.z));
        code = c == 0 ? ch.x : c == 1 ? ch.y : c == 2 ? ch.z : ch.w;
    }
    return code < 0 ? ~code : -1;
}

// the leaf whose three edge planes face w the most (and by how much)
int bruteForce(const SteerGeom &g, V3 w, float &margin)
{
    int best = -1;
    margin = -1e30f;
    for (uint32_t id = 0; id < g.numLeaves(); ++id) {
        const float m = minEdge(&g.leafEdge[3 * (size_t)id], w);
        if (m > margin) { margin = m; best = (int)id; }
    }
    return best;
}

// Random directions; every other one within a few ulps of a border of the start-cell grid G.
struct Directions {
    std::mt19937_64 rng{12345};
    std::normal_distribution<float> nd;
    V3 operator()(long i, int G)
    {
        V3 w = mk(nd(rng), nd(rng), nd(rng));
        if (i % 2) {
            float u, v;
            const int face = cubeFace(w, u, v);
            const float b = std::round((u + 1.f) * 0.5f * (float)G) / (0.5f * (float)G) - 1.f +
                            (float)((i >> 1) % 7 - 3) * 1e-7f;
            float p[3];
            p[face / 2] = (face & 1) ? -1.f : 1.f;
            p[(face / 2 + 1) % 3] = b;
            p[(face / 2 + 2) % 3] = v;
            w = mk(p[0], p[1], p[2]);
        }
        const float l = std::sqrt(dotf(w, w));
        return mk(w.x / l, w.y / l, w.z / l);
    }
};

int check(const SteerGeom &g, const char *name, long n, bool adaptive)
{
    Directions dirs;
    const int G = (int)(adaptive ? kSteerStartGrid : kSteerUniformStartGrid);
    long startBad = 0, listBad = 0, brute = 0;
    for (long i = 0; i < n; ++i) {
        const V3 w = dirs(i, G > 0 ? G : 1);
        const int a = adaptive ? locateAdaptive(g, w, true) : locateUniform(g, w, true);
        const int b = adaptive ? locateAdaptive(g, w, false) : locateUniform(g, w, false);
        startBad += a != b;
        if (i % 64 == 0) {
            float margin;
            const int c = bruteForce(g, w, margin);
            ++brute;
            listBad += (margin > 1e-6f && c != b);
        }
    }
    std::printf("%s: leaves %u, start cells %zu; %ld directions: %ld start-cell disagreements; %ld brute-force "
                "checks: %ld disagreements\n",
                name, g.numLeaves(), g.startCells.size(), n, startBad, brute, listBad);
    return (startBad || listBad) ? 1 : 0;
}

}  // namespace

int main(int argc, char **argv)
{
    const std::string mode = argc > 1 ? argv[1] : "";
    std::string err;
    if (mode == "uniform" && argc == 4) {
        const uint32_t maxLevel = (uint32_t)std::stoul(argv[2]);
        const long n = std::stol(argv[3]);
        int bad = 0;
        for (uint32_t level = 0; level <= maxLevel; ++level) {
            const SteerGeom *g = steerGeometry(level, err);
            if (!g) { std::printf("level %u: %s\n", level, err.c_str()); return 2; }
            const std::string name = "uniform level " + std::to_string(level);
            bad |= check(*g, name.c_str(), n, false);
        }
        return bad;
    }
    if (mode == "adaptive" && argc == 9) {
        const uint32_t W = (uint32_t)std::stoul(argv[3]), H = (uint32_t)std::stoul(argv[4]);
        std::vector<float> rgb((size_t)W * H * 3);
        FILE *f = std::fopen(argv[2], "rb");
        if (!f || std::fread(rgb.data(), 4, rgb.size(), f) != rgb.size()) { std::printf("cannot read the map\n"); return 2; }
        std::fclose(f);
        auto g = steerAdaptiveGeometry(rgb.data(), W, H, (uint32_t)std::stoul(argv[5]), (uint32_t)std::stoul(argv[6]),
                                       std::stof(argv[7]), err);
        if (!g) { std::printf("adaptive build: %s\n", err.c_str()); return 2; }
        return check(*g, "adaptive", std::stol(argv[8]), true);
    }
    std::printf("usage: steer_locator_check uniform <max level> <directions> | adaptive <rgb> <W> <H> <min> <max> "
                "<error> <directions>\n");
    return 2;
}
