// Device-side scene layout shared by the host setup code and the kernels.
//
// Everything a kernel reads lives in HBM in structure-of-arrays form and is
// passed to kernels by value in one SceneView (kernel-parameter space), so a
// launch needs no extra indirection. Geometry is stored the way the closest-
// hit loop consumes it: three float4 per triangle (vertex xyz + one normal
// component in w), one float4 per sphere (centre, radius).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pg3 {

enum : int {
    kMatLambert = 0, kMatGgxConductor = 1, kMatGgxDielectric = 2,
    kMatPhong = 3, kMatSmoothConductor = 4, kMatSmoothDielectric = 5, kMatSra = 6, kNumMatKinds = 7
};
enum : int { kBgNone = 0, kBgConstant = 1, kBgEnvMap = 2 };
// kEmSteerableAdaptive: the steerable sampler over an adaptive triangulation (an internal sampler
// id; the options name it PG3GPU_EM_STEERABLE with a maximum subdivision level above the minimum)
enum : int { kEmCdf = 0, kEmCosine = 1, kEmSteerable = 2, kEmSteerableAdaptive = 3 };

struct DevMaterial {          // 80 bytes
    int kind;
    float r, g, b;            // Lambert reflectance; Phong diffuse reflectance; SRA inner Lambert reflectance
    float alpha;              // GGX roughness (already clamped); SRA outer roughness
    float eta, etaInv;        // inner/outer, outer/inner (SRA: of the outer layer)
    float absorb;             // conductor k (SRA: of the inner conductor)
    float rrProb;             // Russian-roulette continuation probability (clamped to 0.997); Phong: the
                              // diffuse part of its view-dependent estimate
    int zeroRefl;             // zero reflectance (IsReflectanceZero): paths end here (lights)
    int vndfExact;            // GGX: exact visible-normal sampling (1) or the reference's fitted routine (0)
    float alphaS;             // GGX roughness the sampling routines and pdfs use (normally == alpha)
    float gr, gg, gb;         // Phong glossy reflectance; SRA medium attenuation coefficients
    float exponent;           // Phong lobe exponent; SRA medium thickness
    int innerKind;            // SRA: kMatLambert or kMatGgxConductor
    float innerAlpha, innerEta;   // SRA inner conductor: roughness (clamped), n / n_outer
    float pad;
};
static_assert(sizeof(DevMaterial) == 80, "DevMaterial is one 80-byte record");

// One entry of the light table: area lights first, then point lights (the background light is
// the id after the table).
struct DevAreaLight {         // 64 bytes; radiance rides in the w lanes
    float4 p0_invArea;        // p0.xyz, 1/area; a point light: position xyz, -1
    float4 e1_r;              // edge p1 - p0, radiance r (point light: intensity r)
    float4 e2_g;              // edge p2 - p0, radiance g (intensity g)
    float4 n_b;               // frame normal xyz, radiance b (intensity b)
};

// Linear BVH node (Karras 2012 layout, children as signed ids: >= 0 inner node,
// < 0 leaf ~primitive slot); boxes of both children stored in the parent so a
// traversal step is one 64-byte read.
struct BvhNode {
    float4 lo_l;              // left child box min xyz, left child id (as int bits)
    float4 hi_l;              // left child box max xyz, unused
    float4 lo_r;              // right child box min xyz, right child id (as int bits)
    float4 hi_r;              // right child box max xyz, unused
};

// A node of the 4-wide BVH collapsed from the binary LBVH (every node takes its binary node's
// grandchildren): the boxes of its up to 4 children coordinate-major, one float4 per bound, so
// the four slab tests read 6 vector loads; child ids >= 0 are nodes, < 0 ~primitive, INT_MIN none.
struct BvhNode4 {
    float4 lox, hix, loy, hiy, loz, hiz;
    int4 child;
    float4 pad;
};

// Steerable sampler tables (host build in pg3_steerable.cpp, sampling in pg3_steer.cuh).
constexpr int kSteerNodeVec4 = 14;   // float4 per 6-ary tree node: 6 children x 9 weights, padded

struct SteerView {
    const float4 *vdir;       // per vertex: unit direction xyz (w: the antipodal vertex, uniform levels)
    const int4 *tri;          // vertex ids of the triangles of every subdivision level (adaptive: level 0)
    const float *nodeW;       // per 6-ary tree node: 9 coefficients x 6 children of summed weights,
                              // coefficient-major (54 floats), then the first child and the child
                              // count (int bits): kSteerNodeVec4 float4
    const int *nodeChild;     // per node: 8 child slots (>= 0 node, < 0 ~leaf, INT_MIN none)
    const float4 *leafPlane;  // per leaf: unit plane normal, distance from the origin; followed in the
                              // same allocation by the leaf-locator tables and the whole-sphere
                              // weights (pg3_steer.cuh)
    const int4 *faceCells;    // cube-map cells: up to 4 candidate level-0 faces (-1 none)
    const float4 *leafRec;    // per leaf 5 float4: corners A, B, C with the map's luminance there in w;
                              // the luminance at -A, -B, -C (uniform levels); the leaf's plane
                              // (unit normal, distance from the origin)
    const int4 *qtree;        // adaptive: face codes and the subdivided triangles (pg3_steerable.h)
    const int *startCells;    // adaptive: per cube-map cell the quadtree code where point location
                              // starts (INT_MIN: at the level-0 face); null for uniform levels
    uint32_t numLeaves, leafGrid;
    uint32_t level;           // leaf subdivision level (adaptive: the deepest leaf's); uniform levels keep
                              // the triangles of every level in `tri`, level l from 20 (4^l - 1) / 3 on
    int root;
};

struct SceneView {
    // camera (pinhole equivalent of the reference's raster-to-world matrix)
    float3 camPos, camFwd, camRight, camUp;
    float tanX, tanY;
    uint32_t width, height;

    // geometry
    const float4 *tri;        // 3 per triangle
    const int *triMat;
    const float4 *sph;
    const int *sphMat;
    uint32_t ntri, nsph;

    // acceleration structure (null when the list loop is used)
    const BvhNode *bvh;       // useBvh 1: the binary LBVH; 2: BvhNode4 records (the 4-wide BVH)
    uint32_t bvhRoot;         // root node id (valid when nprims > 1)
    int useBvh;               // 0: the primitive list, 1: the binary LBVH, 2: the 4-wide BVH

    // materials and lights
    const DevMaterial *mats;
    const int *mat2light;     // material id -> light id or -1
    uint32_t nmat;
    const DevAreaLight *lights;
    uint32_t nArea;           // entries of the light table (area and point lights)
    uint32_t lightCount;      // light table + background
    int bgKind;
    int bgLightId;
    float3 bgConst;

    // environment map (lat-long, float4 texels) and its samplers
    const float4 *em;
    uint32_t emW, emH;
    const float *emMarg;      // marginal CDF over rows (emH + 1)
    const float *emCond;      // conditional CDFs, emH rows of (emW + 1)
    const float *bgShL;       // 9 SH coefficients of the map's luminance: the background's
                              // light-picking estimate (with area lights present)
    int emSampler;
    SteerView steer;

    // options
    int algorithm;
    uint32_t minPL, maxPL, rrMinPL;
    uint32_t seedLo, seedHi;
    float splitBudget, splitLevel, lightRatio, clipping;   // splitting and indirect clipping
    int treeMode;             // 1: the recursive estimator (splitting / clipping) runs algorithm 7

    // device error word (bounded loops set bits instead of trapping)
    unsigned int *errorFlag;
};

// Per-launch counters (PathTerminationReason histogram + ray totals).
constexpr int kLenBins = 16;   // path-length histogram bins: bin b holds lengths 2^b - 1 .. 2^(b+1) - 2
struct DevStats {
    unsigned long long paths;
    unsigned long long extRays;
    unsigned long long shadowRays;
    unsigned long long byRR;
    unsigned long long byBackground;
    unsigned long long byBlocker;
    unsigned long long byMax;
    unsigned long long bySafety;
    unsigned long long lenHist[kLenBins];   // lengths of the paths ended by all but the safety limit
    unsigned int minLenC, maxLen;           // ~(shortest length) (0: none yet) and the longest length
};

// Adjoint inputs and outputs of one path-replay launch (pg3_wave.cuh).
struct GradArgs {
    const float *dLdI;        // dLoss / d(mean image), rgb per pixel
    float invSpp;             // the mean image is the sum of the samples / spp
    const float *totR, *totG, *totB;   // primal radiance of each path (indexed like the output buffers)
    float *gMat;              // per material: d/d albedo rgb, d/d roughness
    float *gEm;               // per environment-map texel: rgb
    int adjoint;              // 0: primal replay (radiance only), 1: adjoint
    const uint32_t *sampleOffset;   // device word added to every sample index (null: none)
};

enum : unsigned int { kErrTraversalStack = 1u, kErrQueueOverflow = 2u, kErrSteerDescent = 4u, kErrTreeStack = 16u };

// One vertex of the recursive estimator's depth-first walk (traceTree, pg3_estimator.cuh).
struct TreeFrame {
    float3 pt;
    float budget;             // splitting budget of this vertex's children
    float3 n;
    float rr;                 // roulette continuation probability
    float3 wol;
    float sum;                // light-estimate sum for picking
    float3 R;                 // reflected estimate so far
    uint32_t vid;             // preorder index
    float3 att;               // current BSDF sample: attenuation
    float cosAbs;
    float pdfW, compProb;
    int mat;
    uint32_t pl;
    uint32_t i, nBsdf, nLight, flags;   // flags: 1 finite sample, 2 roulette cut the sample
};


}  // namespace pg3
