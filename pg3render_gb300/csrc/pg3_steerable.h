// Steerable environment-map sampler (Subr & Arvo 2007, as structured by the
// reference's EnvironmentMapSteerableSampler, src/em_steerable_sampler.hxx).
//
// Triangulation: the unit icosahedron (src/geom.hxx:291-346) subdivided 4-way
// `level` times with edge midpoints pushed to the sphere -- the reference's
// refinement with minimum = maximum subdivision level (level 3: 1280 triangles).
// Each vertex carries its 9 SH basis values scaled by the environment map's
// luminance in its direction (src/em_steerable_sampler.hxx:181-202, 3084-3095);
// each leaf triangle the planar area times its mean vertex weight (:1277-1296).
// A 6-ary tree is built bottom-up over the leaves in subdivision order
// (:3755-3793).
//
// The build is split by what it depends on:
// * the geometry (triangulation, tree topology, leaf planes and edge normals, the
//   cube-map leaf and face locators) depends only on the level: it is built once per
//   process and level on the host (steerGeometry) and shared by every context;
// * the weights (vertex, leaf and tree-node weights and the whole-sphere integral)
//   depend on the map: they are computed on the device from the uploaded texels
//   (launchSteerWeights), at context creation and again whenever the map changes.
//
// Corrections over the reference (whose sampled and evaluated pdfs disagree):
// * the density is the linear interpolation of the vertex values on the planar
//   triangle, and the reported solid-angle pdf includes the planar-to-sphere
//   Jacobian r^2 / cos;
// * the in-triangle sampler is exact (a mixture of the three corner-weighted
//   densities, each sampled by inverting its cubic marginal);
// * pdf evaluation locates a direction's leaf through the subdivision hierarchy
//   (20 faces, then one of 4 children per level) instead of reading the
//   environment map, so evaluated pdf == sampled pdf.
//
// Adaptive triangulations (the reference's default build: subdivision between a minimum and a
// maximum level wherever the linear approximation of the map's luminance misses the map by more
// than a relative error, src/em_steerable_sampler.hxx:2963-3472) have leaves at several levels.
// Their geometry depends on the map, so it is built per context (steerAdaptiveGeometry) or read
// from a file of the reference (steerGeometryFromLeaves); a quadtree per icosahedron face locates
// a direction's leaf, and the triangulation is no longer centrally symmetric.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace pg3 {

struct SteerGeom {
    uint32_t level = 0;                // uniform: the leaves' level; adaptive: the maximum leaf level
    bool adaptive = false;
    uint32_t minLevel = 0, maxLevel = 0;   // build parameters (uniform: both = level)
    float maxApproxError = 5.f;
    std::vector<int4> leafTri;         // vertex ids of every leaf (w: the leaf's subdivision level)
    std::vector<int4> qtree;           // adaptive: the 20 face codes (5 int4), then per subdivided
                                       // triangle two int4: its edge midpoints (ab, bc, ca) and its
                                       // 4 child codes (children (A,ab,ca), (ab,B,bc), (ca,bc,C),
                                       // (ab,bc,ca)); a code >= 0 is a subdivided triangle, < 0 ~leaf
    std::vector<float4> vdir;          // vertex directions; w: the id of the antipodal vertex (int bits;
                                       // the subdivided icosahedron is centrally symmetric)
    std::vector<int4> tri;             // vertex ids of every triangle of every level (level 0 first)
    std::vector<uint32_t> levelOffset; // first triangle of each level in `tri` (level+1 entries + end)
    std::vector<float> leafArea;       // planar area of every leaf triangle
    std::vector<int> nodeChild;        // 8 child slots per node (6 used, two int4 loads): >= 0 node,
                                       // < 0 ~leaf, INT32_MIN none
    std::vector<uint32_t> layerStart;  // first node of every tree layer, bottom (parents of leaves)
                                       // first, then the end of the node list
    std::vector<float4> leafPlane;     // per leaf: unit normal of the planar triangle, distance from origin
    std::vector<int4> faceCells;       // cube-map cells (6 x kSteerCells^2) x 2: up to 8 candidate level-0 faces
    std::vector<float4> leafEdge;      // per leaf 3 inward great-circle normals (edges ab, bc, ca)
    std::vector<uint4> leafCells;      // cube-map cells (6 x leafGrid^2): up to 8 candidate leaves as
                                       // 16-bit ids (0xffff none); all 0xfffe: more, use the face locator
    uint32_t leafGrid = 0;
    std::vector<int> startCells;       // cube-map cells where point location starts. Adaptive (6 x
                                       // kSteerStartGrid^2): the quadtree code (>= 0 subdivided triangle,
                                       // < 0 ~leaf) of the deepest triangle that contains the whole cell,
                                       // INT32_MIN where no level-0 face does. Uniform (6 x
                                       // kSteerUniformStartGrid^2, empty when 0): ~leaf where one leaf
                                       // contains the whole cell, else INT32_MIN
    int root = 0;
    uint32_t numLeaves() const { return (uint32_t)leafArea.size(); }
    uint32_t numNodes() const { return (uint32_t)(nodeChild.size() / 8); }
};

constexpr int kSteerCells = 8;         // cube-map resolution of the face locator
#ifndef PG3_STEER_START_GRID
#define PG3_STEER_START_GRID 256
#endif
constexpr uint32_t kSteerStartGrid = PG3_STEER_START_GRID;   // cube-map resolution of the adaptive start cells
#ifndef PG3_STEER_UNIFORM_START_GRID
#define PG3_STEER_UNIFORM_START_GRID 256
#endif
constexpr uint32_t kSteerUniformStartGrid = PG3_STEER_UNIFORM_START_GRID;   // of the uniform levels' (0: none)
constexpr uint32_t kSteerLeafNone = 0xffffu, kSteerLeafMany = 0xfffeu;

// The geometry of subdivision level `level` (<= 7), built on first use and kept for the life of
// the process (thread-safe). Returns null with a message in err on failure.
const SteerGeom *steerGeometry(uint32_t level, std::string &err);

constexpr uint32_t kSteerMaxAdaptiveLevel = 12;
constexpr uint32_t kSteerMaxAdaptiveLeaves = 1u << 22;

// Adaptive triangulation of an RGB float map (W x H, row 0 at theta = 0) by the reference's
// refinement rule (TriangulateEm, src/em_steerable_sampler.hxx:2963-3472): a triangle below
// minLevel is subdivided, one at maxLevel is kept, and in between it is subdivided when the
// linear interpolation of its vertices' luminance differs from the map's bilinear luminance by
// more than the factor 1 + maxError at any of its test samples.
std::shared_ptr<SteerGeom> steerAdaptiveGeometry(const float *rgb, uint32_t W, uint32_t H, uint32_t minLevel,
                                                 uint32_t maxLevel, float maxError, std::string &err);

// The geometry of a given set of leaves (a file of the reference): every leaf must be a triangle
// of the icosahedron's 4-way subdivision at its stated level, the leaves must cover the sphere
// exactly once. corners: three unit directions per leaf. Built adaptive (quadtree locator).
std::shared_ptr<SteerGeom> steerGeometryFromLeaves(const std::vector<std::array<float, 9>> &corners,
                                                   const std::vector<uint32_t> &levels, uint32_t minLevel,
                                                   uint32_t maxLevel, float maxError, std::string &err);

// Luminance of the map's bilinear (tent) lookup in direction d, as the reference's
// EnvironmentMapImage::Evaluate (src/em_image.hxx:95-150) with Dir2LatLong (src/geom.hxx:78-95).
float emLuminanceDir(const float *rgb, uint32_t W, uint32_t H, float dx, float dy, float dz);

}  // namespace pg3
