// bvh8.h -- host build of the 8-wide BVH with quantised child bounds.
//
// Replaces the reference's binary SAH build (src/geometry/bvh.cpp:65-323,
// 32-byte LinearBVHNode, two 1-D textures on the GPU) with:
//   1. a binned surface-area-heuristic binary build down to single
//      triangles (exact SAH sweep for ranges of at most 32);
//   2. an SAH-optimal collapse to 8-wide (or 4-wide) nodes by dynamic
//      programming (Ylitie et al., HPG 2017), which also groups triangles
//      into leaf slots of at most 3 (the reference's maxTrisInNode,
//      bvh.cpp:62);
//   3. child slots ordered by octant so that visiting slot k ^ octant(ray)
//      is approximately front to back;
//   4. child boxes quantised to 8 bits per plane relative to the node
//      origin with a power-of-two scale, rounded outward (conservative).
// Every triangle box is widened by a margin proportional to the scene's
// coordinate magnitude before the build, so the GPU's rounded slab tests
// never cull a triangle that the exact Moller-Trumbore test accepts.
#pragma once

#include <cstdint>
#include <vector>

namespace crt {

// 80-byte node, read on the GPU as five 16-byte loads.
struct alignas(16) Bvh8Node {
    float px, py, pz;          // quantisation origin
    uint8_t ex, ey, ez;        // biased exponents of the per-axis scale 2^(e-127)
    uint8_t imask;             // bit s: slot s is an internal node
    uint32_t child_base;       // index of the first internal child
    uint32_t tri_base;         // index of the first triangle record of the leaves
    uint8_t meta[8];           // 0 empty, 0x80 internal, else (count << 5) | offset
    uint8_t qlo[3][8];         // [axis][slot]
    uint8_t qhi[3][8];
};
static_assert(sizeof(Bvh8Node) == 80, "node layout");

// 208-byte node with full-precision child planes (same tree, same child and
// triangle layout as Bvh8Node), read as thirteen 16-byte loads.  Costs 2.6x
// the bytes of the quantised node but half the ALU work per child test.
struct alignas(16) Bvh8FloatNode {
    float lo[3][8];            // [axis][slot]; empty slot: lo = FLT_MAX, hi = -FLT_MAX
    float hi[3][8];
    uint32_t child_base_imask; // child_base | imask << 24
    uint32_t tri_base;
    uint8_t meta[8];
};
static_assert(sizeof(Bvh8FloatNode) == 208, "float node layout");

// 48-byte intersection record: v1.xyz + face index (bits), e1.xyz, e2.xyz.
struct alignas(16) TriRecord {
    float v1[3];
    uint32_t face;
    float e1[3];
    float pad1;
    float e2[3];
    float pad2;
};
static_assert(sizeof(TriRecord) == 48, "triangle layout");

struct Bvh8 {
    std::vector<Bvh8Node> nodes;
    std::vector<Bvh8FloatNode> fnodes;   // the same nodes with FP32 planes
    bool fnodes_ok = true;               // false beyond 2^24 nodes
    std::vector<TriRecord> tris;     // in leaf order
    uint32_t max_depth = 0;
    float margin = 0.f;
};

// v1/e1/e2: [n][3] floats as the scene computes them (e = v - v1, in FP32).
// Returns false (with msg) if the scene is empty or the tree exceeds
// max_levels levels.
// max_children: 8, or 4 for a narrower tree stored in the same node layout.
bool build_bvh8(const float* v1, const float* e1, const float* e2, uint32_t n,
                uint32_t max_levels, Bvh8& out, const char** msg, int max_children = 8);

}  // namespace crt
