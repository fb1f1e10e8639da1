// Acceleration-structure formats shared by the host builder and the
// traversal kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

namespace wfpt {

// BVH2 node, 64 bytes: both children's FP32 boxes live in the parent.
//   f[0..3]  = c0.lo.x c0.hi.x c0.lo.y c0.hi.y
//   f[4..7]  = c1.lo.x c1.hi.x c1.lo.y c1.hi.y
//   f[8..11] = c0.lo.z c0.hi.z c1.lo.z c1.hi.z
//   link[0..1] = children: >= 0 inner node index, < 0 leaf ~(first<<3 | count-1)
struct Bvh2Node {
    float f[12];
    int32_t link[4];
};
static_assert(sizeof(Bvh2Node) == 64, "BVH2 node is 64 bytes");

// BVH8 node, 80 bytes (compressed wide BVH):
//   p[3]      FP32 origin of the quantisation grid
//   e[3]      biased exponents: scale_k = 2^(e_k-127)
//   imask     bit i set when child slot i is an inner node
//   child_base index of the first inner child (inner children are contiguous, in slot order)
//   tri_base  index of the first triangle of this node's leaf children
//   meta[8]   inner child: 0b001<<5 | (24+slot); leaf: unary count<<5 | triangle offset; empty: 0
//   q_lo/q_hi child boxes in grid units (floor / ceil), per axis
struct Bvh8Node {
    float p[3];
    uint8_t e[3];
    uint8_t imask;
    uint32_t child_base;
    uint32_t tri_base;
    uint8_t meta[8];
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8], qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(Bvh8Node) == 80, "BVH8 node is 80 bytes");

// Triangle record, 48 bytes: v0.xyz|prim, v1.xyz|geom, v2.xyz|global index.
struct TriRec {
    float v0[3];
    int32_t prim;
    float v1[3];
    int32_t geom;
    float v2[3];
    uint32_t global;
};
static_assert(sizeof(TriRec) == 48, "triangle record is 48 bytes");

struct HostBvh2 {
    std::vector<Bvh2Node> nodes;
    std::vector<TriRec> tris;
    int depth = 0;
};

struct HostBvh8 {
    std::vector<Bvh8Node> nodes;
    std::vector<TriRec> tris;
};

struct BuildInput {
    const float* positions;
    uint32_t num_vertices;
    const uint32_t* indices;
    uint32_t num_triangles;
    const uint32_t* geom_first;  // may be null
    uint32_t num_geoms;
};

// Binned-SAH BVH2 build with leaves of at most max_leaf triangles.
void build_bvh2(const BuildInput& in, int max_leaf, HostBvh2& out);
// Collapse of a BVH2 into the 8-wide format (leaf children <= 3 triangles),
// by the policy below.
void build_bvh8(const HostBvh2& bvh2, HostBvh8& out);
// Collapse policy: 1 = SAH dynamic programme (default), 0 = greedy; the
// triangle-test cost relative to a node step in percent (default 20).
void set_bvh8_collapse(int mode);
int get_bvh8_collapse();
void set_bvh8_tri_cost_pct(int pct);
int get_bvh8_tri_cost_pct();

// Persistent-traversal work counters: kWorkSlots slots of 16 u32 each
// (next ray, warps finished), zeroed at scene creation.
constexpr int kWorkSlots = 64;

struct SceneDevice {
    const float4* bvh2_nodes = nullptr;
    const float4* bvh2_tris = nullptr;
    const float4* bvh8_nodes = nullptr;
    const float4* bvh8_tris = nullptr;
    uint32_t bvh8_num_tris = 0;
    uint32_t* work = nullptr;
};

}  // namespace wfpt
