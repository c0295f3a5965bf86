// Host-side SAH BVH builder and flat exporters.
//
// This is a C++ restatement of the reference's N-ary top-down SAH builder
// (src/accelerationStructure/aabb.cpp:71-206, aabb.h:40-67,113-147,
// node.h:66-91, node.cpp:254-275) and of its two flatteners:
//   * CompactNodeManager<CompactNodeV3> (compactNode.cpp:11-116), the node
//     view the instrumented renderer traverses;
//   * FastNodeManager<gang, nodeMemory, wg> (fastNodeManager.h:1495-1688),
//     the SoA node/leaf view the performance renderer traverses.
// It also emits the device layout consumed by the sm_103a kernels.
//
// Deliberate differences from the reference, all deterministic:
//   * std::stable_sort replaces std::sort(par_unseq) for the centre sorts
//     (aabb.h:63-66): the reference's order of equal centres is unspecified.
//   * children are built in parallel with std::thread over disjoint ranges,
//     which gives the same tree as a serial build.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

namespace bvhgpu {

struct BuildParams {
  int branching = 4;          // N: maximum children per node
  int leaf_size = 4;          // L: leaf target
  int sort_each_split = 1;    // config.txt sortEachSplit
  int leaf_split_option = 1;  // config.txt leafSplitOption (0, 1, 2)
  float sah_factor = 1.0f;    // sahFactorConfig*.txt sahNodeFactor
  int drop_zero_area = 1;     // gameobject.h:110-146 skips zero-area triangles
};

struct Triangle {
  float p[3][3];      // world-space points
  float bmin[3], bmax[3];
  float center[3];    // bmax*0.5 + bmin*0.5 (triangle.cpp:42-50)
  uint32_t id;        // index in the caller's triangle array
};

// A node of the built tree (reference numbering is assigned at flattening).
struct BuildNode {
  float bmin[3], bmax[3];
  uint32_t begin = 0, end = 0;  // primitive range; begin == end for inner nodes
  uint8_t depth = 0;
  std::vector<std::unique_ptr<BuildNode>> children;
  std::vector<int8_t> order[3];  // traverseOrderEachAxis
};

// Node of the CompactNodeV3 view, in reference (customTreeOrder) numbering.
struct CompactNode {
  float bmin[3], bmax[3];
  uint32_t child_begin;   // id of first child (0 for leaves)
  uint32_t child_count;   // 0 for leaves
  uint32_t prim_begin;    // index into the sorted primitive array
  uint32_t prim_count;    // 0 for inner nodes
  int8_t order[3][16];
  uint8_t depth;
};

class Bvh {
 public:
  BuildParams params;
  std::vector<Triangle> tris;       // in caller order (zero-area ones removed)
  std::vector<uint32_t> prims;      // sorted primitive array: indices into tris
  std::unique_ptr<BuildNode> root;
  std::vector<CompactNode> nodes;   // customTreeOrder numbering, root = 0
  std::vector<BuildNode*> node_ptr; // same numbering
  uint32_t leaf_count = 0;
  uint32_t inner_count = 0;
  int bvh_depth = 0;                // max leaf depth + 1 (bvh.cpp:360-364)
  int max_stack = 0;                // worst-case DFS stack height

  // Builds from T x 9 floats (p0, p1, p2). Returns 0 or a bvhgpu status.
  int build(const float* tri9, uint64_t n_tris, const BuildParams& p);

  // Adopts a tree built elsewhere (e.g. by the reference's own builder), given
  // as the CompactNodeV3 view that export_compact writes: nodes in reference
  // numbering (root 0, children consecutive and numbered after their parent),
  // order48[node*48 + axis*16 + i], primitives in sorted order with their
  // input ids. The structure is validated; depths and the worst-case stack
  // height are recomputed. Returns 0 or a bvhgpu status.
  int import_compact(uint64_t n_nodes, const float* lo3, const float* hi3,
                     const uint32_t* child_begin, const uint32_t* child_count,
                     const uint32_t* prim_begin, const uint32_t* prim_count,
                     const int8_t* order48, uint64_t n_prims, const uint32_t* prim_ids,
                     const float* prim_tri9, int branching, int leaf_size);

 private:
  std::vector<std::unique_ptr<BuildNode>> imported_;  // per-node orders of an imported tree
};

}  // namespace bvhgpu
