// Flat exports of a built BVH: the reference's FastNodeManager view and the
// device layout used by the sm_103a kernels.
#pragma once
#include <cstdint>
#include <vector>

#include "bvh_builder.hpp"

namespace bvhgpu {

// FastNodeManager<gang, node_memory, wg> arrays (fastNodeManager.h:1495-1688).
struct FastView {
  int gang = 4, node_memory = 4, leaf_memory = 4;
  std::vector<float> bounds;       // n_nodes * 6 * node_memory
  std::vector<uint32_t> begin;     // childIdBegin / primIdBegin
  std::vector<int8_t> order;       // n_nodes * 3 * node_memory
  std::vector<uint32_t> child_type;
  std::vector<float> tri_points;   // trianglePoints
};
int export_fast(const Bvh& bvh, int gang, int node_memory, int leaf_memory, FastView& out);

// Device layout.
//
// Inner-node record for branching N (Nm = N rounded up to 4), 16-byte aligned:
//   float    box[6][Nm]     child boxes, SoA: lo.x lo.y lo.z hi.x hi.y hi.z
//   uint32   inner_base     index of the first inner child
//   uint32   leaf_base      index of the first leaf child
//   uint16   leaf_mask      bit j: child j is a leaf
//   uint8    count          number of children
//   uint8    depth          tree depth of this node
//   perm[3][2]              traverseOrderEachAxis as push sequences: for axis a,
//                           perm[a][0] pushes order[a][0], order[a][1], ...
//                           (direction[a] <= 0) and perm[a][1] pushes
//                           order[a][count-1], ..., order[a][0]; one child index
//                           per 4-bit nibble, first push in the low nibble;
//                           each word is perm_word_bytes(Nm) bytes
//   uint8    leaf_cnt[Nm]   triangles of leaf child j (0 for inner children)
// Leaves are not given node records: leaf k is the k-th leaf of the
// reference's customTreeOrder and its triangle block is exactly the
// reference's trianglePoints block (9 * leaf_memory floats, SoA with stride
// = count rounded up to the gang, sentinel (stride, NaN) in the last two
// floats when the stride is below leaf_memory).
//
// Q8 record (branching N, Nm as above), 16-byte aligned: N4 64 B, N8 80 B,
// N12 112 B, N16 144 B (FP32: 128 / 240 / 368 / 464 B):
//   float    origin[3]      parent box lower corner (the quantisation frame)
//   int8     exp[3], pad    per-axis power-of-two step: step = 2^exp
//   uint32   inner_base, leaf_base; uint16 leaf_mask; uint8 count; uint8 depth
//   nibble   leaf_cnt1[Nm]  triangles - 1 of leaf child j, 4 bits each (child j
//                           in bits 4j..4j+3 of the little-endian words; 0 for
//                           inner children), Nm / 2 bytes at 28
//   uint8    q[6][Nm]       child boxes at q8_box_offset: lo = origin + q_lo*step
//                           (rounded down), hi = origin + q_hi*step (rounded up)
// The push sequences perm[3][2] of a Q8 node live in a side array, not in its
// record: q8_perm_bytes(Nm) bytes per inner node in record order, read only by
// traversals that push hit children in the reference's order.
inline int perm_word_bytes(int nm) { return nm <= 4 ? 2 : (nm <= 8 ? 4 : 8); }
inline int fp32_meta_offset(int nm) { return 24 * nm; }
inline int q8_box_offset(int nm) { return (28 + nm / 2 + 3) / 4 * 4; }
inline int q8_perm_bytes(int nm) { return 6 * perm_word_bytes(nm); }
struct DeviceLayout {
  int branching = 4, node_stride = 4, leaf_memory = 4, gang = 4;
  int node_format = 0;
  int record_bytes = 0;
  std::vector<uint8_t> nodes;         // n_inner * record_bytes
  std::vector<uint8_t> q8_perm;       // Q8: n_inner * q8_perm_bytes push sequences
  // n_inner * node_stride: the stack entry of each child slot (the record's
  // leaf / inner numbering resolved per child; 0 for empty slots), read by
  // pushes in child-index order.
  std::vector<uint32_t> child_entry;
  std::vector<float> leaves;          // n_leaves * 9 * leaf_memory
  std::vector<uint32_t> leaf_prim;    // n_leaves * leaf_memory (input ids)
  std::vector<uint8_t> leaf_depth;    // n_leaves
  // n_leaves * 6 * leaf_memory: per triangle slot the smallest (rows 0-2)
  // and largest (rows 3-5) vertex coordinate along x, y, z (IEEE min / max
  // of the three vertices), read by the watertight box pre-test.
  std::vector<float> leaf_bounds;
  uint32_t n_inner = 0, n_leaves = 0;
  uint32_t root_entry = 0;            // stack entry of the root
  uint32_t top_nodes = 0;             // inner nodes laid out first
  // Every child box is finite with lo <= hi on each axis (FP32 records), so
  // a slab test may take the near / far planes by the sign of 1/direction.
  bool boxes_ordered = true;
};

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLeafCountShift = 27;
constexpr uint32_t kLeafIndexMask = (1u << 27) - 1;

inline int round_up(int v, int m) { return ((v + m - 1) / m) * m; }
inline int fp32_record_bytes(int nm) {
  return round_up(24 * nm + 12 + 6 * perm_word_bytes(nm) + nm, 16);
}
inline int q8_record_bytes(int nm) { return round_up(q8_box_offset(nm) + 6 * nm, 16); }

int build_device_layout(const Bvh& bvh, int gang, int leaf_memory, int node_format,
                        int top_levels, DeviceLayout& out);

// sahFactorConfigSse.txt (branchFactor, leafSize, sahNodeFactor).
float sah_factor_sse(int branching, int leaf_size, int gang);

}  // namespace bvhgpu
