// Traversal kernels, templated on the branching factor N (node record size),
// the profile (instrumented / fast), the ray kind (closest / any) and whether
// per-ray counters are recorded.
//
// Semantics (identical for both schemes and matching the reference per ray):
//   * the root's own box is never tested; traversal starts by popping it
//     (fastNodeManager.h:1334-1349, compactNode.cpp:610-621);
//   * an inner node tests every child box with the ray's current tMax and
//     pushes the hit children in traverseOrderEachAxis[code] order, ascending
//     when direction[code] <= 0 and descending otherwise, so the child nearest
//     along the major axis is popped first (compactNode.cpp:781-809). Fast
//     any-hit rays push in child-index order (fastNodeManager.h:1481-1488);
//   * stack entries are not re-culled when popped (useDistance == false);
//   * a leaf tests all its triangles; closest hits shrink tMax as they go;
//     any-hit rays end at the first leaf with a hit (compactNode.cpp:690-706,
//     fastNodeManager.h:1444-1461).
#pragma once
#include "device_common.cuh"

namespace bvhgpu {
namespace dev {

struct SceneDev {
  const uint8_t* nodes;       // inner-node records
  const float* leaves;        // leaf triangle blocks (9 * leaf_memory floats each)
  const uint32_t* leaf_prim;  // leaf_memory input ids per leaf
  const uint8_t* leaf_depth;  // tree depth per leaf
  uint32_t root_entry;
  uint32_t top_nodes;         // inner records laid out first (staged in shared memory)
  int leaf_memory;
  int gang;
  int* status;                // first device-side error (0 = none)
  // FP32 records whose child boxes are all finite with lo <= hi: NaN-free
  // rays may take the near / far slab form (see visit_node).
  int boxes_ordered;
  // Any-hit rays without counters push hit children in child-index order
  // (bvhgpu_trace_opts_t.any_order), else in the profile's order.
  int any_index_order = 0;
  // Q8 records: the push sequences, NodeFmt<N, Q8>::PSB bytes per inner node.
  const uint8_t* q8_perm = nullptr;
  // NodeFmt<N>::NM stack entries per inner node, one per child slot (null:
  // computed from the record).
  const uint32_t* child_entry = nullptr;
  // 6 * leaf_memory floats per leaf: each triangle slot's vertex minima
  // (rows 0-2) and maxima (rows 3-5) per axis (read when BVHGPU_LEAF_BOUNDS).
  const float* leaf_bounds = nullptr;
};

#ifndef BVHGPU_NEARFAR
#define BVHGPU_NEARFAR 1
#endif
// 1: the slab tests of NaN-free rays (near / far and min / max forms)
// compute two children's plane distances per packed f32x2 subtract and
// multiply; 0: one child per instruction.
#ifndef BVHGPU_PAIRED_SLABS
#define BVHGPU_PAIRED_SLABS 1
#endif
// 1: the instrumented profile's watertight pre-test reads the triangles'
// stored bounds (SceneDev::leaf_bounds, which every scene view then carries)
// and loads a triangle's vertices only when it passes.
#ifndef BVHGPU_LEAF_BOUNDS
#define BVHGPU_LEAF_BOUNDS 1
#endif
// Leaf visits with stored bounds: all pre-tests first, then the full tests of
// the passing triangles only; 1: any-hit rays, 2: any-hit and closest-hit
// rays, 0: neither.
#ifndef BVHGPU_LEAF_COMPACT
#define BVHGPU_LEAF_COMPACT 2
#endif
// 1: pushes of hit children in child-index order read their stack entries
// from SceneDev::child_entry; 0: computed from the record.
#ifndef BVHGPU_ENTRY_PUSH
#define BVHGPU_ENTRY_PUSH 1
#endif
// 1: Q8 records take the paired slab test too, decoded two children per
// packed instruction.
#ifndef BVHGPU_PAIRED_Q8
#define BVHGPU_PAIRED_Q8 1
#endif
// 1: leaf triangles loaded four at a time with 128-bit loads; 0: one at a time.
#ifndef BVHGPU_LEAF_VEC
#define BVHGPU_LEAF_VEC 1
#endif

struct TraceArgs {
  const bvhgpu_ray_t* rays;
  uint64_t n;
  bvhgpu_hit_t* hits;
  uint8_t* occluded;
  uint32_t* counters;
  unsigned long long* depth_hist;
  // With counters: visits of nodes with c children (fullness[c]) and of
  // leaves with c triangles (fullness[17 + c]), c <= 16: the reference's
  // Ray::childFullness / primitiveFullness (ray.h:36-37) summed over the rays.
  unsigned long long* fullness = nullptr;
  int stack_cap;              // stack entries per ray
  // Reordered traces: the i-th ray the kernel takes is input ray
  // out_index[i] (null: i), and its results go to that input slot.
  const uint32_t* out_index = nullptr;
  // Stream scheme with counters: per packet and step, (node work, unique
  // nodes, leaf work, unique leaves, terminations) into
  // step_stats[(packet * step_cap + step) * 5 ..] for steps < step_cap, and
  // the packet's step count (with step 0, the set-up) into step_count[packet].
  uint32_t* step_stats = nullptr;
  uint32_t* step_count = nullptr;
  int step_cap = 0;
  // Step log of intersectWide's schedule (a node visit followed by a leaf
  // visit counts as one step) instead of intersectWideAlternative's.
  bool step_wide = false;
};

BVHGPU_DEV uint64_t out_slot(const TraceArgs& a, uint64_t rid) {
  return a.out_index ? (uint64_t)__ldg(a.out_index + rid) : rid;
}

struct Counters {
  uint32_t node_visits = 0, leaf_visits = 0, box_tests = 0, box_hits = 0;
  uint32_t tri_tests = 0, tri_hits = 0, max_stack = 0;
};

constexpr int round4(int n) { return (n + 3) / 4 * 4; }

// Node record formats (the byte layouts are written by build_device_layout).
constexpr int kFmtFP32 = BVHGPU_NODES_FP32;
constexpr int kFmtQ8 = BVHGPU_NODES_Q8;

template <int N, int FMT = kFmtFP32>
struct NodeFmt {
  static constexpr int NM = round4(N);
  // Push-sequence word: one nibble per child.
  static constexpr int PW = NM <= 4 ? 2 : (NM <= 8 ? 4 : 8);
  // FP32: float box[6][NM] | meta (12 B) | perm[3][2] | leaf_cnt[NM]
  // Q8:   origin (3 f32) + exp (3 i8) | meta | (leaf_cnt - 1) nibbles | q[6][NM];
  //       perm[3][2] in the side array (PSB bytes per node)
  static constexpr int META = FMT == kFmtFP32 ? 24 * NM : 16;
  static constexpr int PERM = META + 12;  // FP32 only
  static constexpr int LCNT = FMT == kFmtFP32 ? PERM + 6 * PW : META + 12;
  static constexpr int PSB = 6 * PW;
  static constexpr int QBOX = (28 + NM / 2 + 3) / 4 * 4;
  static constexpr int REC = FMT == kFmtFP32 ? ((24 * NM + 12 + 6 * PW + NM) + 15) / 16 * 16
                                             : ((QBOX + 6 * NM) + 15) / 16 * 16;
};

// Loads from a node record, either in global memory (read-only path) or in
// the block's shared-memory copy of the top levels (generic loads).
template <bool SH> BVHGPU_DEV uint4 rec_u4(const uint8_t* p) {
  if (SH) return *reinterpret_cast<const uint4*>(p);
  return ldgu4(p);
}
template <bool SH> BVHGPU_DEV float4 rec_f4(const uint8_t* p) {
  if (SH) return *reinterpret_cast<const float4*>(p);
  return ldg4(p);
}
template <bool SH> BVHGPU_DEV uint32_t rec_u32(const uint8_t* p) {
  if (SH) return *reinterpret_cast<const uint32_t*>(p);
  return ldgu(p);
}

// Byte i (0 <= i < 16) of a little-endian 16-byte group held as two words.
BVHGPU_DEV int byte_at(uint64_t lo, uint64_t hi, int i) {
  uint64_t w = i >= 8 ? hi : lo;
  return (int)((w >> ((i & 7) * 8)) & 0xFFu);
}

template <int NM, bool SH>
BVHGPU_DEV void load_bytes(const uint8_t* p, uint64_t& lo, uint64_t& hi) {
  // NM bytes at a 4-byte aligned address.
  uint32_t w0 = rec_u32<SH>(p), w1 = NM > 4 ? rec_u32<SH>(p + 4) : 0u;
  uint32_t w2 = NM > 8 ? rec_u32<SH>(p + 8) : 0u, w3 = NM > 12 ? rec_u32<SH>(p + 12) : 0u;
  lo = (uint64_t)w0 | ((uint64_t)w1 << 32);
  hi = (uint64_t)w2 | ((uint64_t)w3 << 32);
}

// 2^e for a normal exponent e (-126 <= e <= 127).
BVHGPU_DEV float exp2i(int e) { return __int_as_float((e + 127) << 23); }

// Byte k of w as a float, exactly: the byte placed in the mantissa of
// 2^23 (one byte permute), minus 2^23. Full-rate ALU and FP32 instructions
// instead of an integer-to-float conversion.
template <int K>
BVHGPU_DEV float byte_to_float(uint32_t w) {
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u | K)) - 8388608.0f;
}

// Four children's Q8 coordinates of one row: origin + q * step, rounded
// down (lower bounds) or up (upper bounds). q * step is exact (q < 256,
// step a power of two), so the decoded box contains the original one.
BVHGPU_DEV float4 q8_row(uint32_t w, float origin, float step, bool up) {
  float4 v;
  const float a = byte_to_float<0>(w) * step, b = byte_to_float<1>(w) * step;
  const float c = byte_to_float<2>(w) * step, d = byte_to_float<3>(w) * step;
  if (up) {
    v.x = __fadd_ru(origin, a); v.y = __fadd_ru(origin, b);
    v.z = __fadd_ru(origin, c); v.w = __fadd_ru(origin, d);
  } else {
    v.x = __fadd_rd(origin, a); v.y = __fadd_rd(origin, b);
    v.z = __fadd_rd(origin, c); v.w = __fadd_rd(origin, d);
  }
  return v;
}

// q8_row as two packed pairs (children 0-1 and 2-3): the same bytes, the
// same exact products and the same directed rounding per half.
BVHGPU_DEV void q8_row2(uint32_t w, uint64_t origin2, uint64_t step2, bool up, uint64_t& p01,
                        uint64_t& p23) {
  const uint64_t bias = f2splat(8388608.0f);
  const uint64_t b01 = f2pack(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u)),
                              __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7541u)));
  const uint64_t b23 = f2pack(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7542u)),
                              __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7543u)));
  const uint64_t q01 = f2mul(f2sub(b01, bias), step2), q23 = f2mul(f2sub(b23, bias), step2);
  p01 = up ? f2add_ru(origin2, q01) : f2add_rd(origin2, q01);
  p23 = up ? f2add_ru(origin2, q23) : f2add_rd(origin2, q23);
}

// One inner-node visit: slab-test the children and push the hits.
// Returns false on stack overflow.
// DIST: the save-distance traversal; each push also stores the child's entry
// distance in dstack (same slot layout as stack).
// NF: near / far form of the IEEE slab test for FP32 records whose boxes are
// ordered (SceneDev::boxes_ordered) and NaN-free rays: per axis the near
// plane is the low one when 1/d >= 0, else the high one, so the per-child
// min / max pair of slab_mm disappears. With lo <= hi, (lo - o) * inv and
// (hi - o) * inv are ordered by the sign of inv (rounding is monotonic), so
// fminf / fmaxf of slab_mm return exactly the near / far values: same t0, t1
// and boolean.
template <int N, int PROFILE, int KIND, bool COUNT, bool MM, int FMT, bool SH, bool DIST = false,
          bool NF = false>
BVHGPU_DEV bool visit_node(const uint8_t* rec, const Ray& r, float tmax, uint32_t* stack,
                           int stride, int& sp, int cap, Counters& ctr, int& depth_out,
                           float* dstack = nullptr, bool index_order = false,
                           const uint8_t* q8_side = nullptr, const uint32_t* ent = nullptr) {
  using F = NodeFmt<N, FMT>;
  constexpr int NM = F::NM;
  const uint4 meta = rec_u4<SH>(rec + F::META);
  const uint32_t inner_base = meta.x, leaf_base = meta.y;
  const uint32_t leaf_mask = meta.z & 0xFFFFu;
  const int count = (int)((meta.z >> 16) & 0xFFu);
  depth_out = (int)(meta.z >> 24) | (count << 8);  // depth | child count << 8

  float ox = 0.f, oy = 0.f, oz = 0.f, sx = 0.f, sy = 0.f, sz = 0.f;
  if (FMT == kFmtQ8) {
    const uint4 h = rec_u4<SH>(rec);
    ox = __uint_as_float(h.x);
    oy = __uint_as_float(h.y);
    oz = __uint_as_float(h.z);
    sx = exp2i((int)(int8_t)(h.w & 0xFFu));
    sy = exp2i((int)(int8_t)((h.w >> 8) & 0xFFu));
    sz = exp2i((int)(int8_t)((h.w >> 16) & 0xFFu));
  }
  uint32_t hit = 0;
  float dist[NM];
  if (NF) {
    // Row of the near plane per axis (0..2 low, 3..5 high); far = near ^ 3 + ...
    const int nx = r.inv[0] >= 0.0f ? 0 : 3, ny = r.inv[1] >= 0.0f ? 1 : 4;
    const int nz = r.inv[2] >= 0.0f ? 2 : 5;
    const int fx = nx == 0 ? 3 : 0, fy = ny == 1 ? 4 : 1, fz = nz == 2 ? 5 : 2;
#if BVHGPU_PAIRED_SLABS
    // Two children per subtract and multiply (f2plane); the minima, maxima
    // and the comparison stay per child.
    const uint64_t o2x = f2pack(r.o[0], r.o[0]), o2y = f2pack(r.o[1], r.o[1]);
    const uint64_t o2z = f2pack(r.o[2], r.o[2]);
    const uint64_t s2x = f2pack(r.inv[0], r.inv[0]), s2y = f2pack(r.inv[1], r.inv[1]);
    const uint64_t s2z = f2pack(r.inv[2], r.inv[2]);
#endif
#pragma unroll
    for (int q = 0; q < NM / 4; ++q) {
      const float4 ax = rec_f4<SH>(rec + (nx * NM + 4 * q) * 4);
      const float4 bx = rec_f4<SH>(rec + (fx * NM + 4 * q) * 4);
      const float4 ay = rec_f4<SH>(rec + (ny * NM + 4 * q) * 4);
      const float4 by = rec_f4<SH>(rec + (fy * NM + 4 * q) * 4);
      const float4 az = rec_f4<SH>(rec + (nz * NM + 4 * q) * 4);
      const float4 bz = rec_f4<SH>(rec + (fz * NM + 4 * q) * 4);
#if BVHGPU_PAIRED_SLABS
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        if (4 * q + 2 * p < N) {
          const int k = 2 * p;
          const float2 nxp = f2plane(f4get(ax, k), f4get(ax, k + 1), o2x, s2x);
          const float2 fxp = f2plane(f4get(bx, k), f4get(bx, k + 1), o2x, s2x);
          const float2 nyp = f2plane(f4get(ay, k), f4get(ay, k + 1), o2y, s2y);
          const float2 fyp = f2plane(f4get(by, k), f4get(by, k + 1), o2y, s2y);
          const float2 nzp = f2plane(f4get(az, k), f4get(az, k + 1), o2z, s2z);
          const float2 fzp = f2plane(f4get(bz, k), f4get(bz, k + 1), o2z, s2z);
          float t0 = fmaxf(fmaxf(fmaxf(nxp.x, 0.0f), nyp.x), nzp.x);
          float t1 = fminf(fminf(fminf(fxp.x, tmax), fyp.x), fzp.x);
          hit |= (uint32_t)(t0 <= t1) << (4 * q + k);
          if (4 * q + k + 1 < N) {
            t0 = fmaxf(fmaxf(fmaxf(nxp.y, 0.0f), nyp.y), nzp.y);
            t1 = fminf(fminf(fminf(fxp.y, tmax), fyp.y), fzp.y);
            hit |= (uint32_t)(t0 <= t1) << (4 * q + k + 1);
          }
        }
      }
#else
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (4 * q + k < N) {
          float t0 = fmaxf((f4get(ax, k) - r.o[0]) * r.inv[0], 0.0f);
          float t1 = fminf((f4get(bx, k) - r.o[0]) * r.inv[0], tmax);
          t0 = fmaxf((f4get(ay, k) - r.o[1]) * r.inv[1], t0);
          t1 = fminf((f4get(by, k) - r.o[1]) * r.inv[1], t1);
          t0 = fmaxf((f4get(az, k) - r.o[2]) * r.inv[2], t0);
          t1 = fminf((f4get(bz, k) - r.o[2]) * r.inv[2], t1);
          hit |= (uint32_t)(t0 <= t1) << (4 * q + k);
        }
      }
#endif
    }
  } else if (BVHGPU_PAIRED_SLABS && MM && !DIST && (FMT == kFmtFP32 || BVHGPU_PAIRED_Q8)) {
    // slab_mm with two children per subtract and multiply (and per Q8
    // decode step), one axis at a time: t0 / t1 take the axes in slab_mm's
    // order.
#pragma unroll
    for (int q = 0; q < NM / 4; ++q) {
      float t0[4], t1[4];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        uint64_t lo[2], hi[2];
        if (FMT == kFmtFP32) {
          const float4 l = rec_f4<SH>(rec + (a * NM + 4 * q) * 4);
          const float4 h = rec_f4<SH>(rec + ((3 + a) * NM + 4 * q) * 4);
          lo[0] = f2pack(l.x, l.y);
          lo[1] = f2pack(l.z, l.w);
          hi[0] = f2pack(h.x, h.y);
          hi[1] = f2pack(h.z, h.w);
        } else {
          const float qo = a == 0 ? ox : (a == 1 ? oy : oz);
          const float qs = a == 0 ? sx : (a == 1 ? sy : sz);
          const uint8_t* qb = rec + F::QBOX + 4 * q;
          q8_row2(rec_u32<SH>(qb + a * NM), f2splat(qo), f2splat(qs), false, lo[0], lo[1]);
          q8_row2(rec_u32<SH>(qb + (3 + a) * NM), f2splat(qo), f2splat(qs), true, hi[0], hi[1]);
        }
        const uint64_t o2 = f2splat(r.o[a]), s2 = f2splat(r.inv[a]);
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          if (4 * q + 2 * p < N) {
            const float2 tn = f2unpack(f2mul(f2sub(lo[p], o2), s2));
            const float2 tf = f2unpack(f2mul(f2sub(hi[p], o2), s2));
            const float mn[2] = {fminf(tn.x, tf.x), fminf(tn.y, tf.y)};
            const float mx[2] = {fmaxf(tn.x, tf.x), fmaxf(tn.y, tf.y)};
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int k = 2 * p + j;
              t0[k] = fmaxf(mn[j], a == 0 ? 0.0f : t0[k]);
              t1[k] = fminf(mx[j], a == 0 ? tmax : t1[k]);
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (4 * q + k < N) hit |= (uint32_t)(t0[k] <= t1[k]) << (4 * q + k);
    }
  } else
#pragma unroll
  for (int q = 0; q < NM / 4; ++q) {
    float4 lx, ly, lz, hx, hy, hz;
    if (FMT == kFmtFP32) {
      lx = rec_f4<SH>(rec + (0 * NM + 4 * q) * 4);
      ly = rec_f4<SH>(rec + (1 * NM + 4 * q) * 4);
      lz = rec_f4<SH>(rec + (2 * NM + 4 * q) * 4);
      hx = rec_f4<SH>(rec + (3 * NM + 4 * q) * 4);
      hy = rec_f4<SH>(rec + (4 * NM + 4 * q) * 4);
      hz = rec_f4<SH>(rec + (5 * NM + 4 * q) * 4);
    } else {
      const uint8_t* qb = rec + F::QBOX + 4 * q;
      lx = q8_row(rec_u32<SH>(qb + 0 * NM), ox, sx, false);
      ly = q8_row(rec_u32<SH>(qb + 1 * NM), oy, sy, false);
      lz = q8_row(rec_u32<SH>(qb + 2 * NM), oz, sz, false);
      hx = q8_row(rec_u32<SH>(qb + 3 * NM), ox, sx, true);
      hy = q8_row(rec_u32<SH>(qb + 4 * NM), oy, sy, true);
      hz = q8_row(rec_u32<SH>(qb + 5 * NM), oz, sz, true);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (4 * q + k < N) {
        bool h;
        if (DIST)
          h = slab_dist<MM>(f4get(lx, k), f4get(ly, k), f4get(lz, k), f4get(hx, k),
                            f4get(hy, k), f4get(hz, k), r, tmax, dist[4 * q + k]);
        else
          h = slab_t<MM>(f4get(lx, k), f4get(ly, k), f4get(lz, k), f4get(hx, k),
                         f4get(hy, k), f4get(hz, k), r, tmax);
        hit |= (uint32_t)h << (4 * q + k);
      }
    }
  }
  hit &= (1u << count) - 1u;
  if (COUNT) {
    ctr.node_visits++;
    ctr.box_tests += (uint32_t)count;
    ctr.box_hits += (uint32_t)__popc(hit);
  }
  if (hit == 0) return true;

  // Leaf child counts: bytes (FP32 records) or (count - 1) nibbles (Q8).
  uint64_t clo = 0, chi = 0;
  uint32_t n0 = 0, n1 = 0;
  if (FMT == kFmtFP32) {
    load_bytes<NM, SH>(rec + F::LCNT, clo, chi);
  } else {
    n0 = rec_u32<SH>(rec + F::LCNT);
    if (NM > 8) n1 = rec_u32<SH>(rec + F::LCNT + 4);
  }
  auto entry = [&](int c) -> uint32_t {
    const uint32_t below = (1u << c) - 1u;
    if ((leaf_mask >> c) & 1u) {
      uint32_t cnt1;
      if (FMT == kFmtFP32) cnt1 = (uint32_t)byte_at(clo, chi, c) - 1u;
      else cnt1 = ((c < 8 ? n0 >> (4 * c) : n1 >> (4 * (c - 8)))) & 15u;
      return kLeafBit | (cnt1 << kLeafCountShift) |
             (leaf_base + (uint32_t)__popc(leaf_mask & below));
    }
    return inner_base + (uint32_t)__popc(~leaf_mask & below);
  };
  // Push sequence: child-index order for fast any-hit rays
  // (fastNodeManager.h:1481-1488), else traverseOrderEachAxis[code] in the
  // ray's direction: ascending positions of the stored sequence when
  // direction[code] <= 0, descending otherwise (compactNode.cpp:781-809).
  // pm holds the positions of the hit children, built from the inverse
  // sequence over the hit children only. With index_order, any-hit rays
  // without counters take child-index order in both profiles: tMax stays
  // fixed until the first hit, which ends the ray, so the order in which
  // the reachable leaves are tested changes no result.
  uint64_t perm;
  uint32_t pm;
  bool descending = false;
  if (KIND == BVHGPU_ANY && (PROFILE == BVHGPU_PROFILE_FAST || (!COUNT && index_order))) {
    if (BVHGPU_ENTRY_PUSH && ent != nullptr) {
      // The children's stack entries precomputed per slot: the same pushes
      // as the loop below (ascending child index), one load per push instead
      // of the record decode and the sequence lookup.
      if (sp + __popc(hit) > cap) return false;
      uint32_t h = hit;
      while (h) {
        const int c = __ffs(h) - 1;
        h &= h - 1u;
        stack[sp * stride] = __ldg(ent + c);
        ++sp;
      }
      return true;
    }
    perm = 0xFEDCBA9876543210ull;
    pm = hit;
  } else {
    // FP32: in the record (shared-memory copy or global); Q8: the side array
    // (global).
    constexpr bool PSH = SH && FMT == kFmtFP32;
    const uint8_t* pp = (FMT == kFmtFP32 ? rec + F::PERM : q8_side) + r.code * 2 * F::PW;
    uint64_t inv;
    if (F::PW == 2) {
      const uint32_t w = rec_u32<PSH>(pp);  // sequence | inverse << 16, 4-byte aligned
      perm = w & 0xFFFFu;
      inv = w >> 16;
    } else if (F::PW == 4) {
      perm = rec_u32<PSH>(pp);
      inv = rec_u32<PSH>(pp + 4);
    } else {
      perm = (uint64_t)rec_u32<PSH>(pp) | ((uint64_t)rec_u32<PSH>(pp + 4) << 32);
      inv = (uint64_t)rec_u32<PSH>(pp + 8) | ((uint64_t)rec_u32<PSH>(pp + 12) << 32);
    }
    pm = 0;
    uint32_t h = hit;
    while (h) {
      const int c = __ffs(h) - 1;
      h &= h - 1u;
      pm |= 1u << (uint32_t)((inv >> (4 * c)) & 15u);
    }
    descending = !r.reverse;
  }
  while (pm) {
    const int k = descending ? 31 - __clz(pm) : __ffs(pm) - 1;
    pm &= ~(1u << k);
    const int c = (int)((perm >> (4 * k)) & 15u);
    if (sp >= cap) return false;
    stack[sp * stride] = entry(c);
    if (DIST) {
      float tc = 0.f;
#pragma unroll
      for (int j = 0; j < NM; ++j)
        if (j == c) tc = dist[j];
      dstack[sp * stride] = tc;
    }
    ++sp;
  }
  return true;
}

// Best closest hit found so far.
struct Best {
  uint32_t leaf = 0xFFFFFFFFu;
  int lane = -1;
  float u = 0.f, v = 0.f;
};

// One leaf visit. Closest rays update tmax / best; any-hit rays return true
// on a hit. With COUNT false, any-hit rays stop at the first hit triangle
// (the leaf's result is the same); with COUNT true all triangles are tested
// like the reference.
template <int PROFILE, int KIND, bool COUNT, bool MM>
BVHGPU_DEV bool visit_leaf_points(const SceneDev& sc, uint32_t e, const Ray& r, float& tmax,
                                  Best& best, Counters& ctr) {
  const uint32_t leaf = e & kLeafIndexMask;
  const int cnt = (int)((e >> kLeafCountShift) & 15u) + 1;
  const int gang = sc.gang;
  const int stride = ((cnt - 1) / gang + 1) * gang;
  const float* blk = sc.leaves + (size_t)leaf * 9 * sc.leaf_memory;
  if (COUNT) {
    ctr.leaf_visits++;
    ctr.tri_tests += (uint32_t)cnt;
  }
  bool any = false;
  // Fast profile closest hit: per-gang-lane minima of triIntersect{L}.
  float leaf_best = 1000000.0f;
  int winner = -1;
  uint32_t lanes_at_best = 0;
  float wu = 0.f, wv = 0.f;

  // Row offsets: instrumented rays read the permuted axes directly.
  int ax0 = 0, ax1 = 1, ax2 = 2;
  if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) { ax0 = r.kx; ax1 = r.ky; ax2 = r.code; }
#if BVHGPU_LEAF_VEC
  for (int g = 0; g < cnt; g += 4) {
    float4 c[3][3];
#pragma unroll
    for (int v = 0; v < 3; ++v) {
      c[v][0] = ldg4(blk + (v * 3 + ax0) * stride + g);
      c[v][1] = ldg4(blk + (v * 3 + ax1) * stride + g);
      c[v][2] = ldg4(blk + (v * 3 + ax2) * stride + g);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = g + k;
      if (i >= cnt) break;
      float p[3][3];
#pragma unroll
      for (int v = 0; v < 3; ++v)
#pragma unroll
        for (int a = 0; a < 3; ++a) p[v][a] = f4get(c[v][a], k);
#else
  {
    for (int i = 0; i < cnt; ++i) {
      float p[3][3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        p[v][0] = __ldg(blk + (v * 3 + ax0) * stride + i);
        p[v][1] = __ldg(blk + (v * 3 + ax1) * stride + i);
        p[v][2] = __ldg(blk + (v * 3 + ax2) * stride + i);
      }
#endif
      float t, b1, b2;
      bool h;
      if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED)
        h = watertight<MM>(p, r, tmax, t, b1, b2);
      else
        h = moller_trumbore(p, r, tmax, t, b1, b2);
      if (!h) continue;
      if (KIND == BVHGPU_ANY) {
        if (COUNT) ctr.tri_hits++;
        any = true;
        if (!COUNT) return true;
        continue;
      }
      if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) {
        // Each accepted triangle overwrites the hit (triangle.cpp:243).
        if (COUNT) ctr.tri_hits++;
        tmax = t;
        best.leaf = leaf;
        best.lane = i;
        best.u = b1;
        best.v = b2;
        any = true;
      } else {
        // triIntersect{L}: lane i % gang keeps its first minimum below its
        // running value (initially 1e6); the result is the largest index
        // among lanes whose minimum equals the leaf minimum
        // (rayTracerTemplate.ispc:28-101).
        if (COUNT) ctr.tri_hits++;
        const uint32_t lane_bit = 1u << (i % gang);
        if (t < leaf_best) {
          leaf_best = t;
          winner = i;
          lanes_at_best = lane_bit;
          wu = b1;
          wv = b2;
        } else if (winner >= 0 && t == leaf_best && !(lanes_at_best & lane_bit)) {
          winner = i;
          lanes_at_best |= lane_bit;
          wu = b1;
          wv = b2;
        }
      }
    }
  }
  if (KIND == BVHGPU_CLOSEST && PROFILE == BVHGPU_PROFILE_FAST && winner >= 0) {
    tmax = leaf_best;
    best.leaf = leaf;
    best.lane = winner;
    best.u = wu;
    best.v = wv;
    any = true;
  }
  return any;
}

// visit_leaf for the instrumented profile with NaN-free rays: watertight()'s
// box pre-test from the stored bounds (SceneDev::leaf_bounds). Rounding of
// a - o is monotonic in a, so (min(p) - o) * inv is the min(p - o) * inv that
// watertight() computes, and the IEEE minima / maxima over the axes do not
// depend on their order. Two triangles per packed subtract and multiply; a
// triangle's vertices are loaded only when it passes (about one test in six
// for ambient-occlusion rays).
template <int KIND, bool COUNT, bool MM>
BVHGPU_DEV bool visit_leaf_bounds(const SceneDev& sc, uint32_t e, const Ray& r, float& tmax,
                                  Best& best, Counters& ctr) {
  const uint32_t leaf = e & kLeafIndexMask;
  const int cnt = (int)((e >> kLeafCountShift) & 15u) + 1;
  const int gang = sc.gang;
  const int stride = ((cnt - 1) / gang + 1) * gang;
  const float* blk = sc.leaves + (size_t)leaf * 9 * sc.leaf_memory;
  if (COUNT) {
    ctr.leaf_visits++;
    ctr.tri_tests += (uint32_t)cnt;
  }
  bool any = false;
  const int ax0 = r.kx, ax1 = r.ky, ax2 = r.code;
  const int lm = sc.leaf_memory;
  const float* bnd = sc.leaf_bounds + (size_t)leaf * 6 * lm;
  if ((BVHGPU_LEAF_COMPACT >= 1 && KIND == BVHGPU_ANY) || BVHGPU_LEAF_COMPACT >= 2) {
    // Every pre-test of the leaf first, with the tMax the ray enters the
    // leaf with: a mask of the triangles that pass, then the full tests of
    // those only, in ascending order as below. The warp then runs as many
    // full tests as its lanes have passing triangles at most (about one in
    // six passes for ambient-occlusion rays), not one per triangle slot in
    // which any lane passes. Any-hit rays keep tMax; a closest-hit ray whose
    // tMax fell at an earlier hit in this leaf repeats the pre-test's tMax
    // condition (the only one that depends on tMax) before a full test.
    uint32_t pass = 0;
    for (int g = 0; g < cnt; g += 4) {
      float lo[4][3], hi[4][3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float4 mn = ldg4(bnd + a * lm + g), mx = ldg4(bnd + (3 + a) * lm + g);
        const uint64_t o2 = f2splat(r.o[a]), s2 = f2splat(r.inv[a]);
        const float2 n01 = f2unpack(f2mul(f2sub(f2pack(mn.x, mn.y), o2), s2));
        const float2 n23 = f2unpack(f2mul(f2sub(f2pack(mn.z, mn.w), o2), s2));
        const float2 x01 = f2unpack(f2mul(f2sub(f2pack(mx.x, mx.y), o2), s2));
        const float2 x23 = f2unpack(f2mul(f2sub(f2pack(mx.z, mx.w), o2), s2));
        lo[0][a] = n01.x; lo[1][a] = n01.y; lo[2][a] = n23.x; lo[3][a] = n23.y;
        hi[0][a] = x01.x; hi[1][a] = x01.y; hi[2][a] = x23.x; hi[3][a] = x23.y;
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float tmin = fmaxf(fmaxf(fminf(lo[k][0], hi[k][0]), fminf(lo[k][1], hi[k][1])),
                                 fminf(lo[k][2], hi[k][2]));
        const float tmx = fminf(fminf(fmaxf(lo[k][0], hi[k][0]), fmaxf(lo[k][1], hi[k][1])),
                                fmaxf(lo[k][2], hi[k][2]));
        if (!(tmx < 0 || tmin > tmx || tmax < tmin)) pass |= 1u << (g + k);
      }
    }
    pass &= (1u << cnt) - 1u;  // slots past the leaf's count hold padding
    const float tmax_in = tmax;
    while (pass) {
      const int i = __ffs(pass) - 1;
      pass &= pass - 1u;
      if (KIND == BVHGPU_CLOSEST && tmax != tmax_in) {
        float m[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float lo = (__ldg(bnd + a * lm + i) - r.o[a]) * r.inv[a];
          const float hi = (__ldg(bnd + (3 + a) * lm + i) - r.o[a]) * r.inv[a];
          m[a] = fminf(lo, hi);
        }
        if (tmax < fmaxf(fmaxf(m[0], m[1]), m[2])) continue;
      }
      float p[3][3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        p[v][0] = __ldg(blk + (v * 3 + ax0) * stride + i);
        p[v][1] = __ldg(blk + (v * 3 + ax1) * stride + i);
        p[v][2] = __ldg(blk + (v * 3 + ax2) * stride + i);
      }
      float t, b1, b2;
      if (!watertight<MM, false>(p, r, tmax, t, b1, b2)) continue;
      if (COUNT) ctr.tri_hits++;
      any = true;
      if (KIND == BVHGPU_ANY) {
        if (!COUNT) return true;
        continue;
      }
      // Each accepted triangle overwrites the hit (triangle.cpp:243).
      tmax = t;
      best.leaf = leaf;
      best.lane = i;
      best.u = b1;
      best.v = b2;
    }
    return any;
  }
  for (int g = 0; g < cnt; g += 4) {
    float lo[4][3], hi[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float4 mn = ldg4(bnd + a * lm + g), mx = ldg4(bnd + (3 + a) * lm + g);
      const uint64_t o2 = f2splat(r.o[a]), s2 = f2splat(r.inv[a]);
      const float2 n01 = f2unpack(f2mul(f2sub(f2pack(mn.x, mn.y), o2), s2));
      const float2 n23 = f2unpack(f2mul(f2sub(f2pack(mn.z, mn.w), o2), s2));
      const float2 x01 = f2unpack(f2mul(f2sub(f2pack(mx.x, mx.y), o2), s2));
      const float2 x23 = f2unpack(f2mul(f2sub(f2pack(mx.z, mx.w), o2), s2));
      lo[0][a] = n01.x; lo[1][a] = n01.y; lo[2][a] = n23.x; lo[3][a] = n23.y;
      hi[0][a] = x01.x; hi[1][a] = x01.y; hi[2][a] = x23.x; hi[3][a] = x23.y;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int i = g + k;
      if (i >= cnt) break;
      const float tmin = fmaxf(fmaxf(fminf(lo[k][0], hi[k][0]), fminf(lo[k][1], hi[k][1])),
                               fminf(lo[k][2], hi[k][2]));
      const float tmx = fminf(fminf(fmaxf(lo[k][0], hi[k][0]), fmaxf(lo[k][1], hi[k][1])),
                              fmaxf(lo[k][2], hi[k][2]));
      if (tmx < 0 || tmin > tmx || tmax < tmin) continue;
      float p[3][3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        p[v][0] = __ldg(blk + (v * 3 + ax0) * stride + i);
        p[v][1] = __ldg(blk + (v * 3 + ax1) * stride + i);
        p[v][2] = __ldg(blk + (v * 3 + ax2) * stride + i);
      }
      float t, b1, b2;
      if (!watertight<MM, false>(p, r, tmax, t, b1, b2)) continue;
      if (COUNT) ctr.tri_hits++;
      any = true;
      if (KIND == BVHGPU_ANY) {
        if (!COUNT) return true;
        continue;
      }
      // Each accepted triangle overwrites the hit (triangle.cpp:243).
      tmax = t;
      best.leaf = leaf;
      best.lane = i;
      best.u = b1;
      best.v = b2;
    }
  }
  return any;
}

template <int PROFILE, int KIND, bool COUNT, bool MM>
BVHGPU_DEV bool visit_leaf(const SceneDev& sc, uint32_t e, const Ray& r, float& tmax, Best& best,
                           Counters& ctr) {
  if constexpr (BVHGPU_LEAF_BOUNDS && PROFILE == BVHGPU_PROFILE_INSTRUMENTED && MM)
    return visit_leaf_bounds<KIND, COUNT, MM>(sc, e, r, tmax, best, ctr);
  else
    return visit_leaf_points<PROFILE, KIND, COUNT, MM>(sc, e, r, tmax, best, ctr);
}

// Visits with the IEEE min / max forms unless the ray can produce a NaN.
// Node e is read from the block's shared copy of the top levels when e <
// top (top == 0: all nodes from global memory).
template <int N, int PROFILE, int KIND, bool COUNT, int FMT, bool DIST = false>
BVHGPU_DEV bool node_step(const SceneDev& sc, uint32_t e, const uint8_t* top_smem, uint32_t top,
                          const Ray& r, float tmax, uint32_t* stack, int stride, int& sp, int cap,
                          Counters& ctr, int& depth, float* dstack = nullptr) {
  constexpr int REC = NodeFmt<N, FMT>::REC;
  const uint8_t* side =
      FMT == kFmtFP32 ? nullptr : sc.q8_perm + (size_t)e * NodeFmt<N, FMT>::PSB;
  const uint32_t* ent =
      sc.child_entry != nullptr ? sc.child_entry + (size_t)e * NodeFmt<N, FMT>::NM : nullptr;
  if (e < top) {
    const uint8_t* rec = top_smem + (size_t)e * REC;
    if (r.exact)
      return visit_node<N, PROFILE, KIND, COUNT, false, FMT, true, DIST>(
          rec, r, tmax, stack, stride, sp, cap, ctr, depth, dstack, sc.any_index_order != 0, side, ent);
    return visit_node<N, PROFILE, KIND, COUNT, true, FMT, true, DIST>(
        rec, r, tmax, stack, stride, sp, cap, ctr, depth, dstack, sc.any_index_order != 0, side, ent);
  }
  const uint8_t* rec = sc.nodes + (size_t)e * REC;
  if (r.exact)
    return visit_node<N, PROFILE, KIND, COUNT, false, FMT, false, DIST>(
        rec, r, tmax, stack, stride, sp, cap, ctr, depth, dstack, sc.any_index_order != 0, side, ent);
  constexpr bool kNF = BVHGPU_NEARFAR && FMT == kFmtFP32 && !DIST;
  if (kNF && sc.boxes_ordered)
    return visit_node<N, PROFILE, KIND, COUNT, true, FMT, false, DIST, kNF>(
        rec, r, tmax, stack, stride, sp, cap, ctr, depth, dstack, sc.any_index_order != 0, side, ent);
  return visit_node<N, PROFILE, KIND, COUNT, true, FMT, false, DIST>(
      rec, r, tmax, stack, stride, sp, cap, ctr, depth, dstack, sc.any_index_order != 0, side, ent);
}

template <int PROFILE, int KIND, bool COUNT>
BVHGPU_DEV bool leaf_step(const SceneDev& sc, uint32_t e, const Ray& r, float& tmax, Best& best,
                          Counters& ctr) {
  if (r.exact) return visit_leaf<PROFILE, KIND, COUNT, false>(sc, e, r, tmax, best, ctr);
  return visit_leaf<PROFILE, KIND, COUNT, true>(sc, e, r, tmax, best, ctr);
}

BVHGPU_DEV void record_error(int* status, int code) { atomicCAS(status, 0, code); }

// Counting launches: one node visit (depth_count = depth | child count << 8,
// as node_step returns it) into the per-depth histogram and childFullness
// (compactNode.cpp:714-716), one leaf visit into the per-depth histogram and
// primitiveFullness (compactNode.cpp:653-656).
BVHGPU_DEV void count_node(const TraceArgs& a, int depth_count) {
  if (a.depth_hist) atomicAdd(a.depth_hist + min(depth_count & 0xFF, 63), 1ull);
  if (a.fullness) atomicAdd(a.fullness + min(depth_count >> 8, 16), 1ull);
}
BVHGPU_DEV void count_leaf(const SceneDev& sc, const TraceArgs& a, uint32_t e) {
  if (a.depth_hist)
    atomicAdd(a.depth_hist + 64 + min((int)sc.leaf_depth[e & kLeafIndexMask], 63), 1ull);
  if (a.fullness) atomicAdd(a.fullness + 17 + (int)((e >> kLeafCountShift) & 15u) + 1, 1ull);
}

// Rays are 32-byte records read with two 128-bit loads (16-byte aligned buffer).
BVHGPU_DEV bvhgpu_ray_t load_ray(const bvhgpu_ray_t* rays, uint64_t i) {
  const float4* p = reinterpret_cast<const float4*>(rays + i);
  const float4 a = __ldg(p), b = __ldg(p + 1);
  bvhgpu_ray_t r;
  r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tmax = a.w;
  r.dx = b.x; r.dy = b.y; r.dz = b.z; r.pad = b.w;
  return r;
}

template <bool COUNT>
BVHGPU_DEV void flush_counters(const TraceArgs& a, uint64_t rid, const Counters& c) {
  if (!COUNT || a.counters == nullptr) return;
  uint32_t* o = a.counters + out_slot(a, rid) * BVHGPU_COUNTERS_PER_RAY;
  o[0] = c.node_visits;
  o[1] = c.leaf_visits;
  o[2] = c.box_tests;
  o[3] = c.box_hits;
  o[4] = c.tri_tests;
  o[5] = c.tri_hits;
  o[6] = c.max_stack;
  o[7] = 0;
}

template <int KIND>
BVHGPU_DEV void write_result(const SceneDev& sc, const TraceArgs& a, uint64_t rid, bool hit,
                             float tmax, const Best& best) {
  const uint64_t slot = out_slot(a, rid);
  if (KIND == BVHGPU_ANY) {
    a.occluded[slot] = hit ? 1 : 0;
    return;
  }
  bvhgpu_hit_t h;
  if (best.lane >= 0) {
    h.prim = (int32_t)__ldg(sc.leaf_prim + (size_t)best.leaf * sc.leaf_memory + best.lane);
    h.t = tmax;
    h.u = best.u;
    h.v = best.v;
  } else {
    h.prim = -1;
    h.t = tmax;
    h.u = 0.f;
    h.v = 0.f;
  }
  reinterpret_cast<float4*>(a.hits)[slot] =
      make_float4(__int_as_float(h.prim), h.t, h.u, h.v);
}

// ---------------------------------------------------------------------------
// Per-ray depth-first traversal: one thread per ray, the traversal stack in
// shared memory (stack[slot][thread], conflict-free across a warp).
// DIST: intersectSaveDistance (fastNodeManager.h:1232-1326) /
// intersectImmediately(ray, useDistance = true) (compactNode.cpp:623-645):
// every entry also carries its box's entry distance (in a second shared
// array after the stack), the root enters with 0, and a pop whose distance
// exceeds the current tMax is dropped before it is visited or counted.
// LSTACK > 0: the stack is a per-thread array of LSTACK entries in local
// memory (stride 1) instead of shared memory (the stack-placement knob of the
// autotuner); the caller guarantees a_stack_cap <= LSTACK.
template <int N, int PROFILE, int KIND, bool COUNT, int FMT, bool DIST = false, int LSTACK = 0>
__global__ void __launch_bounds__(128) trace_dfs_kernel(SceneDev sc, TraceArgs a) {
  extern __shared__ uint32_t smem[];
  uint32_t lstack[LSTACK > 0 ? LSTACK : 1];
  const int stride = LSTACK > 0 ? 1 : (int)blockDim.x;
  uint32_t* stack = LSTACK > 0 ? lstack : smem + threadIdx.x;
  float* dstack = DIST ? reinterpret_cast<float*>(smem + (size_t)a.stack_cap * stride) + threadIdx.x
                       : nullptr;
  unsigned long long* hist = nullptr;
  const uint64_t rid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (rid >= a.n) return;

  const bvhgpu_ray_t in = load_ray(a.rays, out_slot(a, rid));
  if (isnan(in.ox)) {
    Best none;
    write_result<KIND>(sc, a, rid, false, in.tmax, none);
    Counters c0;
    flush_counters<COUNT>(a, rid, c0);
    return;
  }
  const Ray r = make_ray<PROFILE>(in);
  float tmax = r.tmax;
  Best best;
  Counters ctr;
  bool hit = false;
  int sp = 0;
  stack[0] = sc.root_entry;
  if (DIST) dstack[0] = 0.f;
  sp = 1;
  const int cap = a.stack_cap;
  while (sp > 0) {
    --sp;
    const uint32_t e = stack[sp * stride];
    if (DIST && dstack[sp * stride] > tmax) continue;
    if (e & kLeafBit) {
      if (COUNT) count_leaf(sc, a, e);
      bool h = leaf_step<PROFILE, KIND, COUNT>(sc, e, r, tmax, best, ctr);
      if (h) {
        hit = true;
        if (KIND == BVHGPU_ANY) break;
      }
    } else {
      int depth;
      if (!node_step<N, PROFILE, KIND, COUNT, FMT, DIST>(sc, e, nullptr, 0u, r, tmax, stack,
                                                         stride, sp, cap, ctr, depth, dstack)) {
        record_error(sc.status, kDevErrStackOverflow);
        hit = false;
        best = Best();
        break;
      }
      if (COUNT) count_node(a, depth);
      if (COUNT) ctr.max_stack = max(ctr.max_stack, (uint32_t)sp);
    }
  }
  (void)hist;
  write_result<KIND>(sc, a, rid, hit, tmax, best);
  flush_counters<COUNT>(a, rid, ctr);
}


// ---------------------------------------------------------------------------
// Ray-stream traversal (FastNodeManager::intersectWideAlternative,
// fastNodeManager.h:835-1049, and its instrumented twin compactNode.cpp:357-601).
// One block holds a packet of blockDim.x rays. Each step, the work list holds
// the rays whose stack top is an inner node at the front and the rays whose
// stack top is a leaf at the back; thread t takes list entry t, so after the
// ballot / popc compaction a warp is (but for one boundary warp) all node
// visits or all leaf visits. Ray state, stacks and hits live in shared memory
// because a ray moves between threads from step to step.
struct StreamRay {
  float o[3], d[3], inv[3];
  float tmax;
  float sx, sy, sz;
  uint32_t bits;  // code | reverse << 2 | kx << 3 | ky << 5
};

BVHGPU_DEV void pack_ray(const Ray& r, StreamRay& s) {
  for (int k = 0; k < 3; ++k) { s.o[k] = r.o[k]; s.d[k] = r.d[k]; s.inv[k] = r.inv[k]; }
  s.tmax = r.tmax;
  s.sx = r.sx; s.sy = r.sy; s.sz = r.sz;
  s.bits = (uint32_t)r.code | ((uint32_t)r.reverse << 2) | ((uint32_t)r.kx << 3) |
           ((uint32_t)r.ky << 5) | ((uint32_t)r.exact << 7);
}
BVHGPU_DEV Ray unpack_ray(const StreamRay& s) {
  Ray r;
  for (int k = 0; k < 3; ++k) { r.o[k] = s.o[k]; r.d[k] = s.d[k]; r.inv[k] = s.inv[k]; }
  r.tmax = s.tmax;
  r.sx = s.sx; r.sy = s.sy; r.sz = s.sz;
  r.code = (int)(s.bits & 3u);
  r.reverse = ((s.bits >> 2) & 1u) != 0;
  r.kx = (int)((s.bits >> 3) & 3u);
  r.ky = (int)((s.bits >> 5) & 3u);
  r.exact = ((s.bits >> 7) & 1u) != 0;
  return r;
}

struct StreamShared {
  int node_rays, leaf_rays, next_node, next_leaf;
  int unique_nodes, unique_leaves, terminations, extra_leaf_work;  // step log
};

// Shared-memory bytes of the stream kernel for a packet of p rays (with the
// step log: a hash set of 2p entries for the unique node / leaf counts).
inline size_t stream_smem_bytes(int p, int stack_cap, bool count, bool steps = false) {
  size_t b = sizeof(StreamShared);
  b = (b + 15) / 16 * 16;
  if (steps) b += (size_t)p * 2 * 4;
  b += (size_t)p * sizeof(StreamRay);
  b += (size_t)p * stack_cap * 4;        // stacks
  b += (size_t)p * 4 * 4;                // best: leaf, lane|hit|sp, u, v
  b += (size_t)p * 2 * 2;                // two work lists
  if (count) b += (size_t)p * 8 * 4;     // counters
  return b;
}

// Insert into an open-addressing set in shared memory (linear probing,
// atomicCAS); true if the key was not there yet. At most size / 2 keys go
// into a set, so a free slot is always found within `size` probes.
constexpr uint32_t kSetEmpty = 0x7FFFFFFFu;  // no node index or leaf entry has this value
BVHGPU_DEV bool set_insert(uint32_t* tbl, int size, uint32_t key) {
  uint32_t h = (key * 2654435761u) % (uint32_t)size;
  for (int probe = 0; probe < size; ++probe) {
    const uint32_t old = atomicCAS(tbl + h, kSetEmpty, key);
    if (old == kSetEmpty) return true;
    if (old == key) return false;
    h = (h + 1 == (uint32_t)size) ? 0u : h + 1u;
  }
  return false;
}

// Rays left in a packet below which its threads finish them alone (bench
// frame, stream scheme: 0 24.2 ms, 32 23.6, 64 23.1, 128 21.6).
#ifndef BVHGPU_STREAM_TAIL
#define BVHGPU_STREAM_TAIL 128
#endif
// Packets of up to 256 rays, two per SM (at most 128 registers): with the
// stored-bounds leaf test the compiler otherwise takes 142 registers and
// one packet per SM (bench frame: 42.5 against 27.1 ms).
#ifndef BVHGPU_STREAM_MIN_BLOCKS
#define BVHGPU_STREAM_MIN_BLOCKS 2
#endif
template <int N, int PROFILE, int KIND, bool COUNT>
__global__ void __launch_bounds__(256, BVHGPU_STREAM_MIN_BLOCKS)
    trace_stream_kernel(SceneDev sc, TraceArgs a) {
  extern __shared__ __align__(16) uint8_t smem_raw[];
  const int P = blockDim.x;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  StreamShared* ctl = reinterpret_cast<StreamShared*>(smem_raw);
  uint8_t* base = smem_raw + (sizeof(StreamShared) + 15) / 16 * 16;
  // Step log (workgroup analysis of CameraData, cameraData.h:660-1109): per
  // step the node and leaf work, the unique nodes and leaves among them and
  // the rays that terminate, as intersectWideAlternative collects them
  // (compactNode.cpp:357-601).
  const bool log = COUNT && a.step_stats != nullptr;
  uint32_t* set = nullptr;
  if (log) {
    set = reinterpret_cast<uint32_t*>(base);
    base += (size_t)P * 2 * 4;
  }
  StreamRay* rays = reinterpret_cast<StreamRay*>(base);
  base += (size_t)P * sizeof(StreamRay);
  uint32_t* stacks = reinterpret_cast<uint32_t*>(base);  // stacks[slot * P + ray]
  base += (size_t)P * a.stack_cap * 4;
  uint32_t* best_leaf = reinterpret_cast<uint32_t*>(base);
  int32_t* best_misc = reinterpret_cast<int32_t*>(best_leaf + P);  // lane | sp << 8 | hit << 31
  float* best_u = reinterpret_cast<float*>(best_misc + P);
  float* best_v = best_u + P;
  base += (size_t)P * 16;
  uint16_t* work0 = reinterpret_cast<uint16_t*>(base);  // list c at work0 + c * P
  base += (size_t)P * 4;
  uint32_t* ctrs = reinterpret_cast<uint32_t*>(base);  // [8][P]

  const uint64_t first = (uint64_t)blockIdx.x * P;
  const uint64_t rid = first + tid;
  const int cap = a.stack_cap;

  if (tid == 0) {
    ctl->node_rays = 0; ctl->leaf_rays = 0; ctl->next_node = 0; ctl->next_leaf = 0;
    ctl->unique_nodes = 0; ctl->unique_leaves = 0; ctl->terminations = 0;
    ctl->extra_leaf_work = 0;
  }
  __syncthreads();
  // Set-up: active rays go to the node part of list 0 (the root entry is an
  // inner node unless the whole tree is one leaf).
  bool active = false;
  if (rid < a.n) {
    const bvhgpu_ray_t in = load_ray(a.rays, out_slot(a, rid));
    Ray r = make_ray<PROFILE>(in);
    pack_ray(r, rays[tid]);
    best_leaf[tid] = 0xFFFFFFFFu;
    best_misc[tid] = -1 & 0xFF;
    best_u[tid] = 0.f;
    best_v[tid] = 0.f;
    if (COUNT) for (int k = 0; k < 8; ++k) ctrs[k * P + tid] = 0;
    active = !isnan(in.ox);
    if (active) {
      stacks[tid] = sc.root_entry;
      best_misc[tid] = 0xFF | (1 << 8);  // lane -1, sp 1
    }
  }
  const bool root_leaf = (sc.root_entry & kLeafBit) != 0;
  {
    const unsigned m = __ballot_sync(0xFFFFFFFFu, active);
    int pos = 0;
    if (m) {
      int b = 0;
      if (lane == __ffs(m) - 1) {
        if (root_leaf) b = atomicAdd(&ctl->leaf_rays, __popc(m));
        else b = atomicAdd(&ctl->node_rays, __popc(m));
      }
      b = __shfl_sync(0xFFFFFFFFu, b, __ffs(m) - 1);
      pos = b + __popc(m & ((1u << lane) - 1u));
    }
    if (active) {
      if (root_leaf) work0[P - 1 - pos] = (uint16_t)tid;
      else work0[pos] = (uint16_t)tid;
    }
  }
  __syncthreads();
  // Step 0, the state before the loop: the active rays at the root, the
  // inactive ones terminated (compactNode.cpp:410-415).
  int step = 1;
  if (log && tid == 0 && a.step_cap > 0) {
    const uint32_t wide = (uint32_t)(a.n - first < (uint64_t)P ? a.n - first : (uint64_t)P);
    const uint32_t act = (uint32_t)(ctl->node_rays + ctl->leaf_rays);
    uint32_t* rec = a.step_stats + (size_t)blockIdx.x * a.step_cap * 5;
    rec[0] = root_leaf ? 0u : act;
    rec[1] = root_leaf ? 0u : 1u;
    rec[2] = root_leaf ? act : 0u;
    rec[3] = root_leaf ? (act ? 1u : 0u) : 0u;
    rec[4] = wide - act;
  }

  int cur = 0;
  while (true) {
    const int node_rays = ctl->node_rays, leaf_rays = ctl->leaf_rays;
    if (node_rays == 0 && leaf_rays == 0) break;
    if (log) {
      for (int i = tid; i < 2 * P; i += P) set[i] = kSetEmpty;
      __syncthreads();
    }
    int ray = -1;
    bool is_node = false;
    const uint16_t* wcur = work0 + cur * P;
    if (tid < node_rays) { ray = wcur[tid]; is_node = true; }
    else if (tid >= P - leaf_rays) { ray = wcur[tid]; }
    bool want_node = false, want_leaf = false;
    // The packet's tail: once at most BVHGPU_STREAM_TAIL rays are left (and
    // no step log is kept), each thread finishes its ray alone, step after
    // step without the block's barriers. A ray's visits are the same either
    // way (it pops its own stack), so are its results and counters.
    const bool finish = !log && node_rays + leaf_rays <= BVHGPU_STREAM_TAIL;
    while (ray >= 0) {
      Ray r = unpack_ray(rays[ray]);
      float tmax = r.tmax;
      int32_t misc = best_misc[ray];
      int sp = (misc >> 8) & 0x7FFF;
      bool done = false;
      Counters ctr;
      --sp;
      const uint32_t e = stacks[sp * P + ray];
      if (log && set_insert(set, 2 * P, e))
        atomicAdd(is_node ? &ctl->unique_nodes : &ctl->unique_leaves, 1);
      auto leaf_visit = [&](uint32_t le) {
        if (COUNT) count_leaf(sc, a, le);
        Best best;
        best.leaf = best_leaf[ray];
        best.lane = (int)(int8_t)(misc & 0xFF);
        best.u = best_u[ray];
        best.v = best_v[ray];
        bool h = leaf_step<PROFILE, KIND, COUNT>(sc, le, r, tmax, best, ctr);
        if (h) {
          misc |= (int32_t)0x80000000;
          if (KIND == BVHGPU_ANY) done = true;
          else {
            rays[ray].tmax = tmax;
            best_leaf[ray] = best.leaf;
            misc = (misc & ~0xFF) | (best.lane & 0xFF);
            best_u[ray] = best.u;
            best_v[ray] = best.v;
          }
        }
      };
      if (is_node) {
        int depth;
        if (!node_step<N, PROFILE, KIND, COUNT, kFmtFP32>(sc, e, nullptr, 0u, r, tmax, stacks + ray,
                                                          P, sp, cap, ctr, depth)) {
          record_error(sc.status, kDevErrStackOverflow);
          best_leaf[ray] = 0xFFFFFFFFu;
          misc = 0xFF;
          done = true;
          sp = 0;
        }
        if (COUNT) count_node(a, depth);
        // intersectWide's schedule (compactNode.cpp:118-356, step log only):
        // a ray whose next entry is a leaf visits it in the same step.
        if (log && a.step_wide && !done && sp > 0 && (stacks[(sp - 1) * P + ray] & kLeafBit)) {
          ctrs[6 * P + ray] = max(ctrs[6 * P + ray], (uint32_t)sp);
          --sp;
          const uint32_t le = stacks[sp * P + ray];
          if (set_insert(set, 2 * P, le)) atomicAdd(&ctl->unique_leaves, 1);
          atomicAdd(&ctl->extra_leaf_work, 1);
          leaf_visit(le);
        }
      } else {
        leaf_visit(e);
      }
      if (COUNT) {
        ctrs[0 * P + ray] += ctr.node_visits;
        ctrs[1 * P + ray] += ctr.leaf_visits;
        ctrs[2 * P + ray] += ctr.box_tests;
        ctrs[3 * P + ray] += ctr.box_hits;
        ctrs[4 * P + ray] += ctr.tri_tests;
        ctrs[5 * P + ray] += ctr.tri_hits;
        ctrs[6 * P + ray] = max(ctrs[6 * P + ray], (uint32_t)sp);
      }
      if (!done && sp > 0) {
        const uint32_t top = stacks[(sp - 1) * P + ray];
        if (top & kLeafBit) want_leaf = true;
        else want_node = true;
      }
      if (done) sp = 0;
      if (log && sp == 0) atomicAdd(&ctl->terminations, 1);
      misc = (misc & ~(0x7FFF << 8)) | (sp << 8);
      best_misc[ray] = misc;
      if (!finish || !(want_node || want_leaf)) break;
      is_node = want_node;
      want_node = want_leaf = false;
    }
    if (finish) {
      __syncthreads();  // every ray's state is final before the results
      break;
    }
    // Compact into the next list: inner-node rays from the front, leaf rays
    // from the back.
    const int nxt = cur ^ 1;
    {
      const unsigned mn = __ballot_sync(0xFFFFFFFFu, want_node);
      const unsigned ml = __ballot_sync(0xFFFFFFFFu, want_leaf);
      int bn = 0, bl = 0;
      if (mn && lane == __ffs(mn) - 1) bn = atomicAdd(&ctl->next_node, __popc(mn));
      if (ml && lane == __ffs(ml) - 1) bl = atomicAdd(&ctl->next_leaf, __popc(ml));
      if (mn) bn = __shfl_sync(0xFFFFFFFFu, bn, __ffs(mn) - 1);
      if (ml) bl = __shfl_sync(0xFFFFFFFFu, bl, __ffs(ml) - 1);
      const unsigned below = (1u << lane) - 1u;
      uint16_t* wnxt = work0 + nxt * P;
      if (want_node) wnxt[bn + __popc(mn & below)] = (uint16_t)ray;
      if (want_leaf) wnxt[P - 1 - (bl + __popc(ml & below))] = (uint16_t)ray;
    }
    __syncthreads();
    if (tid == 0) {
      if (log && step < a.step_cap) {
        uint32_t* rec = a.step_stats + ((size_t)blockIdx.x * a.step_cap + step) * 5;
        rec[0] = (uint32_t)node_rays;
        rec[1] = (uint32_t)ctl->unique_nodes;
        rec[2] = (uint32_t)(leaf_rays + ctl->extra_leaf_work);
        rec[3] = (uint32_t)ctl->unique_leaves;
        rec[4] = (uint32_t)ctl->terminations;
      }
      ctl->unique_nodes = 0;
      ctl->unique_leaves = 0;
      ctl->terminations = 0;
      ctl->extra_leaf_work = 0;
      ctl->node_rays = ctl->next_node;
      ctl->leaf_rays = ctl->next_leaf;
      ctl->next_node = 0;
      ctl->next_leaf = 0;
    }
    ++step;
    cur = nxt;
    __syncthreads();
  }
  if (log && tid == 0) a.step_count[blockIdx.x] = (uint32_t)step;

  // Results of this thread's own ray slot.
  if (rid < a.n) {
    const int32_t misc = best_misc[tid];
    const bool hit = (misc & (int32_t)0x80000000) != 0;
    Best best;
    best.leaf = best_leaf[tid];
    best.lane = (int)(int8_t)(misc & 0xFF);
    best.u = best_u[tid];
    best.v = best_v[tid];
    write_result<KIND>(sc, a, rid, hit, rays[tid].tmax, best);
    if (COUNT && a.counters) {
      uint32_t* o = a.counters + out_slot(a, rid) * BVHGPU_COUNTERS_PER_RAY;
      for (int k = 0; k < 7; ++k) o[k] = ctrs[k * P + tid];
      o[7] = 0;
    }
  }
}


// ---------------------------------------------------------------------------
// Persistent depth-first traversal. A grid sized to fill the GPU once loops
// until a global ray queue is drained; each warp refills its finished lanes
// with the next rays (one atomicAdd per refill) so warps stay full on
// incoherent rays, the GPU form of the reference's refill structure
// (RefillStructure, fastNodeManager.h:92-156, 277-450). Lanes keep the
// per-ray depth-first order, so every ray's visits and results are those of
// the plain kernel; only the interleaving between lanes changes.
//
// POLICY 0 ("while-while"): each round, lanes whose stack top is an inner node
// visit nodes until every active lane has a leaf on top, then all of them
// visit their leaf together. POLICY 1 ("if-if"): one node or leaf visit per
// lane per round. POLICY 2: while-while with leaves set aside (speculative
// traversal) for any-hit rays without counters.
struct QueueArgs {
  unsigned long long* head;  // next unclaimed ray (zeroed before the launch)
  int refill_min;            // refill when at least this many lanes are idle
  uint32_t top_nodes;        // inner records staged in shared memory (0: none)
  uint32_t stall_bytes;      // failure-detection tests: bytes the staging wait expects extra
};

#ifndef BVHGPU_PERSIST_MIN_BLOCKS
#define BVHGPU_PERSIST_MIN_BLOCKS 6
#endif

// POLICY 4: the ray constants a leaf test needs, one 48-byte record per
// thread in shared memory (written when the lane takes the ray), so that any
// lane of the warp can test a triangle for any other lane's ray.
// Instrumented profile: origin, tMax | 1 / direction, shear x | shear y, z,
// axes (kx | ky << 2 | kz << 4 | exact << 6). Fast profile: origin, tMax |
// direction, 0 | 0, 0, exact << 6.
constexpr int kRayRecWords = 12;
// POLICIES 3 and 4: leaves a lane may set aside per round (1 or 2).
#ifndef BVHGPU_SPEC_LEAVES
#define BVHGPU_SPEC_LEAVES 2
#endif

template <int PROFILE>
BVHGPU_DEV void store_ray_rec(float4* rec, const Ray& r) {
  const int packed = r.kx | (r.ky << 2) | (r.code << 4) | ((r.exact ? 1 : 0) << 6);
  if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) {
    rec[0] = make_float4(r.o[0], r.o[1], r.o[2], r.tmax);
    rec[1] = make_float4(r.inv[0], r.inv[1], r.inv[2], r.sx);
    rec[2] = make_float4(r.sy, r.sz, __int_as_float(packed), 0.f);
  } else {
    rec[0] = make_float4(r.o[0], r.o[1], r.o[2], r.tmax);
    rec[1] = make_float4(r.d[0], r.d[1], r.d[2], 0.f);
    rec[2] = make_float4(0.f, 0.f, __int_as_float(packed), 0.f);
  }
}

// The fields of a Ray that the leaf tests read, from its shared record.
template <int PROFILE>
BVHGPU_DEV Ray load_ray_rec(const float4* rec) {
  Ray r;
  const float4 a = rec[0], b = rec[1], c = rec[2];
  const int packed = __float_as_int(c.z);
  r.o[0] = a.x; r.o[1] = a.y; r.o[2] = a.z;
  r.tmax = a.w;
  if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) {
    r.inv[0] = b.x; r.inv[1] = b.y; r.inv[2] = b.z;
    r.sx = b.w; r.sy = c.x; r.sz = c.y;
  } else {
    r.d[0] = b.x; r.d[1] = b.y; r.d[2] = b.z;
  }
  r.kx = packed & 3;
  r.ky = (packed >> 2) & 3;
  r.code = (packed >> 4) & 3;
  r.exact = (packed >> 6) & 1;
  return r;
}

// POLICY 4 leaf phase: the leaves the warp's lanes set aside (e0 / e1, with
// c0 / c1 triangles; 0 triangles where a slot is empty) form one pool of
// (ray, triangle) pairs, and the 32 lanes test 32 pairs at a time: pair p
// belongs to the lane j with off_j <= p < off_j + c0_j + c1_j (a warp prefix
// sum), and a lane testing it reads ray j's record from shared memory. A
// lane's result is the OR over its pairs, as testing its leaves one after
// the other would give (any-hit, tMax fixed). Every lane of the warp calls it.
template <int PROFILE>
BVHGPU_DEV bool coop_leaf_phase(const SceneDev& sc, const float4* warp_recs, uint32_t e0,
                                uint32_t e1, int c0, int c1, unsigned lane) {
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const int c = c0 + c1;
  int incl = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(FULL, incl, d);
    if ((int)lane >= d) incl += v;
  }
  const int total = __shfl_sync(FULL, incl, 31);
  const int off = incl - c;
  bool mine = false;
  for (int base = 0; base < total; base += 32) {
    const int p = base + (int)lane;
    // Owner: the largest lane j with off_j <= p (lanes without pairs share
    // the next lane's offset, so the largest such j has pairs when p < total).
    int j = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
      const int v = __shfl_sync(FULL, off, j + step);
      if (v <= p) j += step;
    }
    const int off_j = __shfl_sync(FULL, off, j);
    const uint32_t e0_j = __shfl_sync(FULL, e0, j), e1_j = __shfl_sync(FULL, e1, j);
    const int c0_j = __shfl_sync(FULL, c0, j);
    bool h = false;
    if (p < total) {
      const int q = p - off_j;
      const uint32_t e = q < c0_j ? e0_j : e1_j;
      const int i = q < c0_j ? q : q - c0_j;
      const int cnt = (int)((e >> kLeafCountShift) & 15u) + 1;
      const int stride = ((cnt - 1) / sc.gang + 1) * sc.gang;
      const float* blk = sc.leaves + (size_t)(e & kLeafIndexMask) * 9 * sc.leaf_memory;
      const Ray r = load_ray_rec<PROFILE>(warp_recs + (size_t)j * 3);
      int ax0 = 0, ax1 = 1, ax2 = 2;
      if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) { ax0 = r.kx; ax1 = r.ky; ax2 = r.code; }
      float pt[3][3];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        pt[v][0] = __ldg(blk + (v * 3 + ax0) * stride + i);
        pt[v][1] = __ldg(blk + (v * 3 + ax1) * stride + i);
        pt[v][2] = __ldg(blk + (v * 3 + ax2) * stride + i);
      }
      float t, b1, b2;
      if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED)
        h = r.exact ? watertight<false>(pt, r, r.tmax, t, b1, b2)
                    : watertight<true>(pt, r, r.tmax, t, b1, b2);
      else
        h = moller_trumbore(pt, r, r.tmax, t, b1, b2);
    }
    const unsigned hits = __ballot_sync(FULL, h);
    // This lane's pairs in the window [base, base + 32).
    const int lo = min(max(off - base, 0), 32), hi = min(max(off + c - base, 0), 32);
    if (hi > lo) {
      const unsigned upto = hi == 32 ? FULL : ((1u << hi) - 1u);
      const unsigned from = lo == 32 ? 0u : ~((1u << lo) - 1u);
      if (hits & upto & from) mine = true;
    }
  }
  return mine;
}
template <int N, int PROFILE, int KIND, bool COUNT, int POLICY, int FMT>
__global__ void __launch_bounds__(128, BVHGPU_PERSIST_MIN_BLOCKS)
    trace_persistent_kernel(SceneDev sc, TraceArgs a, QueueArgs q) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint64_t top_bar;
  const int stride = blockDim.x;
  uint32_t* stack = smem + threadIdx.x;
  // The first q.top_nodes inner records (the top levels, laid out first) are
  // copied into shared memory once per block with one bulk (TMA) copy.
  uint8_t* top_smem = reinterpret_cast<uint8_t*>(smem + (size_t)a.stack_cap * stride);
  const uint32_t top = q.top_nodes;
  if (top > 0) {
    const uint32_t bytes = top * (uint32_t)NodeFmt<N, FMT>::REC;
    if (threadIdx.x == 0) mbar_init(&top_bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      // q.stall_bytes (failure-detection tests only) makes the barrier wait
      // for bytes no copy delivers, so the bounded wait below runs out.
      mbar_arrive_expect_tx(&top_bar, bytes + q.stall_bytes);
      for (uint32_t off = 0; off < bytes; off += 32768u)
        bulk_copy_g2s(top_smem + off, sc.nodes + off, min(32768u, bytes - off), &top_bar);
    }
    if (!mbar_wait(&top_bar, 0, 500000000ull)) {  // 0.5 s
      record_error(sc.status, kDevErrTimeout);
      mbar_wait(&top_bar, 0, 500000000ull);  // let a late copy land before the block exits
      return;
    }
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  const int cap = a.stack_cap;
  constexpr unsigned FULL = 0xFFFFFFFFu;
  // POLICY 4: per-thread ray records after the top levels (16-byte aligned).
  float4* ray_recs = reinterpret_cast<float4*>(
      top_smem + (((size_t)top * NodeFmt<N, FMT>::REC + 15) / 16) * 16);
  float4* my_rec = ray_recs + (size_t)threadIdx.x * 3;
  const float4* warp_recs = ray_recs + (size_t)(threadIdx.x & ~31u) * 3;
  uint32_t post1 = 0xFFFFFFFFu;  // POLICIES 3, 4: second leaf set aside
  (void)my_rec;
  (void)warp_recs;

  Ray r;
  float tmax = 0.f;
  Best best;
  Counters ctr;
  bool active = false, hit = false;
  int sp = 0;
  uint64_t rid = 0;
  bool drained = false;
  uint32_t postponed = 0xFFFFFFFFu;  // POLICY 2: leaf set aside

  while (true) {
    const unsigned idle = __ballot_sync(FULL, !active);
    if (!drained && idle != 0 && ((int)__popc(idle) >= q.refill_min || idle == FULL)) {
      const int leader = __ffs(idle) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(q.head, (unsigned long long)__popc(idle));
      base = __shfl_sync(FULL, base, leader);
      if (base + __popc(idle) >= a.n) drained = true;
      if (!active) {
        const uint64_t my = base + __popc(idle & below);
        if (my < a.n) {
          rid = my;
          const bvhgpu_ray_t in = load_ray(a.rays, out_slot(a, rid));
          if (isnan(in.ox)) {
            Best none;
            write_result<KIND>(sc, a, rid, false, in.tmax, none);
            Counters c0;
            flush_counters<COUNT>(a, rid, c0);
          } else {
            r = make_ray<PROFILE>(in);
            tmax = r.tmax;
            best = Best();
            ctr = Counters();
            hit = false;
            stack[0] = sc.root_entry;
            sp = 1;
            active = true;
            if (POLICY == 4) store_ray_rec<PROFILE>(my_rec, r);
          }
        }
      }
    }
    if (__ballot_sync(FULL, active) == 0) {
      if (drained) break;
      continue;
    }

    if (POLICY == 3 || POLICY == 4) {
      // Any-hit rays without counters, speculative with two leaves per lane:
      // a lane sets aside the leaves it reaches (up to two) and keeps
      // visiting nodes while another lane still has no leaf. Then each lane
      // tests its set-aside leaves in turn (POLICY 3; the second only if the
      // first has no hit), or the warp tests all of them together, 32 (ray,
      // triangle) pairs at a time (POLICY 4, coop_leaf_phase). A ray whose
      // leaves hit is done; the others go on. Whether an any-hit ray is
      // occluded does not depend on the order in which its reachable leaves
      // are tested (tMax does not change), so results equal the depth-first
      // order's; a leaf that the depth-first order would have skipped after
      // an earlier hit costs work but changes no result.
      constexpr bool kTwo = BVHGPU_SPEC_LEAVES >= 2;
      while (true) {
        while (active && sp > 0 && (kTwo ? post1 : postponed) == 0xFFFFFFFFu &&
               (stack[(sp - 1) * stride] & kLeafBit) != 0u) {
          --sp;
          const uint32_t le = stack[sp * stride];
          if (postponed == 0xFFFFFFFFu) postponed = le;
          else post1 = le;
        }
        const bool want = active && sp > 0 && (kTwo ? post1 : postponed) == 0xFFFFFFFFu &&
                          (stack[(sp - 1) * stride] & kLeafBit) == 0u;
        const unsigned holding =
            __ballot_sync(FULL, !active || postponed != 0xFFFFFFFFu || sp == 0);
        if (__ballot_sync(FULL, want) == 0 || holding == FULL) break;
        if (want) {
          --sp;
          const uint32_t e = stack[sp * stride];
          int depth;
          if (!node_step<N, PROFILE, KIND, COUNT, FMT>(sc, e, top_smem, top, r, tmax, stack,
                                                       stride, sp, cap, ctr, depth)) {
            record_error(sc.status, kDevErrStackOverflow);
            hit = false;
            sp = 0;
            postponed = post1 = 0xFFFFFFFFu;
          }
        }
      }
      const bool holds = active && postponed != 0xFFFFFFFFu;
      if (POLICY == 3) {
        if (holds) {
          bool h = leaf_step<PROFILE, KIND, COUNT>(sc, postponed, r, tmax, best, ctr);
          if (!h && post1 != 0xFFFFFFFFu)
            h = leaf_step<PROFILE, KIND, COUNT>(sc, post1, r, tmax, best, ctr);
          if (h) {
            hit = true;
            sp = 0;
          }
        }
        postponed = post1 = 0xFFFFFFFFu;
      } else if (__ballot_sync(FULL, holds) != 0) {
        const uint32_t e0 = holds ? postponed : 0u;
        const uint32_t e1 = (holds && post1 != 0xFFFFFFFFu) ? post1 : 0u;
        const int c0 = holds ? (int)((e0 >> kLeafCountShift) & 15u) + 1 : 0;
        const int c1 = (holds && post1 != 0xFFFFFFFFu) ? (int)((e1 >> kLeafCountShift) & 15u) + 1 : 0;
        __syncwarp();  // the lanes' ray records are visible to the whole warp
        if (coop_leaf_phase<PROFILE>(sc, warp_recs, e0, e1, c0, c1, lane) && holds) {
          hit = true;
          sp = 0;
        }
        postponed = post1 = 0xFFFFFFFFu;
      }
    } else if (POLICY == 2) {
      // Any-hit rays without counters: a lane that reaches a leaf sets it
      // aside and keeps visiting nodes until every lane holds a leaf (or has
      // no node left); then all lanes test their leaf together. Whether an
      // any-hit ray is occluded does not depend on the order in which its
      // reachable leaves are tested (tMax does not change), so results equal
      // the depth-first order's.
      while (true) {
        if (active && sp > 0 && postponed == 0xFFFFFFFFu &&
            (stack[(sp - 1) * stride] & kLeafBit) != 0u) {
          --sp;
          postponed = stack[sp * stride];
        }
        const bool want =
            active && sp > 0 && (stack[(sp - 1) * stride] & kLeafBit) == 0u;
        const unsigned holding = __ballot_sync(FULL, !active || postponed != 0xFFFFFFFFu);
        if (__ballot_sync(FULL, want) == 0 || holding == FULL) break;
        if (want) {
          --sp;
          const uint32_t e = stack[sp * stride];
          int depth;
          if (!node_step<N, PROFILE, KIND, COUNT, FMT>(sc, e, top_smem, top, r, tmax, stack,
                                                       stride, sp, cap, ctr, depth)) {
            record_error(sc.status, kDevErrStackOverflow);
            hit = false;
            sp = 0;
            postponed = 0xFFFFFFFFu;
          }
        }
      }
      if (active && postponed != 0xFFFFFFFFu) {
        if (leaf_step<PROFILE, KIND, COUNT>(sc, postponed, r, tmax, best, ctr)) {
          hit = true;
          sp = 0;
        }
        postponed = 0xFFFFFFFFu;
      }
    } else if (POLICY == 0) {
      // Node visits until every active lane has a leaf on top (or is done).
      while (true) {
        const bool want =
            active && sp > 0 && (stack[(sp - 1) * stride] & kLeafBit) == 0u;
        if (__ballot_sync(FULL, want) == 0) break;
        if (want) {
          --sp;
          const uint32_t e = stack[sp * stride];
          int depth;
          if (!node_step<N, PROFILE, KIND, COUNT, FMT>(sc, e, top_smem, top, r, tmax, stack,
                                                       stride, sp, cap, ctr, depth)) {
            record_error(sc.status, kDevErrStackOverflow);
            hit = false;
            best = Best();
            sp = 0;
          }
          if (COUNT) count_node(a, depth);
          if (COUNT) ctr.max_stack = max(ctr.max_stack, (uint32_t)sp);
        }
      }
      if (active && sp > 0) {
        --sp;
        const uint32_t e = stack[sp * stride];
        if (COUNT) count_leaf(sc, a, e);
        if (leaf_step<PROFILE, KIND, COUNT>(sc, e, r, tmax, best, ctr)) {
          hit = true;
          if (KIND == BVHGPU_ANY) sp = 0;
        }
      }
    } else {
      if (active && sp > 0) {
        --sp;
        const uint32_t e = stack[sp * stride];
        if (e & kLeafBit) {
          if (COUNT) count_leaf(sc, a, e);
          if (leaf_step<PROFILE, KIND, COUNT>(sc, e, r, tmax, best, ctr)) {
            hit = true;
            if (KIND == BVHGPU_ANY) sp = 0;
          }
        } else {
          int depth;
          if (!node_step<N, PROFILE, KIND, COUNT, FMT>(sc, e, top_smem, top, r, tmax, stack,
                                                       stride, sp, cap, ctr, depth)) {
            record_error(sc.status, kDevErrStackOverflow);
            hit = false;
            best = Best();
            sp = 0;
          }
          if (COUNT) count_node(a, depth);
          if (COUNT) ctr.max_stack = max(ctr.max_stack, (uint32_t)sp);
        }
      }
    }
    if (active && sp == 0 && postponed == 0xFFFFFFFFu) {
      write_result<KIND>(sc, a, rid, hit, tmax, best);
      flush_counters<COUNT>(a, rid, ctr);
      active = false;
    }
  }
}

}  // namespace dev
}  // namespace bvhgpu
