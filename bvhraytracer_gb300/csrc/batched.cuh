// Batched persistent traversal: one launch over many scenes of uneven size and
// uneven ray counts. The jobs (scene + ray batch + kind + outputs) travel in the
// kernel's parameter block; a global queue hands out rays of the concatenated
// job list, warps refill finished lanes, and every lane traverses its own ray
// in its own scene (node width, node format and ray kind are per lane). Per ray
// the visits and results are those of the per-scene kernels.
#pragma once
#include "traverse.cuh"

namespace bvhgpu {
namespace dev {

constexpr int kMaxJobs = 192;  // 192 jobs x 104 bytes in the parameter block

struct JobDev {
  const uint8_t* nodes;
  const float* leaves;
  const uint32_t* leaf_prim;
  const bvhgpu_ray_t* rays;
  void* out;               // hits (closest) or occluded (any)
  int* status;
  uint64_t ray_begin;      // index of the job's first ray in the concatenation
  uint32_t n;
  uint32_t root_entry;
  int32_t leaf_memory;
  int16_t gang;
  int8_t nm;               // node slots: 4, 8, 12 or 16
  int8_t fmt;              // node format
  int8_t kind;             // BVHGPU_CLOSEST / BVHGPU_ANY
  int8_t boxes_ordered;    // SceneDev::boxes_ordered of the job's scene
  int8_t any_index_order;  // SceneDev::any_index_order for the job's rays
  int8_t pad[5];
  // Reordered job: the job's i-th ray in queue order is ray perm[i], and its
  // result goes to slot perm[i] (null: i).
  const uint32_t* perm;
  const uint8_t* q8_perm;  // SceneDev::q8_perm of the job's scene
  const float* leaf_bounds;  // SceneDev::leaf_bounds of the job's scene
};
static_assert(sizeof(JobDev) == 104, "job record size");

struct JobTable {
  JobDev jobs[kMaxJobs];
  int n_jobs;
  uint64_t total;
  unsigned long long* head;
  int refill_min;
  int stack_cap;
  int policy;  // 0 while-while, 2 speculative any-hit
  // KMODE 3: rays [0, split) belong to closest-hit jobs, [split, total) to
  // any-hit jobs (the jobs are ordered so); the any-hit rays have their own
  // queue head.
  uint64_t split;
  unsigned long long* head_any;
};

// Node visit dispatched on the lane's node width and format.
template <int PROFILE, int KIND>
BVHGPU_DEV bool batched_node_step(const SceneDev& sc, int nm, int fmt, uint32_t e, const Ray& r,
                                  float tmax, uint32_t* stack, int stride, int& sp, int cap) {
  Counters ctr;
  int depth;
  if (fmt == kFmtFP32) {
    switch (nm) {
      case 4: return node_step<4, PROFILE, KIND, false, kFmtFP32>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
      case 8: return node_step<8, PROFILE, KIND, false, kFmtFP32>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
      case 12: return node_step<12, PROFILE, KIND, false, kFmtFP32>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
      default: return node_step<16, PROFILE, KIND, false, kFmtFP32>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
    }
  }
  switch (nm) {
    case 4: return node_step<4, PROFILE, KIND, false, kFmtQ8>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
    case 8: return node_step<8, PROFILE, KIND, false, kFmtQ8>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
    case 12: return node_step<12, PROFILE, KIND, false, kFmtQ8>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
    default: return node_step<16, PROFILE, KIND, false, kFmtQ8>(sc, e, nullptr, 0u, r, tmax, stack, stride, sp, cap, ctr, depth);
  }
}

// Five blocks per SM (up to 102 registers per thread): the kernel carries
// every node width, format and ray kind, and at six blocks (80 registers)
// it spills more (batch of 64 scenes, one launch per ray kind: 7.23 ms at
// six blocks, 6.11 at five, 6.87 at four).
#ifndef BVHGPU_BATCHED_MIN_BLOCKS
#define BVHGPU_BATCHED_MIN_BLOCKS 5
#endif
// The persistent loop over the job list. KMODE 0: every lane takes its job's
// ray kind; 1: closest-hit jobs only; 2: any-hit jobs only (the other kind's
// code is compiled out). KSEG 0: every job's rays from t.head; 1: the
// closest-hit segment [0, t.split) from t.head; 2: the any-hit segment
// [t.split, t.total) from t.head_any (the jobs are ordered closest-hit first).
template <int PROFILE, int KMODE, int KSEG = 0>
__device__ __forceinline__ void batched_loop(const JobTable& t) {
  extern __shared__ __align__(16) uint32_t smem[];
  const int stride = blockDim.x;
  uint32_t* stack = smem + threadIdx.x;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  const int cap = t.stack_cap;
  constexpr unsigned FULL = 0xFFFFFFFFu;
  constexpr uint32_t NONE = 0xFFFFFFFFu;

  Ray r;
  float tmax = 0.f;
  Best best;
  bool active = false, hit = false;
  int sp = 0;
  uint32_t local = 0;  // ray index inside the job
  int job = 0;
  SceneDev sc;
  sc.leaf_depth = nullptr;
  sc.top_nodes = 0;
  int nm = 8, fmt = 0;
  int kind = KMODE == 2 ? BVHGPU_ANY : BVHGPU_CLOSEST;
  bool drained = KSEG != 0 && (KSEG == 1 ? t.split == 0 : t.split >= t.total);
  uint32_t postponed = NONE;

  while (true) {
    const unsigned idle = __ballot_sync(FULL, !active);
    // The segment's bounds and queue head, read from the parameter bank
    // where used rather than held in registers.
    const uint64_t seg_begin = KSEG == 2 ? t.split : 0;
    const uint64_t seg_end = KSEG == 1 ? t.split : t.total;
    if (!drained && idle != 0 && ((int)__popc(idle) >= t.refill_min || idle == FULL)) {
      const int leader = __ffs(idle) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(KSEG == 2 ? t.head_any : t.head, (unsigned long long)__popc(idle));
      base = __shfl_sync(FULL, base, leader);
      if (seg_begin + base + __popc(idle) >= seg_end) drained = true;
      if (!active) {
        const uint64_t g = seg_begin + base + __popc(idle & below);
        if (g < seg_end) {
          // Job of global ray g: last job whose ray_begin <= g.
          int lo = 0, hi = t.n_jobs - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (t.jobs[mid].ray_begin <= g) lo = mid;
            else hi = mid - 1;
          }
          job = lo;
          const JobDev& J = t.jobs[job];
          local = (uint32_t)(g - J.ray_begin);
          if (J.perm) local = __ldg(J.perm + local);
          sc.nodes = J.nodes;
          sc.leaves = J.leaves;
          sc.leaf_prim = J.leaf_prim;
          sc.root_entry = J.root_entry;
          sc.leaf_memory = J.leaf_memory;
          sc.gang = J.gang;
          sc.status = J.status;
          sc.boxes_ordered = J.boxes_ordered;
          sc.any_index_order = J.any_index_order;
          sc.q8_perm = J.q8_perm;
          sc.leaf_bounds = J.leaf_bounds;
          nm = J.nm;
          fmt = J.fmt;
          if (KMODE == 0) kind = J.kind;
          const bvhgpu_ray_t in = load_ray(J.rays, local);
          best = Best();
          hit = false;
          postponed = NONE;
          if (isnan(in.ox)) {
            tmax = in.tmax;
            sp = 0;
            active = true;  // retires below with a miss
          } else {
            r = make_ray<PROFILE>(in);
            tmax = r.tmax;
            stack[0] = sc.root_entry;
            sp = 1;
            active = true;
          }
        }
      }
    }
    if (__ballot_sync(FULL, active) == 0) {
      if (drained) break;
      continue;
    }

    const bool spec = t.policy == 2 && kind == BVHGPU_ANY;
    // Node visits until every lane is ready for a leaf (or done).
    while (true) {
      if (spec && active && sp > 0 && postponed == NONE &&
          (stack[(sp - 1) * stride] & kLeafBit) != 0u) {
        --sp;
        postponed = stack[sp * stride];
      }
      const bool want = active && sp > 0 && (stack[(sp - 1) * stride] & kLeafBit) == 0u;
      const bool ready = !active || !want || (spec && postponed != NONE);
      if (__ballot_sync(FULL, want) == 0 || __ballot_sync(FULL, ready) == FULL) break;
      if (want) {
        --sp;
        const uint32_t e = stack[sp * stride];
        const bool ok = kind == BVHGPU_ANY
            ? batched_node_step<PROFILE, BVHGPU_ANY>(sc, nm, fmt, e, r, tmax, stack, stride, sp, cap)
            : batched_node_step<PROFILE, BVHGPU_CLOSEST>(sc, nm, fmt, e, r, tmax, stack, stride, sp, cap);
        if (!ok) {
          record_error(sc.status, kDevErrStackOverflow);
          hit = false;
          best = Best();
          sp = 0;
          postponed = NONE;
        }
      }
    }
    // Leaf visit: the set-aside leaf, or the leaf on top of the stack.
    if (active) {
      uint32_t e = NONE;
      if (postponed != NONE) {
        e = postponed;
        postponed = NONE;
      } else if (sp > 0) {
        --sp;
        e = stack[sp * stride];
      }
      if (e != NONE) {
        Counters ctr;
        if (kind == BVHGPU_ANY) {
          if (leaf_step<PROFILE, BVHGPU_ANY, false>(sc, e, r, tmax, best, ctr)) {
            hit = true;
            sp = 0;
          }
        } else if (leaf_step<PROFILE, BVHGPU_CLOSEST, false>(sc, e, r, tmax, best, ctr)) {
          hit = true;
        }
      }
    }
    if (active && sp == 0 && postponed == NONE) {
      const JobDev& J = t.jobs[job];
      if (kind == BVHGPU_ANY) {
        static_cast<uint8_t*>(J.out)[local] = hit ? 1 : 0;
      } else {
        float4 h;
        if (best.lane >= 0) {
          h = make_float4(__int_as_float((int32_t)__ldg(sc.leaf_prim + (size_t)best.leaf *
                                                                    sc.leaf_memory + best.lane)),
                          tmax, best.u, best.v);
        } else {
          h = make_float4(__int_as_float(-1), tmax, 0.f, 0.f);
        }
        static_cast<float4*>(J.out)[local] = h;
      }
      active = false;
    }
  }
}

// KMODE 0 to 2: one batched_loop over every job's rays. KMODE 3: both kinds
// in one launch with kind-uniform warps: each warp runs the closest-hit loop
// until the closest-hit queue is empty and its lanes are done, then the
// any-hit loop over the any-hit queue (each loop compiled for its kind).
template <int PROFILE, int KMODE>
__global__ void __launch_bounds__(128, BVHGPU_BATCHED_MIN_BLOCKS)
    trace_batched_kernel(const __grid_constant__ JobTable t) {
  if (KMODE == 3) {
    batched_loop<PROFILE, 1, 1>(t);
    batched_loop<PROFILE, 2, 2>(t);
  } else {
    batched_loop<PROFILE, KMODE>(t);
  }
}

}  // namespace dev
}  // namespace bvhgpu
