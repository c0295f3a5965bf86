// C ABI (include/bvhgpu.h): host BVH build and export, device scene
// management and trace launches.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>
#include <algorithm>
#include <atomic>

#include "bvh_builder.hpp"
#include "bvh_export.hpp"
#include "bvhgpu.h"
#include "bvhgpu_status.hpp"
#include "launch.cuh"
#include "reorder.cuh"
#include "raygen.cuh"
#include "q8_encode.cuh"
#include "batched.cuh"
#include "adjoint.cuh"

// Streams (and staging regions) of the host-buffer pipeline: a chunk's copy
// in waits until the chunk this many places earlier has been traced and
// copied out. 1M-triangle frame, median step: 2 streams 8.63 ms, 3 streams
// 8.38 ms, 4 streams 8.39 ms.
#ifndef BVHGPU_HOST_STREAMS
#define BVHGPU_HOST_STREAMS 3
#endif

namespace bvhgpu {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg) {
  if (code != BVHGPU_OK) g_last_error = msg;
  return code;
}

static int cuda_error(cudaError_t e, const char* what) {
  return set_error(BVHGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace bvhgpu

using namespace bvhgpu;

struct bvhgpu_bvh {
  Bvh bvh;
  uint64_t n_input = 0;
};

// Device copy of a flat BVH plus the buffers its launches reuse.
struct bvhgpu_scene {
  int device = 0;
  DeviceLayout layout;  // host copy of the uploaded arrays (sizes and ids)
  int max_stack = 0;
  int stack_limit = 0;  // 0: max_stack; else traversal stack entries per ray
  uint32_t stall_bytes = 0;  // failure-detection tests: staging wait never completes
  std::vector<uint32_t> prim_slot;  // input triangle id -> leaf * leaf_memory + lane
  uint8_t* d_nodes = nullptr;
  uint8_t* d_q8_perm = nullptr;  // Q8 scenes: push sequences, q8_perm_bytes per inner node
  float* d_leaves = nullptr;
  uint32_t* d_leaf_prim = nullptr;
  uint8_t* d_leaf_depth = nullptr;
  uint32_t* d_child_entry = nullptr;
  float* d_leaf_bounds = nullptr;
  int* d_status = nullptr;
  uint32_t* d_prim_slot = nullptr;  // uploaded on first FP64 check
  // Queue heads of the persistent scheme: one slot per launch, round robin,
  // so up to kQueueSlots launches may be in flight on different streams.
  static constexpr int kQueueSlots = 64;
  unsigned long long* d_queue = nullptr;
  std::atomic<unsigned> queue_next{0};
  int sm_count = 0;
  // Staging for bvhgpu_trace_host (grown on demand): one region per
  // pipeline stream, and the streams / events that order them.
  static constexpr int kHostStreams = BVHGPU_HOST_STREAMS;
  std::mutex staging_mu;
  void* d_stage = nullptr;
  size_t stage_bytes = 0;
  cudaStream_t host_stream[kHostStreams] = {};
  cudaEvent_t host_event[kHostStreams + 1] = {};

  dev::SceneDev dev_view() const {
    dev::SceneDev s;
    s.nodes = d_nodes;
    s.leaves = d_leaves;
    s.leaf_prim = d_leaf_prim;
    s.leaf_depth = d_leaf_depth;
    s.root_entry = layout.root_entry;
    s.top_nodes = layout.top_nodes;
    s.leaf_memory = layout.leaf_memory;
    s.gang = layout.gang;
    s.status = d_status;
    s.boxes_ordered = layout.boxes_ordered ? 1 : 0;
    s.q8_perm = d_q8_perm;
    s.child_entry = d_child_entry;
    s.leaf_bounds = d_leaf_bounds;
    return s;
  }
  void release() {
    cudaFree(d_nodes);
    cudaFree(d_q8_perm);
    cudaFree(d_leaves);
    cudaFree(d_leaf_prim);
    cudaFree(d_leaf_depth);
    cudaFree(d_child_entry);
    cudaFree(d_leaf_bounds);
    cudaFree(d_status);
    cudaFree(d_queue);
    cudaFree(d_prim_slot);
    cudaFree(d_stage);
    for (auto& h : host_stream)
      if (h) cudaStreamDestroy(h);
    for (auto& ev : host_event)
      if (ev) cudaEventDestroy(ev);
    d_nodes = nullptr;
    d_q8_perm = nullptr;
    d_leaves = nullptr;
    d_leaf_prim = nullptr;
    d_leaf_depth = nullptr;
    d_child_entry = nullptr;
    d_leaf_bounds = nullptr;
    d_status = nullptr;
    d_queue = nullptr;
    d_prim_slot = nullptr;
    d_stage = nullptr;
  }
};

template <typename T>
static int upload(T** dst, const std::vector<T>& src) {
  size_t bytes = std::max<size_t>(src.size() * sizeof(T), 16);
  cudaError_t e = cudaMalloc((void**)dst, bytes);
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
  if (!src.empty()) {
    e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_error(e, "cudaMemcpy");
  }
  return BVHGPU_OK;
}

// Traversal stack entries per ray: the tree's worst case unless a smaller
// limit was set (then deeper rays fail with BVHGPU_ERR_STACK_OVERFLOW).
static int stack_cap(const bvhgpu_scene* s) {
  return (s->stack_limit > 0 && s->stack_limit < s->max_stack) ? s->stack_limit : s->max_stack;
}

static int check_opts(const bvhgpu_trace_opts_t* o, dev::LaunchCfg& c) {
  if (!o) return set_error(BVHGPU_ERR_BAD_ARG, "null options");
  if (o->kind != BVHGPU_CLOSEST && o->kind != BVHGPU_ANY) return set_error(BVHGPU_ERR_BAD_ARG, "kind");
  if (o->scheme != BVHGPU_PER_RAY && o->scheme != BVHGPU_STREAM && o->scheme != BVHGPU_PERSISTENT)
    return set_error(BVHGPU_ERR_BAD_ARG, "scheme");
  if (o->policy < 0 || o->policy > 4) return set_error(BVHGPU_ERR_BAD_ARG, "policy");
  if (o->refill < 0 || o->refill > 32) return set_error(BVHGPU_ERR_BAD_ARG, "refill");
  c.policy = o->policy;
  c.refill_min = o->refill ? o->refill : 8;
  if (o->profile != BVHGPU_PROFILE_INSTRUMENTED && o->profile != BVHGPU_PROFILE_FAST)
    return set_error(BVHGPU_ERR_BAD_ARG, "profile");
  c.kind = o->kind;
  c.scheme = o->scheme;
  c.profile = o->profile;
  c.block = o->block ? o->block : 128;
  if (c.block != 32 && c.block != 64 && c.block != 128)
    return set_error(BVHGPU_ERR_BAD_ARG, "block must be 32, 64 or 128");
  int wg = o->workgroup ? o->workgroup : 16;
  if (wg != 8 && wg != 16)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stream workgroup must be 8 or 16 (64 or 256 rays)");
  c.packet = wg * wg;
  if (o->save_distance && o->scheme != BVHGPU_PER_RAY)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "save_distance needs the per-ray scheme");
  c.save_distance = o->save_distance != 0;
  if (o->reorder < 0 || o->reorder > dev::kReorderMaxK)
    return set_error(BVHGPU_ERR_BAD_ARG, "reorder must be 0..32 bins per cube face side");
  c.reorder = o->reorder;
  if (o->stack_local && o->scheme != BVHGPU_PER_RAY)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stack_local needs the per-ray scheme");
  c.stack_local = o->stack_local != 0;
  c.any_order = o->any_order != 0;
  return BVHGPU_OK;
}

// The traversal stacks of a launch must fit the 227 KB of shared memory a
// block may use (the stream scheme keeps a whole packet's state there).
static int check_smem_fit(const dev::LaunchCfg& cfg, int cap) {
  if (cfg.scheme == BVHGPU_STREAM &&
      dev::stream_smem_bytes(cfg.packet, cap, cfg.count) > 227 * 1024)
    return set_error(BVHGPU_ERR_UNSUPPORTED,
                     "stream packet does not fit shared memory for this tree depth");
  // persistent scheme: plus up to 8 KB of staged top levels and 6 KB of ray
  // records (policy 3)
  const size_t extra = cfg.scheme == BVHGPU_PERSISTENT ? 8192 + 128 * 48 : 0;
  if (cfg.scheme != BVHGPU_STREAM &&
      (size_t)cap * 128 * 4 * (cfg.save_distance ? 2 : 1) + extra > 227 * 1024)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stack does not fit shared memory for this tree depth");
  return BVHGPU_OK;
}

// Shared memory per block for the persistent kernel's copy of the top levels;
// small enough to keep six blocks per SM next to the traversal stacks.
constexpr uint32_t kTopStageBytes = 8192;

static int launch(bvhgpu_scene_t s, const dev::TraceArgs& a, dev::LaunchCfg cfg,
                  cudaStream_t st) {
  dev::SceneDev sc = s->dev_view();
  sc.any_index_order = cfg.any_order ? 1 : 0;
  cfg.sm_count = s->sm_count;
  cfg.queue = s->d_queue + (s->queue_next.fetch_add(1) % bvhgpu_scene::kQueueSlots);
  cfg.fmt = s->layout.node_format;
  if (cfg.scheme == BVHGPU_PERSISTENT) {
    // Stage the top levels (up to kTopStageBytes) in shared memory.
    const uint32_t fit = kTopStageBytes / (uint32_t)s->layout.record_bytes;
    cfg.top_nodes = std::min(s->layout.top_nodes, fit);
    cfg.stall_bytes = s->stall_bytes;
  }
  if (cfg.scheme == BVHGPU_STREAM && cfg.fmt != BVHGPU_NODES_FP32)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "the stream scheme traverses FP32 nodes only");
  cudaError_t e;
  switch (s->layout.node_stride) {
    case 4: e = dev::launch_trace_n4(sc, a, cfg, st); break;
    case 8: e = dev::launch_trace_n8(sc, a, cfg, st); break;
    case 12: e = dev::launch_trace_n12(sc, a, cfg, st); break;
    case 16: e = dev::launch_trace_n16(sc, a, cfg, st); break;
    default: return set_error(BVHGPU_ERR_UNSUPPORTED, "node width");
  }
  if (e != cudaSuccess) return cuda_error(e, "trace launch");
  return BVHGPU_OK;
}

static size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Stream-ordered scratch for the reorder passes comes from a memory pool of
// the library's own (one per device, created on first use) that keeps freed
// memory instead of returning it at every synchronisation, so repeated
// traces reuse it; the process's default pool is left as the caller set it.
static int scratch_alloc(int device, void** p, size_t bytes, cudaStream_t st) {
  static std::mutex mu;
  static std::vector<cudaMemPool_t> pools;
  cudaMemPool_t pool = nullptr;
  {
    std::lock_guard<std::mutex> lock(mu);
    if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
    if (!pools[device]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.handleTypes = cudaMemHandleTypeNone;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device;
      cudaError_t e = cudaMemPoolCreate(&pools[device], &props);
      if (e != cudaSuccess) {
        pools[device] = nullptr;
        return cuda_error(e, "scratch memory pool");
      }
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pools[device], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = pools[device];
  }
  cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, st);
  return e == cudaSuccess ? BVHGPU_OK : set_error(BVHGPU_ERR_OOM, "scratch allocation failed");
}

// Scratch bytes of a reordered launch of n rays into k x k cells per face.
static size_t reorder_bytes(uint64_t n, int k) {
  return align256(n * 4) + dev::reorder_scratch_bytes(n, k);
}

// launch() after grouping the rays by direction when cfg.reorder > 0: a
// counting sort writes the input indices in bin order, the kernels take the
// rays in that order and write every result to its input slot. The scratch
// (about 6 bytes per ray, reorder_bytes) is the caller's `scratch` or is
// allocated and freed on the stream.
static int launch_reordered(bvhgpu_scene_t s, dev::TraceArgs a, const dev::LaunchCfg& cfg,
                            cudaStream_t st, void* scratch = nullptr) {
  if (cfg.reorder <= 0 || a.n < 2) return launch(s, a, cfg, st);
  if (a.n > 0xFFFFFFFFull)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "reorder: at most 2^32 - 1 rays per call");
  const size_t perm_bytes = align256(a.n * 4);
  void* p = scratch;
  if (!p) {
    int arc = scratch_alloc(s->device, &p, reorder_bytes(a.n, cfg.reorder), st);
    if (arc) return arc;
  }
  cudaError_t e;
  auto* perm = reinterpret_cast<uint32_t*>(p);
  e = dev::reorder_rays(a.rays, a.n, cfg.reorder, perm, static_cast<uint8_t*>(p) + perm_bytes,
                        st);
  int rc;
  if (e != cudaSuccess) {
    rc = cuda_error(e, "reorder");
  } else {
    a.out_index = perm;
    rc = launch(s, a, cfg, st);
  }
  if (!scratch) {
    e = cudaFreeAsync(p, st);
    if (rc == BVHGPU_OK && e != cudaSuccess) rc = cuda_error(e, "reorder scratch free");
  }
  return rc;
}

extern "C" {

const char* bvhgpu_last_error(void) { return g_last_error.c_str(); }

int bvhgpu_bvh_build(const float* tris, uint64_t n_tris, const bvhgpu_build_params_t* params,
                     bvhgpu_bvh_t* out) {
  if (!tris || !params || !out) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  *out = nullptr;
  BuildParams p;
  p.branching = params->branching;
  p.leaf_size = params->leaf_size;
  p.sort_each_split = params->sort_each_split;
  p.leaf_split_option = params->leaf_split_option;
  p.sah_factor = params->sah_factor;
  p.drop_zero_area = params->drop_zero_area;
  if (!std::isfinite(p.sah_factor)) return set_error(BVHGPU_ERR_BAD_ARG, "sah_factor not finite");
  auto* h = new (std::nothrow) bvhgpu_bvh();
  if (!h) return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  int rc;
  try {
    rc = h->bvh.build(tris, n_tris, p);
  } catch (const std::bad_alloc&) {
    rc = BVHGPU_ERR_OOM;
  }
  if (rc != BVHGPU_OK) {
    delete h;
    return set_error(rc, "bvh build failed (check N in 2..16, L in 1..16, sort_each_split=1, "
                         "finite vertices, at least one non-degenerate triangle)");
  }
  h->n_input = n_tris;
  *out = h;
  return BVHGPU_OK;
}

int bvhgpu_bvh_import_compact(uint64_t n_nodes, const float* lo3, const float* hi3,
                              const uint32_t* child_begin, const uint32_t* child_count,
                              const uint32_t* prim_begin, const uint32_t* prim_count,
                              const int8_t* order48, uint64_t n_prims, const uint32_t* prim_ids,
                              const float* prim_tri9, int32_t branching, int32_t leaf_size,
                              bvhgpu_bvh_t* out) {
  if (!out) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  *out = nullptr;
  auto* h = new (std::nothrow) bvhgpu_bvh();
  if (!h) return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  int rc;
  try {
    rc = h->bvh.import_compact(n_nodes, lo3, hi3, child_begin, child_count, prim_begin,
                               prim_count, order48, n_prims, prim_ids, prim_tri9, branching,
                               leaf_size);
  } catch (const std::bad_alloc&) {
    rc = BVHGPU_ERR_OOM;
  }
  if (rc != BVHGPU_OK) {
    delete h;
    return set_error(rc, "import: not a valid CompactNodeV3 tree (children after their parent, "
                         "one parent each, orders are permutations, leaves of 1..L primitives "
                         "inside the primitive array, finite vertices)");
  }
  uint32_t max_id = 0;
  for (uint64_t i = 0; i < n_prims; ++i) max_id = std::max(max_id, prim_ids[i]);
  h->n_input = (uint64_t)max_id + 1;
  *out = h;
  return BVHGPU_OK;
}

int bvhgpu_bvh_info(bvhgpu_bvh_t h, bvhgpu_bvh_info_t* info) {
  if (!h || !info) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  const Bvh& b = h->bvh;
  info->n_input_tris = h->n_input;
  info->n_tris = b.tris.size();
  info->n_nodes = b.nodes.size();
  info->n_inner = b.inner_count;
  info->n_leaves = b.leaf_count;
  info->depth = b.bvh_depth;
  info->max_stack = b.max_stack;
  info->branching = b.params.branching;
  info->leaf_size = b.params.leaf_size;
  for (int k = 0; k < 3; ++k) {
    info->root_lo[k] = b.nodes[0].bmin[k];
    info->root_hi[k] = b.nodes[0].bmax[k];
  }
  return BVHGPU_OK;
}

int bvhgpu_bvh_free(bvhgpu_bvh_t h) {
  delete h;
  return BVHGPU_OK;
}

int bvhgpu_sah_factor(int32_t branching, int32_t leaf_size, int32_t gang, float* out) {
  if (!out || branching < 1 || leaf_size < 1 || (gang != 4 && gang != 8))
    return set_error(BVHGPU_ERR_BAD_ARG, "bad sah factor query");
  *out = sah_factor_sse(branching, leaf_size, gang);
  return BVHGPU_OK;
}

int bvhgpu_bvh_export_compact(bvhgpu_bvh_t h, float* lo3, float* hi3, uint32_t* child_begin,
                              uint32_t* child_count, uint32_t* prim_begin, uint32_t* prim_count,
                              int8_t* order48, uint8_t* depth, uint32_t* prim_ids,
                              float* prim_tri9) {
  if (!h) return set_error(BVHGPU_ERR_BAD_ARG, "null bvh");
  const Bvh& b = h->bvh;
  for (size_t i = 0; i < b.nodes.size(); ++i) {
    const CompactNode& c = b.nodes[i];
    for (int k = 0; k < 3; ++k) {
      if (lo3) lo3[i * 3 + k] = c.bmin[k];
      if (hi3) hi3[i * 3 + k] = c.bmax[k];
    }
    if (child_begin) child_begin[i] = c.child_begin;
    if (child_count) child_count[i] = c.child_count;
    if (prim_begin) prim_begin[i] = c.prim_begin;
    if (prim_count) prim_count[i] = c.prim_count;
    if (order48) std::memcpy(order48 + i * 48, &c.order[0][0], 48);
    if (depth) depth[i] = c.depth;
  }
  for (size_t i = 0; i < b.prims.size(); ++i) {
    const Triangle& t = b.tris[b.prims[i]];
    if (prim_ids) prim_ids[i] = t.id;
    if (prim_tri9)
      for (int v = 0; v < 3; ++v)
        for (int k = 0; k < 3; ++k) prim_tri9[i * 9 + v * 3 + k] = t.p[v][k];
  }
  return BVHGPU_OK;
}

int bvhgpu_bvh_fast_sizes(bvhgpu_bvh_t h, int32_t gang, int32_t node_memory, int32_t leaf_memory,
                          uint64_t* n_nodes, uint64_t* n_tri_floats) {
  if (!h || !n_nodes || !n_tri_floats) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  if ((gang != 4 && gang != 8) || node_memory < h->bvh.params.branching || node_memory % gang ||
      leaf_memory < h->bvh.params.leaf_size || leaf_memory % gang || node_memory > 32)
    return set_error(BVHGPU_ERR_BAD_ARG, "node/leaf memory must be gang multiples >= N/L");
  *n_nodes = h->bvh.nodes.size();
  *n_tri_floats = (uint64_t)h->bvh.leaf_count * leaf_memory * 9;
  return BVHGPU_OK;
}

int bvhgpu_bvh_export_fast(bvhgpu_bvh_t h, int32_t gang, int32_t node_memory, int32_t leaf_memory,
                           float* bounds, uint32_t* begin, int8_t* order, uint32_t* child_type,
                           float* tri_points) {
  if (!h) return set_error(BVHGPU_ERR_BAD_ARG, "null bvh");
  FastView v;
  int rc = export_fast(h->bvh, gang, node_memory, leaf_memory, v);
  if (rc) return set_error(rc, "fast export failed");
  if (bounds) std::memcpy(bounds, v.bounds.data(), v.bounds.size() * 4);
  if (begin) std::memcpy(begin, v.begin.data(), v.begin.size() * 4);
  if (order) std::memcpy(order, v.order.data(), v.order.size());
  if (child_type) std::memcpy(child_type, v.child_type.data(), v.child_type.size() * 4);
  if (tri_points) std::memcpy(tri_points, v.tri_points.data(), v.tri_points.size() * 4);
  return BVHGPU_OK;
}

int bvhgpu_scene_create(bvhgpu_bvh_t h, const bvhgpu_scene_params_t* params, bvhgpu_scene_t* out) {
  if (!h || !params || !out) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return set_error(BVHGPU_ERR_NO_DEVICE, "no CUDA device");
  if (params->device < 0 || params->device >= ndev)
    return set_error(BVHGPU_ERR_BAD_ARG, "device ordinal out of range");
  if (params->node_format != BVHGPU_NODES_FP32 && params->node_format != BVHGPU_NODES_Q8)
    return set_error(BVHGPU_ERR_BAD_ARG, "node format");
  auto* s = new (std::nothrow) bvhgpu_scene();
  if (!s) return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  s->device = params->device;
  // Q8 records are encoded on the device from the FP32 ones.
  const bool q8 = params->node_format == BVHGPU_NODES_Q8;
  int rc = build_device_layout(h->bvh, params->gang, params->leaf_memory, BVHGPU_NODES_FP32,
                               params->top_levels, s->layout);
  if (rc == BVHGPU_OK && q8) {
    s->layout.node_format = BVHGPU_NODES_Q8;
    s->layout.record_bytes = q8_record_bytes(s->layout.node_stride);
    s->layout.boxes_ordered = false;
  }
  if (rc) {
    delete s;
    return set_error(rc, "device layout failed (gang 4/8, leaf_memory >= L and a gang multiple <= 16)");
  }
  {
    // The host layout and the kernels must agree on the record size.
    const int nm = s->layout.node_stride, fmt = s->layout.node_format;
    int expect = 0;
    if (fmt == BVHGPU_NODES_FP32)
      expect = nm == 4 ? dev::NodeFmt<4, 0>::REC : nm == 8 ? dev::NodeFmt<8, 0>::REC
             : nm == 12 ? dev::NodeFmt<12, 0>::REC : dev::NodeFmt<16, 0>::REC;
    else
      expect = nm == 4 ? dev::NodeFmt<4, 1>::REC : nm == 8 ? dev::NodeFmt<8, 1>::REC
             : nm == 12 ? dev::NodeFmt<12, 1>::REC : dev::NodeFmt<16, 1>::REC;
    if (expect != s->layout.record_bytes) {
      delete s;
      return set_error(BVHGPU_ERR_UNSUPPORTED, "internal: node record size mismatch");
    }
  }
  s->max_stack = h->bvh.max_stack;
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) {
    delete s;
    return cuda_error(e, "cudaSetDevice");
  }
  if ((rc = upload(&s->d_nodes, s->layout.nodes)) || (rc = upload(&s->d_leaves, s->layout.leaves)) ||
      (rc = upload(&s->d_leaf_prim, s->layout.leaf_prim)) ||
      (rc = upload(&s->d_leaf_depth, s->layout.leaf_depth)) ||
      (rc = upload(&s->d_child_entry, s->layout.child_entry)) ||
      (rc = upload(&s->d_leaf_bounds, s->layout.leaf_bounds))) {
    s->release();
    delete s;
    return rc;
  }
  e = cudaMalloc((void**)&s->d_status, 16);
  if (e == cudaSuccess) e = cudaMemset(s->d_status, 0, 16);
  if (e == cudaSuccess && q8) {
    uint8_t* q8_nodes = nullptr;
    const size_t bytes = std::max<size_t>((size_t)s->layout.n_inner * s->layout.record_bytes, 16);
    const size_t pbytes =
        std::max<size_t>((size_t)s->layout.n_inner * q8_perm_bytes(s->layout.node_stride), 16);
    e = cudaMalloc((void**)&q8_nodes, bytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&s->d_q8_perm, pbytes);
    if (e == cudaSuccess)
      e = dev::launch_q8_encode(s->layout.node_stride, s->d_nodes, q8_nodes, s->d_q8_perm,
                                s->layout.n_inner, s->d_status, nullptr);
    int st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&st, s->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(s->d_nodes);
    s->d_nodes = q8_nodes;
    if (e == cudaSuccess && st != 0) {
      s->release();
      delete s;
      return set_error(BVHGPU_ERR_UNSUPPORTED, "Q8 encoding: a box could not be enclosed");
    }
  }
  if (e == cudaSuccess)
    e = cudaMalloc((void**)&s->d_queue, sizeof(unsigned long long) * bvhgpu_scene::kQueueSlots);
  if (e == cudaSuccess)
    e = cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->device);
  if (e != cudaSuccess) {
    s->release();
    delete s;
    return cuda_error(e, "status word");
  }
  {
    uint32_t max_id = 0;
    for (uint32_t id : s->layout.leaf_prim)
      if (id != 0xFFFFFFFFu) max_id = std::max(max_id, id);
    s->prim_slot.assign((size_t)max_id + 1, 0xFFFFFFFFu);
    for (size_t k = 0; k < s->layout.leaf_prim.size(); ++k)
      if (s->layout.leaf_prim[k] != 0xFFFFFFFFu) s->prim_slot[s->layout.leaf_prim[k]] = (uint32_t)k;
  }
  // The host copy of the big arrays is not needed after the upload.
  s->layout.nodes.clear();
  s->layout.nodes.shrink_to_fit();
  s->layout.leaves.clear();
  s->layout.leaves.shrink_to_fit();
  *out = s;
  return BVHGPU_OK;
}

int bvhgpu_scene_node_records(bvhgpu_scene_t s, void* out, uint64_t capacity, uint64_t* bytes) {
  if (!s || !bytes) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  const uint64_t n = (uint64_t)s->layout.n_inner * (uint64_t)s->layout.record_bytes;
  const uint64_t np = s->d_q8_perm
                          ? (uint64_t)s->layout.n_inner * q8_perm_bytes(s->layout.node_stride)
                          : 0;
  *bytes = n + np;
  if (!out) return BVHGPU_OK;
  if (capacity < n + np) return set_error(BVHGPU_ERR_BAD_ARG, "node records: buffer too small");
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess) e = cudaMemcpy(out, s->d_nodes, n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && np)
    e = cudaMemcpy(static_cast<uint8_t*>(out) + n, s->d_q8_perm, np, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? BVHGPU_OK : cuda_error(e, "node records");
}

int bvhgpu_bvh_node_records(bvhgpu_bvh_t h, const bvhgpu_scene_params_t* p, void* out,
                            uint64_t capacity, uint64_t* bytes) {
  if (!h || !p || !bytes) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  DeviceLayout lay;
  int rc = build_device_layout(h->bvh, p->gang, p->leaf_memory, p->node_format, p->top_levels, lay);
  if (rc) return set_error(rc, "device layout failed");
  *bytes = lay.nodes.size() + lay.q8_perm.size();
  if (!out) return BVHGPU_OK;
  if (capacity < *bytes) return set_error(BVHGPU_ERR_BAD_ARG, "node records: buffer too small");
  std::memcpy(out, lay.nodes.data(), lay.nodes.size());
  if (!lay.q8_perm.empty())
    std::memcpy(static_cast<uint8_t*>(out) + lay.nodes.size(), lay.q8_perm.data(),
                lay.q8_perm.size());
  return BVHGPU_OK;
}

int bvhgpu_scene_free(bvhgpu_scene_t s) {
  if (!s) return BVHGPU_OK;
  cudaSetDevice(s->device);
  s->release();
  delete s;
  return BVHGPU_OK;
}

int bvhgpu_scene_bytes(bvhgpu_scene_t s, uint64_t* node_bytes, uint64_t* leaf_bytes,
                       uint64_t* node_record_bytes, uint64_t* leaf_record_bytes) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  const DeviceLayout& L = s->layout;
  if (node_bytes) *node_bytes = (uint64_t)L.n_inner * L.record_bytes;
  if (leaf_bytes) *leaf_bytes = (uint64_t)L.n_leaves * L.leaf_memory * 9 * 4;
  if (node_record_bytes) *node_record_bytes = (uint64_t)L.record_bytes;
  if (leaf_record_bytes) *leaf_record_bytes = (uint64_t)L.leaf_memory * 9 * 4;
  return BVHGPU_OK;
}

// bvhgpu_trace and bvhgpu_trace_steps: a trace of device rays, with the
// stream kernel's step log when step_stats is given.
static int trace_device(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n,
                        const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                        uint32_t* counters, uint64_t* depth_hist, int32_t step_cap,
                        int32_t wide_alternative, uint32_t* step_stats, uint32_t* step_count,
                        void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  dev::LaunchCfg cfg;
  int rc = check_opts(opts, cfg);
  if (rc) return rc;
  if (n == 0) return BVHGPU_OK;
  if (!rays || ((uintptr_t)rays & 15)) return set_error(BVHGPU_ERR_BAD_ARG, "rays: null or not 16-byte aligned");
  if (cfg.kind == BVHGPU_CLOSEST && (!hits || ((uintptr_t)hits & 15)))
    return set_error(BVHGPU_ERR_BAD_ARG, "hits: null or not 16-byte aligned");
  if (cfg.kind == BVHGPU_ANY && !occluded) return set_error(BVHGPU_ERR_BAD_ARG, "occluded: null");
  if (n > (1ull << 40)) return set_error(BVHGPU_ERR_BAD_ARG, "too many rays");
  cfg.count = counters != nullptr || depth_hist != nullptr;
  dev::TraceArgs a;
  a.rays = rays;
  a.n = n;
  a.hits = hits;
  a.occluded = occluded;
  a.counters = counters;
  a.depth_hist = reinterpret_cast<unsigned long long*>(depth_hist);
  if (opts->fullness) {
    if (!depth_hist)
      return set_error(BVHGPU_ERR_BAD_ARG, "fullness: needs depth_hist (2 x 64 + 2 x 17 entries)");
    a.fullness = a.depth_hist + 128;
  }
  a.stack_cap = stack_cap(s);
  if (step_stats) {
    if (cfg.scheme != BVHGPU_STREAM || !cfg.count || !step_count || step_cap < 1 || cfg.reorder)
      return set_error(BVHGPU_ERR_BAD_ARG,
                       "step log: stream scheme, counters, no reorder, step_count and step_cap >= 1");
    a.step_stats = step_stats;
    a.step_count = step_count;
    a.step_cap = step_cap;
    a.step_wide = wide_alternative == 0;
    if (dev::stream_smem_bytes(cfg.packet, a.stack_cap, true, true) > 227 * 1024)
      return set_error(BVHGPU_ERR_UNSUPPORTED, "stream packet with step log does not fit shared memory");
  }
  if ((rc = check_smem_fit(cfg, a.stack_cap))) return rc;
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  return launch_reordered(s, a, cfg, (cudaStream_t)stream);
}

int bvhgpu_trace(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n,
                 const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                 uint32_t* counters, uint64_t* depth_hist, void* stream) {
  return trace_device(s, rays, n, opts, hits, occluded, counters, depth_hist, 0, 1, nullptr,
                      nullptr, stream);
}

int bvhgpu_trace_steps(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n,
                       const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                       uint32_t* counters, uint64_t* depth_hist, int32_t step_cap,
                       int32_t wide_alternative, uint32_t* step_stats, uint32_t* step_count,
                       void* stream) {
  if (n > 0 && (!step_stats || !step_count))
    return set_error(BVHGPU_ERR_BAD_ARG, "step log: null step_stats or step_count");
  return trace_device(s, rays, n, opts, hits, occluded, counters, depth_hist, step_cap,
                      wide_alternative, step_stats, step_count, stream);
}

}  // extern "C"

// Host-buffer pipeline: chunks per batch and the largest chunk (Mi rays)
// when the chunks do not grow. Measured on the 1M-triangle frame (20.7M rays
// in three batches): 4 / 4 Mi 9.24 ms, 8 / 2 Mi 9.54, 8 / 4 Mi 9.55,
// 3 / 8 Mi 9.37, 2 / 8 Mi 9.75, 16 / 1 Mi 9.68.
#ifndef BVHGPU_HOST_CHUNKS
#define BVHGPU_HOST_CHUNKS 4
#endif
#ifndef BVHGPU_HOST_CHUNK_MAX
#define BVHGPU_HOST_CHUNK_MAX 4
#endif
// 1: chunks that grow from BVHGPU_HOST_GROW_FIRST Ki rays by
// BVHGPU_HOST_GROW_PCT percent per chunk, up to BVHGPU_HOST_GROW_MAX Mi, over
// the whole call (across batch boundaries), instead of quarters of each
// batch. Same frame, with the reorder scratch held per stream, two streams:
// median step 8.74-8.75 ms doubling up to 8 Mi, 8.84-9.15 ms in quarters.
// (With the scratch allocated per launch from the pool, growing chunks
// alternated between 8.75 and 10.25 ms per step from run to run.)
// Three streams, median step by growth / cap (three runs on three GPUs):
// 200 % / 8 Mi 8.33-8.39 ms, 200 % / 4 Mi 8.36, 175 % / 3 Mi 8.30,
// 150 % / 8, 6, 4, 3, 2 Mi 8.25, 8.27, 8.03, 8.27, 7.95-8.27,
// 135 % / 4 Mi 8.06, 125 % / 6, 4, 3, 2 Mi 9.05, 7.88 (twice), 7.91, 7.93,
// 115 % / 4 Mi 8.05, 110 % / 8 Mi 8.07; first chunk 128 / 256 / 512 Ki at
// 125 % / 4 Mi: 7.98 / 7.88 / 7.87. With the kernels of a 6.99 ms frame:
// 125 % / 4 Mi 7.21 ms, 125 % / 2 Mi 7.24, 110 % / 4 Mi 7.39, 150 % / 4 Mi
// 7.38. A chunk's copy in waits for the copy out
// of the chunk three before it (same stream, same staging region), so
// chunks that grow slowly keep the copies ahead of the traces without
// leaving one large chunk to trace after the last copy.
#ifndef BVHGPU_HOST_GROW
#define BVHGPU_HOST_GROW 1
#endif
#ifndef BVHGPU_HOST_GROW_MAX
#define BVHGPU_HOST_GROW_MAX 4
#endif
#ifndef BVHGPU_HOST_GROW_PCT
#define BVHGPU_HOST_GROW_PCT 125
#endif
#ifndef BVHGPU_HOST_GROW_FIRST
#define BVHGPU_HOST_GROW_FIRST 256
#endif

namespace {
// One batch of a host-buffer trace: host rays in, host results out.
struct HostBatch {
  const bvhgpu_ray_t* rays;
  uint64_t n;
  dev::LaunchCfg cfg;
  bvhgpu_hit_t* hits;
  uint8_t* occluded;
};
}  // namespace

// Pipeline of host-buffer traces: the rays of every batch go in chunks over
// BVHGPU_HOST_STREAMS internal streams (chunk k on stream k mod that number),
// so the copy of one chunk in, the trace of another and the copy of a third
// out run at the same time, across batch boundaries too. The streams wait
// for `st` first; `st` waits for all of them at the end, and the call
// returns with the results on the host.
static int trace_host_pipeline(bvhgpu_scene_t s, const HostBatch* b, int nb, cudaStream_t st) {
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  std::lock_guard<std::mutex> lock(s->staging_mu);
  constexpr int NS = bvhgpu_scene::kHostStreams;
  for (int i = 0; i < NS; ++i) {
    if (!s->host_stream[i]) {
      e = cudaStreamCreateWithFlags(&s->host_stream[i], cudaStreamNonBlocking);
      if (e != cudaSuccess) return cuda_error(e, "create pipeline stream");
    }
  }
  for (auto& ev : s->host_event) {
    if (!ev) {
      e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_error(e, "create pipeline event");
    }
  }
  // The chunks (batch, first ray, rays). Growing: the first chunk is small,
  // so the copy in that no trace overlaps is short, and each next one a
  // quarter larger (copies run faster than traces, so a chunk's copy ends
  // while the previous chunk traces), up to a cap; a batch's remainder below half
  // the current size joins its last chunk. Otherwise: a quarter of each
  // batch, between 256 Ki and 4 Mi rays.
  struct Chunk {
    int batch;
    uint64_t first, n;
  };
  std::vector<Chunk> chunks;
  uint64_t max_chunk = 0;
  if (BVHGPU_HOST_GROW) {
    uint64_t size = (uint64_t)BVHGPU_HOST_GROW_FIRST << 10;
    const uint64_t cap = (uint64_t)BVHGPU_HOST_GROW_MAX << 20;
    for (int k = 0; k < nb; ++k) {
      for (uint64_t first = 0; first < b[k].n;) {
        uint64_t m = std::min<uint64_t>(size, b[k].n - first);
        if (b[k].n - first - m < size / 2) m = b[k].n - first;
        chunks.push_back({k, first, m});
        max_chunk = std::max(max_chunk, m);
        first += m;
        size = std::min<uint64_t>(size * BVHGPU_HOST_GROW_PCT / 100, cap);
      }
    }
  } else {
    for (int k = 0; k < nb; ++k) {
      uint64_t c = (b[k].n + BVHGPU_HOST_CHUNKS - 1) / BVHGPU_HOST_CHUNKS;
      c = std::max<uint64_t>(c, 256ull << 10);
      c = std::min<uint64_t>(c, (uint64_t)BVHGPU_HOST_CHUNK_MAX << 20);
      c = std::min<uint64_t>(c, b[k].n);
      for (uint64_t first = 0; first < b[k].n; first += c) {
        chunks.push_back({k, first, std::min<uint64_t>(c, b[k].n - first)});
        max_chunk = std::max(max_chunk, c);
      }
    }
  }
  if (max_chunk == 0) return BVHGPU_OK;
  // Per stream: the chunk's rays, its results and the reorder scratch of the
  // largest reordered chunk (held for the call, so that no allocation on one
  // stream waits for memory the other stream frees).
  size_t sort_bytes = 0;
  for (const Chunk& c : chunks)
    if (b[c.batch].cfg.reorder > 0 && c.n >= 2)
      sort_bytes = std::max(sort_bytes, reorder_bytes(c.n, b[c.batch].cfg.reorder));
  const size_t ray_bytes = align256(max_chunk * sizeof(bvhgpu_ray_t));
  const size_t out_bytes = align256(max_chunk * sizeof(bvhgpu_hit_t));
  const size_t per_stream = ray_bytes + out_bytes + sort_bytes;
  const size_t need = per_stream * NS;
  if (need > s->stage_bytes) {
    cudaStreamSynchronize(st);
    for (int i = 0; i < NS; ++i) cudaStreamSynchronize(s->host_stream[i]);
    cudaFree(s->d_stage);
    s->d_stage = nullptr;
    s->stage_bytes = 0;
    e = cudaMalloc(&s->d_stage, need);
    if (e != cudaSuccess) return set_error(BVHGPU_ERR_OOM, "staging allocation failed");
    s->stage_bytes = need;
  }
  e = cudaEventRecord(s->host_event[NS], st);
  if (e != cudaSuccess) return cuda_error(e, "pipeline start event");
  for (int i = 0; i < NS; ++i) {
    e = cudaStreamWaitEvent(s->host_stream[i], s->host_event[NS], 0);
    if (e != cudaSuccess) return cuda_error(e, "pipeline wait");
  }
  int rc = BVHGPU_OK;
  for (size_t k = 0; k < chunks.size() && rc == BVHGPU_OK; ++k) {
    const HostBatch& B = b[chunks[k].batch];
    const bool closest = B.cfg.kind == BVHGPU_CLOSEST;
    const size_t out_rec = closest ? sizeof(bvhgpu_hit_t) : 1;
    const uint64_t first = chunks[k].first, m = chunks[k].n;
    const int si = (int)(k % NS);  // the chunk counter picks the stream
    cudaStream_t cs = s->host_stream[si];
    uint8_t* base = static_cast<uint8_t*>(s->d_stage) + per_stream * si;
    auto* d_rays = reinterpret_cast<bvhgpu_ray_t*>(base);
    uint8_t* d_out = base + ray_bytes;
    e = cudaMemcpyAsync(d_rays, B.rays + first, m * sizeof(bvhgpu_ray_t),
                        cudaMemcpyHostToDevice, cs);
    if (e != cudaSuccess) {
      rc = cuda_error(e, "copy rays in");
      break;
    }
    dev::TraceArgs a;
    a.rays = d_rays;
    a.n = m;
    a.hits = closest ? reinterpret_cast<bvhgpu_hit_t*>(d_out) : nullptr;
    a.occluded = closest ? nullptr : d_out;
    a.counters = nullptr;
    a.depth_hist = nullptr;
    a.stack_cap = stack_cap(s);
    rc = launch_reordered(s, a, B.cfg, cs, sort_bytes ? base + ray_bytes + out_bytes : nullptr);
    if (rc) break;
    void* dst = closest ? (void*)(B.hits + first) : (void*)(B.occluded + first);
    e = cudaMemcpyAsync(dst, d_out, m * out_rec, cudaMemcpyDeviceToHost, cs);
    if (e != cudaSuccess) rc = cuda_error(e, "copy results out");
  }
  for (int i = 0; i < NS; ++i) {
    cudaEventRecord(s->host_event[i], s->host_stream[i]);
    cudaStreamWaitEvent(st, s->host_event[i], 0);
  }
  e = cudaStreamSynchronize(st);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_error(e, "synchronise");
  return BVHGPU_OK;
}

extern "C" {

int bvhgpu_trace_host(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n,
                      const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                      void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  HostBatch b{rays, n, {}, hits, occluded};
  int rc = check_opts(opts, b.cfg);
  if (rc) return rc;
  if (n == 0) return BVHGPU_OK;
  if ((rc = check_smem_fit(b.cfg, stack_cap(s)))) return rc;
  if (!rays) return set_error(BVHGPU_ERR_BAD_ARG, "rays: null");
  if (b.cfg.kind == BVHGPU_CLOSEST ? !hits : !occluded)
    return set_error(BVHGPU_ERR_BAD_ARG, "result buffer: null");
  return trace_host_pipeline(s, &b, 1, (cudaStream_t)stream);
}

int bvhgpu_trace_host_batches(bvhgpu_scene_t s, const bvhgpu_host_batch_t* batches,
                              int32_t n_batches, void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  if (n_batches < 0 || (n_batches > 0 && !batches))
    return set_error(BVHGPU_ERR_BAD_ARG, "batches: null");
  std::vector<HostBatch> b;
  b.reserve((size_t)n_batches);
  for (int i = 0; i < n_batches; ++i) {
    const bvhgpu_host_batch_t& x = batches[i];
    HostBatch h{x.rays, x.n, {}, x.hits, x.occluded};
    int rc = check_opts(x.opts, h.cfg);
    if (rc) return rc;
    if (x.n == 0) continue;
    if ((rc = check_smem_fit(h.cfg, stack_cap(s)))) return rc;
    if (!x.rays) return set_error(BVHGPU_ERR_BAD_ARG, "rays: null");
    if (h.cfg.kind == BVHGPU_CLOSEST ? !x.hits : !x.occluded)
      return set_error(BVHGPU_ERR_BAD_ARG, "result buffer: null");
    b.push_back(h);
  }
  if (b.empty()) return BVHGPU_OK;
  return trace_host_pipeline(s, b.data(), (int)b.size(), (cudaStream_t)stream);
}

}  // extern "C"

namespace bvhgpu {
namespace dev {
cudaError_t launch_batched(const JobTable& t, int profile, int kmode, int sm_count,
                           cudaStream_t s);
cudaError_t launch_aabb_calls(int n, const float* bounds, const uint32_t* offset,
                              const float* fastrays, float* distances, uint8_t* result,
                              uint64_t count, cudaStream_t s);
cudaError_t launch_tri_calls(int l, int gang, const float* tri, const uint32_t* tri_id,
                             float* fastrays, int32_t* result, uint64_t count, cudaStream_t s);
cudaError_t launch_any_calls(int l, const float* tri, const uint32_t* tri_id,
                             const float* fastrays, uint8_t* result, uint64_t count,
                             cudaStream_t s);
}  // namespace dev
}  // namespace bvhgpu

static bool ispc_width(int32_t w) { return w == 4 || w == 8 || w == 12 || w == 16; }

extern "C" {

int bvhgpu_gang_size(void) { return 4; }

int bvhgpu_aabb_intersect(int32_t n, const float* bounds, const uint32_t* offset,
                          const float* fastrays, float* distances, uint8_t* result,
                          uint64_t count, void* stream) {
  if (!ispc_width(n)) return set_error(BVHGPU_ERR_BAD_ARG, "aabbIntersect: n must be 4, 8, 12 or 16");
  if (count == 0) return BVHGPU_OK;
  if (!bounds || !offset || !fastrays || !distances || !result)
    return set_error(BVHGPU_ERR_BAD_ARG, "aabbIntersect: null buffer");
  cudaError_t e = dev::launch_aabb_calls(n, bounds, offset, fastrays, distances, result, count,
                                         (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "aabbIntersect launch");
  return BVHGPU_OK;
}

int bvhgpu_tri_intersect(int32_t l, int32_t gang, const float* tri, const uint32_t* tri_id,
                         float* fastrays, int32_t* result, uint64_t count, void* stream) {
  if (!ispc_width(l)) return set_error(BVHGPU_ERR_BAD_ARG, "triIntersect: l must be 4, 8, 12 or 16");
  if (gang != 4 && gang != 8) return set_error(BVHGPU_ERR_BAD_ARG, "triIntersect: gang 4 or 8");
  if (count == 0) return BVHGPU_OK;
  if (!tri || !tri_id || !fastrays || !result)
    return set_error(BVHGPU_ERR_BAD_ARG, "triIntersect: null buffer");
  cudaError_t e = dev::launch_tri_calls(l, gang, tri, tri_id, fastrays, result, count,
                                        (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "triIntersect launch");
  return BVHGPU_OK;
}

int bvhgpu_tri_any_hit(int32_t l, const float* tri, const uint32_t* tri_id,
                       const float* fastrays, uint8_t* result, uint64_t count, void* stream) {
  if (!ispc_width(l)) return set_error(BVHGPU_ERR_BAD_ARG, "triAnyHit: l must be 4, 8, 12 or 16");
  if (count == 0) return BVHGPU_OK;
  if (!tri || !tri_id || !fastrays || !result)
    return set_error(BVHGPU_ERR_BAD_ARG, "triAnyHit: null buffer");
  cudaError_t e = dev::launch_any_calls(l, tri, tri_id, fastrays, result, count,
                                        (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "triAnyHit launch");
  return BVHGPU_OK;
}

}  // extern "C"

extern "C" {

// Batch of 64 scenes (N8L8, primary + shadow + AO jobs): one launch 10.92 ms,
// one per ray kind 6.12 ms; with N and L tuned per scene (N8 / N16 mixed):
// per ray kind 6.50 ms, per ray kind, node width and format 6.32 ms.
#ifndef BVHGPU_JOBS_SPLIT
#define BVHGPU_JOBS_SPLIT 2
#endif

int bvhgpu_trace_jobs(const bvhgpu_job_t* jobs, int32_t n_jobs, const bvhgpu_trace_opts_t* opts,
                      void* stream) {
  if (n_jobs < 0 || n_jobs > dev::kMaxJobs)
    return set_error(BVHGPU_ERR_BAD_ARG, "at most BVHGPU_MAX_JOBS (192) jobs per launch");
  if (n_jobs > 0 && !jobs) return set_error(BVHGPU_ERR_BAD_ARG, "null jobs");
  dev::LaunchCfg cfg;
  int rc = check_opts(opts, cfg);
  if (rc) return rc;
  if (cfg.policy == 1) return set_error(BVHGPU_ERR_UNSUPPORTED, "jobs: policy 0 or 2");
  static_assert(BVHGPU_MAX_JOBS == dev::kMaxJobs, "job limit");
  std::unique_ptr<dev::JobTable> t(new (std::nothrow) dev::JobTable());
  if (!t) return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  uint64_t total = 0;
  int device = -1, stack = 1, sms = 0;
  bvhgpu_scene_t first = nullptr;
  int nj = 0;
  // Reordered jobs: one segmented counting sort over all of them.
  std::unique_ptr<dev::SegTable> seg(new (std::nothrow) dev::SegTable());
  if (!seg) return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  int seg_k = 0;
  size_t seg_bytes = 0;
  std::vector<size_t> seg_off;
  std::vector<int> seg_job;  // job table slot of each reordered job
  for (int i = 0; i < n_jobs; ++i) {
    const bvhgpu_job_t& j = jobs[i];
    if (!j.scene) return set_error(BVHGPU_ERR_BAD_ARG, "job without a scene");
    if (j.reorder < 0 || j.reorder > dev::kReorderMaxK)
      return set_error(BVHGPU_ERR_BAD_ARG, "job reorder must be 0..32");
    if (j.reorder && seg_k && j.reorder != seg_k)
      return set_error(BVHGPU_ERR_UNSUPPORTED, "reordered jobs of one call must share K");
    if (j.kind != BVHGPU_CLOSEST && j.kind != BVHGPU_ANY) return set_error(BVHGPU_ERR_BAD_ARG, "job kind");
    if (j.n >= (1ull << 32)) return set_error(BVHGPU_ERR_BAD_ARG, "job with 2^32 rays or more");
    if (device >= 0 && j.scene->device != device)
      return set_error(BVHGPU_ERR_BAD_ARG, "jobs on different devices");
    device = j.scene->device;
    if (j.n == 0) continue;
    if (!j.rays || ((uintptr_t)j.rays & 15)) return set_error(BVHGPU_ERR_BAD_ARG, "job rays");
    if (j.kind == BVHGPU_CLOSEST ? (!j.hits || ((uintptr_t)j.hits & 15)) : !j.occluded)
      return set_error(BVHGPU_ERR_BAD_ARG, "job result buffer");
    if (!first) first = j.scene;
    dev::JobDev& d = t->jobs[nj++];
    d.nodes = j.scene->d_nodes;
    d.leaves = j.scene->d_leaves;
    d.leaf_prim = j.scene->d_leaf_prim;
    d.rays = j.rays;
    d.out = j.kind == BVHGPU_CLOSEST ? (void*)j.hits : (void*)j.occluded;
    d.status = j.scene->d_status;
    d.ray_begin = total;
    d.n = (uint32_t)j.n;
    d.root_entry = j.scene->layout.root_entry;
    d.leaf_memory = j.scene->layout.leaf_memory;
    d.gang = (int16_t)j.scene->layout.gang;
    d.nm = (int8_t)j.scene->layout.node_stride;
    d.fmt = (int8_t)j.scene->layout.node_format;
    d.kind = (int8_t)j.kind;
    d.boxes_ordered = j.scene->layout.boxes_ordered ? 1 : 0;
    d.any_index_order = j.any_order ? 1 : 0;
    d.perm = nullptr;
    d.q8_perm = j.scene->d_q8_perm;
    d.leaf_bounds = j.scene->d_leaf_bounds;
    if (j.reorder && j.n > 1) {
      seg_k = j.reorder;
      seg_off.push_back(seg_bytes);
      seg_bytes += dev::seg_job_scratch_bytes(j.n, seg_k);
      seg_job.push_back(nj - 1);
      dev::SegJob& sj = seg->jobs[seg->n_jobs++];
      sj.rays = j.rays;
      sj.n = (uint32_t)j.n;
    }
    total += j.n;
    stack = std::max(stack, stack_cap(j.scene));
    sms = j.scene->sm_count;
  }
  if (nj == 0) return BVHGPU_OK;
  if ((size_t)stack * 128 * 4 > 227 * 1024)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stack does not fit shared memory for these trees");
  t->n_jobs = nj;
  t->total = total;
  t->head = first->d_queue + (first->queue_next.fetch_add(1) % bvhgpu_scene::kQueueSlots);
  t->refill_min = cfg.refill_min;
  t->stack_cap = stack;
  t->policy = cfg.policy;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  void* scratch = nullptr;
  if (seg->n_jobs > 0) {
    int arc = scratch_alloc(device, &scratch, seg_bytes, st);
    if (arc) return arc;
    seg->k = seg_k;
    uint32_t chunk = 0;
    for (int i = 0; i < seg->n_jobs; ++i) {
      dev::SegJob& sj = seg->jobs[i];
      dev::seg_job_carve(sj, static_cast<uint8_t*>(scratch) + seg_off[i], sj.n, seg_k);
      sj.first_chunk = chunk;
      chunk += sj.nchunks;
      t->jobs[seg_job[i]].perm = sj.perm;
    }
    seg->total_chunks = chunk;
    e = dev::reorder_jobs(*seg, st);
    if (e != cudaSuccess) {
      cudaFreeAsync(scratch, st);
      return cuda_error(e, "job reorder");
    }
  }
  // Jobs run in groups of one ray kind (BVHGPU_JOBS_SPLIT 1), or of one ray
  // kind and node width and format (2), one persistent launch per group on
  // the stream, each kernel compiled for its kind: lanes of one warp then
  // take one code path. 0: one launch, kind per lane.
  auto group_of = [&](const dev::JobDev& d) {
    const int k = d.kind == BVHGPU_ANY ? 1 : 0;
    return BVHGPU_JOBS_SPLIT >= 2 ? (k << 8) | ((int)d.nm << 1) | (int)d.fmt : k;
  };
  std::vector<int> groups;
  for (int i = 0; i < nj; ++i) {
    const int g = group_of(t->jobs[i]);
    if (std::find(groups.begin(), groups.end(), g) == groups.end()) groups.push_back(g);
  }
  std::sort(groups.begin(), groups.end());
  if (opts->one_launch) {
    // One launch: closest-hit jobs first in queue order, then any-hit jobs.
    std::unique_ptr<dev::JobTable> one(new (std::nothrow) dev::JobTable());
    if (!one) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess) {
      *one = *t;
      int m = 0;
      uint64_t begin = 0;
      for (int pass = 0; pass < 2; ++pass)
        for (int i = 0; i < nj; ++i) {
          if ((t->jobs[i].kind == BVHGPU_ANY) != (pass == 1)) continue;
          one->jobs[m] = t->jobs[i];
          one->jobs[m].ray_begin = begin;
          begin += t->jobs[i].n;
          ++m;
        }
        // (pass 0 ends at the split between the kinds)
      one->split = 0;
      for (int i = 0; i < nj; ++i)
        if (t->jobs[i].kind != BVHGPU_ANY) one->split += t->jobs[i].n;
      one->head_any = first->d_queue + (first->queue_next.fetch_add(1) % bvhgpu_scene::kQueueSlots);
      e = dev::launch_batched(*one, cfg.profile, 3, sms, st);
    }
  } else if (!BVHGPU_JOBS_SPLIT) {
    int kinds = 0;
    for (int i = 0; i < nj; ++i) kinds |= t->jobs[i].kind == BVHGPU_ANY ? 2 : 1;
    e = dev::launch_batched(*t, cfg.profile, kinds == 3 ? 0 : kinds, sms, st);
  } else if (groups.size() == 1) {
    e = dev::launch_batched(*t, cfg.profile, t->jobs[0].kind == BVHGPU_ANY ? 2 : 1, sms, st);
  } else {
    std::unique_ptr<dev::JobTable> part(new (std::nothrow) dev::JobTable());
    if (!part) e = cudaErrorMemoryAllocation;
    for (size_t gi = 0; gi < groups.size() && e == cudaSuccess; ++gi) {
      *part = *t;
      int m = 0, kind = BVHGPU_CLOSEST;
      uint64_t begin = 0;
      for (int i = 0; i < nj; ++i) {
        if (group_of(t->jobs[i]) != groups[gi]) continue;
        part->jobs[m] = t->jobs[i];
        part->jobs[m].ray_begin = begin;
        begin += t->jobs[i].n;
        kind = t->jobs[i].kind;
        ++m;
      }
      part->n_jobs = m;
      part->total = begin;
      part->head = first->d_queue + (first->queue_next.fetch_add(1) % bvhgpu_scene::kQueueSlots);
      e = dev::launch_batched(*part, cfg.profile, kind == BVHGPU_ANY ? 2 : 1, sms, st);
    }
  }
  if (scratch) {
    cudaError_t f = cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = f;
  }
  if (e != cudaSuccess) return cuda_error(e, "batched launch");
  return BVHGPU_OK;
}

}  // extern "C"

extern "C" {

int bvhgpu_adjoint(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n, const float* grad_hits,
                   float* grad_tri9, float* grad_rays, void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  if (n == 0) return BVHGPU_OK;
  if (!rays || !grad_hits || !grad_tri9 || !grad_rays || ((uintptr_t)rays & 15) ||
      ((uintptr_t)grad_hits & 15) || ((uintptr_t)grad_rays & 15))
    return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: null or misaligned buffer");
  if (s->layout.node_format != BVHGPU_NODES_FP32)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "adjoint: FP32 node scenes only");
  if ((size_t)s->max_stack * 128 * 4 > 227 * 1024)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stack does not fit shared memory for this tree depth");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  dev::AdjointArgs a{rays, n, reinterpret_cast<const float4*>(grad_hits), grad_tri9, grad_rays,
                     stack_cap(s)};
  e = dev::launch_adjoint(s->dev_view(), s->layout.node_stride, a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "adjoint launch");
  return BVHGPU_OK;
}


int bvhgpu_adjoint_vertices(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, uint64_t n,
                            const float* grad_hits, const int32_t* faces, uint64_t n_faces,
                            uint64_t n_verts, float* grad_verts, float* grad_rays,
                            void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  if (n == 0) return BVHGPU_OK;
  if (!rays || !grad_hits || !faces || !grad_verts || !grad_rays || ((uintptr_t)rays & 15) ||
      ((uintptr_t)grad_hits & 15) || ((uintptr_t)grad_rays & 15) || ((uintptr_t)faces & 3) ||
      ((uintptr_t)grad_verts & 3))
    return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: null or misaligned buffer");
  if (n_faces < s->prim_slot.size())
    return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: fewer faces than input triangles");
  if (n_verts >= (1ull << 32)) return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: 2^32 vertices or more");
  if (s->layout.node_format != BVHGPU_NODES_FP32)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "adjoint: FP32 node scenes only");
  if ((size_t)s->max_stack * 128 * 4 > 227 * 1024)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "stack does not fit shared memory for this tree depth");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  dev::AdjointArgs a{rays, n, reinterpret_cast<const float4*>(grad_hits), nullptr, grad_rays,
                     stack_cap(s)};
  a.faces = faces;
  a.grad_verts = grad_verts;
  a.n_verts = (uint32_t)n_verts;
  e = dev::launch_adjoint(s->dev_view(), s->layout.node_stride, a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "adjoint launch");
  return BVHGPU_OK;
}

int bvhgpu_adjoint_hits(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, const bvhgpu_hit_t* hits,
                        uint64_t n, const float* grad_t, const float* grad_u,
                        const float* grad_v, const int32_t* faces, uint64_t n_faces,
                        uint64_t n_verts, float* grad_verts, float* grad_tri9, float* grad_rays,
                        void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  if (n == 0) return BVHGPU_OK;
  if (!rays || !hits || !grad_rays || ((uintptr_t)rays & 15) || ((uintptr_t)hits & 15) ||
      ((uintptr_t)grad_rays & 15) || ((uintptr_t)grad_t & 3) || ((uintptr_t)grad_u & 3) ||
      ((uintptr_t)grad_v & 3))
    return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: null or misaligned buffer");
  if (faces) {
    if (!grad_verts || grad_tri9 || ((uintptr_t)faces & 3) || ((uintptr_t)grad_verts & 3))
      return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: faces need grad_verts (and no grad_tri9)");
    if (n_faces < s->prim_slot.size())
      return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: fewer faces than input triangles");
    if (n_verts >= (1ull << 32))
      return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: 2^32 vertices or more");
  } else if (!grad_tri9 || grad_verts) {
    return set_error(BVHGPU_ERR_BAD_ARG, "adjoint: grad_tri9 without faces");
  }
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  {
    std::lock_guard<std::mutex> lock(s->staging_mu);
    if (!s->d_prim_slot) {
      int rc = upload(&s->d_prim_slot, s->prim_slot);
      if (rc) return rc;
    }
  }
  dev::AdjointArgs a{rays, n, nullptr, grad_tri9, grad_rays, stack_cap(s)};
  a.grad_t = grad_t;
  a.grad_u = grad_u;
  a.grad_v = grad_v;
  a.faces = faces;
  a.grad_verts = grad_verts;
  a.n_verts = (uint32_t)n_verts;
  a.hits = reinterpret_cast<const float4*>(hits);
  a.prim_slot = s->d_prim_slot;
  a.n_prims = (uint32_t)s->prim_slot.size();
  e = dev::launch_adjoint(s->dev_view(), s->layout.node_stride, a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "adjoint launch");
  return BVHGPU_OK;
}

}  // extern "C"

namespace bvhgpu {
namespace dev {
struct Fp64Args {
  const bvhgpu_ray_t* rays;
  const float4* hits;
  uint64_t n;
  const uint32_t* prim_slot;
  uint32_t n_prims;
  int profile;
  double* out;
};
cudaError_t launch_fp64_check(const SceneDev& sc, const Fp64Args& a, cudaStream_t s);
}  // namespace dev
}  // namespace bvhgpu

extern "C" {

int bvhgpu_fp64_check(bvhgpu_scene_t s, const bvhgpu_ray_t* rays, const bvhgpu_hit_t* hits,
                      uint64_t n, int32_t profile, double* out, void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  if (n == 0) return BVHGPU_OK;
  if (!rays || !hits || !out || ((uintptr_t)rays & 15) || ((uintptr_t)hits & 15) ||
      ((uintptr_t)out & 7))
    return set_error(BVHGPU_ERR_BAD_ARG, "fp64 check: null or misaligned buffer");
  if (profile != BVHGPU_PROFILE_INSTRUMENTED && profile != BVHGPU_PROFILE_FAST)
    return set_error(BVHGPU_ERR_BAD_ARG, "profile");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  {
    std::lock_guard<std::mutex> lock(s->staging_mu);
    if (!s->d_prim_slot) {
      int rc = upload(&s->d_prim_slot, s->prim_slot);
      if (rc) return rc;
    }
  }
  dev::Fp64Args a{rays, reinterpret_cast<const float4*>(hits), n, s->d_prim_slot,
                  (uint32_t)s->prim_slot.size(), profile, out};
  e = dev::launch_fp64_check(s->dev_view(), a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "fp64 check launch");
  return BVHGPU_OK;
}

int bvhgpu_scene_inject_stall(bvhgpu_scene_t s, int32_t on) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  s->stall_bytes = on ? 16u : 0u;
  return BVHGPU_OK;
}

int bvhgpu_camera_rays(const bvhgpu_camera_t* c, bvhgpu_ray_t* rays, void* stream) {
  if (!c) return set_error(BVHGPU_ERR_BAD_ARG, "null camera");
  if (c->width == 0 || c->height == 0) return BVHGPU_OK;
  if (!rays || ((uintptr_t)rays & 15))
    return set_error(BVHGPU_ERR_BAD_ARG, "camera rays: null or not 16-byte aligned");
  if (c->workgroup < 1 || c->workgroup > 4096)
    return set_error(BVHGPU_ERR_BAD_ARG, "camera rays: workgroup must be 1..4096");
  if ((uint64_t)c->width * c->height > (1ull << 36))
    return set_error(BVHGPU_ERR_BAD_ARG, "camera rays: at most 2^36 pixels");
  dev::CameraArgs a;
  for (int k = 0; k < 3; ++k) a.pos[k] = c->pos[k];
  for (int k = 0; k < 16; ++k) a.transform[k] = c->transform[k];
  a.width = c->width;
  a.height = c->height;
  a.workgroup = c->workgroup;
  a.focal = c->focal;
  a.tmax = c->tmax;
  a.n = (uint64_t)c->width * c->height;
  cudaError_t e = dev::launch_camera_rays(a, rays, (cudaStream_t)stream);
  return e == cudaSuccess ? BVHGPU_OK : cuda_error(e, "camera rays");
}

int bvhgpu_secondary_rays(bvhgpu_scene_t s, const bvhgpu_ray_t* primary, const bvhgpu_hit_t* hits,
                          uint64_t n, const bvhgpu_secondary_t* p, bvhgpu_ray_t* shadow,
                          bvhgpu_ray_t* ao, void* stream) {
  if (!s || !p) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  if (p->ao_samples < 0 || p->ao_samples > 1024)
    return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: ao_samples must be 0..1024");
  if (p->sampling != BVHGPU_AO_COSINE && p->sampling != BVHGPU_AO_REFERENCE)
    return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: sampling");
  if (n == 0) return BVHGPU_OK;
  if (n > (1ull << 36)) return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: at most 2^36 rays");
  if (!primary || !hits || ((uintptr_t)primary & 15) || ((uintptr_t)hits & 15))
    return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: primary rays / hits null or misaligned");
  if (shadow && ((uintptr_t)shadow & 15))
    return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: shadow not 16-byte aligned");
  if (p->ao_samples > 0 && (!ao || ((uintptr_t)ao & 15)))
    return set_error(BVHGPU_ERR_BAD_ARG, "secondary rays: ao null or not 16-byte aligned");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  {
    std::lock_guard<std::mutex> lock(s->staging_mu);
    if (!s->d_prim_slot) {
      int rc = upload(&s->d_prim_slot, s->prim_slot);
      if (rc) return rc;
    }
  }
  dev::SecondaryArgs a;
  a.primary = primary;
  a.hits = reinterpret_cast<const float4*>(hits);
  a.n = n;
  a.prim_slot = s->d_prim_slot;
  a.n_prims = (uint32_t)s->prim_slot.size();
  a.shadow = shadow;
  a.ao = p->ao_samples > 0 ? ao : nullptr;
  for (int k = 0; k < 3; ++k) a.light[k] = p->light[k];
  a.offset = p->offset;
  a.ao_samples = p->ao_samples;
  a.ao_length = p->ao_length;
  a.sampling = p->sampling;
  a.seed = p->seed;
  e = dev::launch_secondary_rays(s->dev_view(), a, (cudaStream_t)stream);
  return e == cudaSuccess ? BVHGPU_OK : cuda_error(e, "secondary rays");
}

int bvhgpu_ao_factor(const uint8_t* occluded, uint64_t n, int32_t samples, float* factor,
                     void* stream) {
  if (samples < 1) return set_error(BVHGPU_ERR_BAD_ARG, "ao factor: samples must be >= 1");
  if (n == 0) return BVHGPU_OK;
  if (n > (1ull << 36)) return set_error(BVHGPU_ERR_BAD_ARG, "ao factor: at most 2^36 pixels");
  if (!occluded || !factor) return set_error(BVHGPU_ERR_BAD_ARG, "ao factor: null buffer");
  cudaError_t e = dev::launch_ao_factor(occluded, n, samples, factor, (cudaStream_t)stream);
  return e == cudaSuccess ? BVHGPU_OK : cuda_error(e, "ao factor");
}

int bvhgpu_scene_set_stack_limit(bvhgpu_scene_t s, int32_t entries) {
  if (!s || entries < 0) return set_error(BVHGPU_ERR_BAD_ARG, "stack limit");
  s->stack_limit = entries;
  return BVHGPU_OK;
}

// FastRay: tMax, pos[3], invDirection[3], direction[3] (src/fastRay.h:14-29).
static void fastrays_to_rays(const float* fr, uint64_t n, std::vector<bvhgpu_ray_t>& rays) {
  rays.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    const float* f = fr + i * 10;
    rays[i] = bvhgpu_ray_t{f[1], f[2], f[3], f[0], f[7], f[8], f[9], 0.0f};
  }
}

int bvhgpu_intersect_fastrays(bvhgpu_scene_t s, float* fastrays, uint64_t n, int32_t scheme,
                              uint32_t* leaf_index, int8_t* tri_index, void* stream) {
  if (!s || (n && (!fastrays || !leaf_index || !tri_index)))
    return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  if (n == 0) return BVHGPU_OK;
  std::vector<bvhgpu_ray_t> rays;
  std::vector<bvhgpu_hit_t> hits(n);
  try {
    fastrays_to_rays(fastrays, n, rays);
  } catch (const std::bad_alloc&) {
    return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  }
  bvhgpu_trace_opts_t o{BVHGPU_CLOSEST, scheme, BVHGPU_PROFILE_FAST, 16, 128, 0, 0, 0, 0, 0};
  int rc = bvhgpu_trace_host(s, rays.data(), n, &o, hits.data(), nullptr, stream);
  if (rc) return rc;
  const uint32_t lm = (uint32_t)s->layout.leaf_memory;
  for (uint64_t i = 0; i < n; ++i) {
    if (hits[i].prim < 0) {
      tri_index[i] = -1;
      continue;
    }
    const uint32_t slot = s->prim_slot[(uint32_t)hits[i].prim];
    leaf_index[i] = (slot / lm) * 9 * lm;
    tri_index[i] = (int8_t)(slot % lm);
    fastrays[i * 10] = hits[i].t;
  }
  return BVHGPU_OK;
}

int bvhgpu_intersect_secondary_fastrays(bvhgpu_scene_t s, const float* fastrays, uint64_t n,
                                        int32_t scheme, uint16_t* result, void* stream) {
  if (!s || (n && (!fastrays || !result))) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  if (n == 0) return BVHGPU_OK;
  std::vector<bvhgpu_ray_t> rays;
  std::vector<uint8_t> occ(n);
  try {
    fastrays_to_rays(fastrays, n, rays);
  } catch (const std::bad_alloc&) {
    return set_error(BVHGPU_ERR_OOM, "host allocation failed");
  }
  bvhgpu_trace_opts_t o{BVHGPU_ANY, scheme, BVHGPU_PROFILE_FAST, 16, 128, 0, 0, 0, 0, 0};
  int rc = bvhgpu_trace_host(s, rays.data(), n, &o, nullptr, occ.data(), stream);
  if (rc) return rc;
  for (uint64_t i = 0; i < n; ++i) result[i] = (uint16_t)(result[i] + occ[i]);
  return BVHGPU_OK;
}

int bvhgpu_scene_status(bvhgpu_scene_t s, void* stream) {
  if (!s) return set_error(BVHGPU_ERR_BAD_ARG, "null scene");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  int code = 0;
  e = cudaMemcpyAsync(&code, s->d_status, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "status read");
  if (code != 0) {
    cudaMemsetAsync(s->d_status, 0, sizeof(int), (cudaStream_t)stream);
    cudaStreamSynchronize((cudaStream_t)stream);
    const char* what = code == BVHGPU_ERR_STACK_OVERFLOW ? "device: traversal stack overflow"
                       : code == BVHGPU_ERR_TIMEOUT     ? "device: bounded wait timed out"
                       : code == BVHGPU_ERR_BAD_ARG     ? "device: vertex or triangle id out of range"
                       : code == BVHGPU_ERR_UNSUPPORTED ? "device: node encoding failed"
                                                        : "device: error";
    return set_error(code, what);
  }
  return BVHGPU_OK;
}


}  // extern "C"

// ---------------------------------------------------------------------------
// Entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc while they trace: a renderer plugin
// whose host application owns the GPU memory budget and forbids growing it
// after start-up, or a frame loop that cannot afford the device-wide
// synchronisation an allocation may cause. bvhgpu_trace_batches_noalloc
// serves them: it runs the persistent traversal kernel with its only scratch
// (one ray-queue head per batch) in the fixed array below, so the call itself
// allocates nothing; the caller passes the rays and the result buffers.
//
// The array is a file-scope device variable: every GPU that loads the library
// holds its kNoAllocQueueSlots * 8 bytes until the process exits. Host code
// may not use the symbol as an address, so the device address is looked up
// with cudaGetSymbolAddress (with that device current) on the first call for
// that device, and again on the first call after the device's context was
// destroyed and re-created (cudaDeviceReset), since the array then lives at a
// new address; make that first call before any stream capture. The first call
// with a given ray kind, profile, policy and node width may also load that
// kernel variant into the context (CUDA's lazy module loading), which can
// take device memory for the code itself; a caller that must see no device
// memory change at all warms up every combination it will use.
// Every call shares the array and leaves its contents behind: each call clears
// the heads it uses before its launches, and calls that overlap on the GPU
// (different streams of one device) race on the heads, so serialise them.
namespace {

constexpr int kNoAllocQueueSlots = 64;  // at most 64 batches per call (512 bytes)
static __device__ __align__(256) unsigned long long g_noalloc_queue[kNoAllocQueueSlots];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned long long* g_noalloc_addr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};  // context id of each address

// Unique id of the calling thread's current context (ids are never reused
// within a process, unlike context handles), through the driver entry points
// the runtime hands out, so the library does not link libcuda itself.
// Returns 0 when the driver does not provide them.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
  });
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of g_noalloc_queue on `device` (which must be current): looked
// up once per device and context.
int noalloc_scratch(int device, unsigned long long** out) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "no-alloc trace: device ordinal above 63");
  const unsigned long long ctx = current_context_id();
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device] || ctx == 0 || g_noalloc_ctx[device] != ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_queue);
    if (e != cudaSuccess) return cuda_error(e, "no-alloc trace: cudaGetSymbolAddress");
    g_noalloc_addr[device] = static_cast<unsigned long long*>(p);
    g_noalloc_ctx[device] = ctx;
  }
  *out = g_noalloc_addr[device];
  return BVHGPU_OK;
}

}  // namespace

extern "C" {

int bvhgpu_trace_batches_noalloc(bvhgpu_scene_t s, const bvhgpu_batch_t* batches,
                                 int32_t n_batches, const bvhgpu_trace_opts_t* opts,
                                 void* stream) {
  if (n_batches < 0 || n_batches > kNoAllocQueueSlots)
    return set_error(BVHGPU_ERR_BAD_ARG,
                     "no-alloc trace: at most 64 batches per call (the fixed scratch holds 64 "
                     "queue heads)");
  if (!s || (n_batches > 0 && !batches)) return set_error(BVHGPU_ERR_BAD_ARG, "null argument");
  dev::LaunchCfg cfg;
  int rc = check_opts(opts, cfg);
  if (rc) return rc;
  if (cfg.reorder)
    return set_error(BVHGPU_ERR_UNSUPPORTED, "no-alloc trace: reorder needs scratch memory");
  if (cfg.save_distance || cfg.stack_local)
    return set_error(BVHGPU_ERR_UNSUPPORTED,
                     "no-alloc trace runs the persistent scheme: no save_distance or stack_local");
  cfg.scheme = BVHGPU_PERSISTENT;
  for (int i = 0; i < n_batches; ++i) {
    const bvhgpu_batch_t& b = batches[i];
    if (b.kind != BVHGPU_CLOSEST && b.kind != BVHGPU_ANY)
      return set_error(BVHGPU_ERR_BAD_ARG, "no-alloc trace: batch kind");
    if (b.n == 0) continue;
    if (b.n > (1ull << 40)) return set_error(BVHGPU_ERR_BAD_ARG, "too many rays");
    if (!b.rays || ((uintptr_t)b.rays & 15))
      return set_error(BVHGPU_ERR_BAD_ARG, "no-alloc trace: rays null or not 16-byte aligned");
    if (b.kind == BVHGPU_CLOSEST ? (!b.hits || ((uintptr_t)b.hits & 15)) : !b.occluded)
      return set_error(BVHGPU_ERR_BAD_ARG, "no-alloc trace: result buffer null or misaligned");
  }
  if ((rc = check_smem_fit(cfg, stack_cap(s)))) return rc;
  if (n_batches == 0) return BVHGPU_OK;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  unsigned long long* heads = nullptr;
  if ((rc = noalloc_scratch(s->device, &heads))) return rc;
  // The heads keep the previous call's values: clear the ones this call uses.
  e = cudaMemsetAsync(heads, 0, sizeof(unsigned long long) * (size_t)n_batches, st);
  if (e != cudaSuccess) return cuda_error(e, "no-alloc trace: clear queue heads");
  dev::SceneDev sc = s->dev_view();
  sc.any_index_order = cfg.any_order ? 1 : 0;
  for (int i = 0; i < n_batches; ++i) {
    const bvhgpu_batch_t& b = batches[i];
    if (b.n == 0) continue;
    dev::TraceArgs a;
    a.rays = b.rays;
    a.n = b.n;
    a.hits = b.kind == BVHGPU_CLOSEST ? b.hits : nullptr;
    a.occluded = b.kind == BVHGPU_ANY ? b.occluded : nullptr;
    a.counters = nullptr;
    a.depth_hist = nullptr;
    a.stack_cap = stack_cap(s);
    dev::LaunchCfg c = cfg;
    c.kind = b.kind;
    c.count = false;
    c.sm_count = s->sm_count;
    c.queue = heads + i;
    c.queue_cleared = true;
    c.fmt = s->layout.node_format;
    // Top levels staged in shared memory, as the regular persistent launches do.
    c.top_nodes = std::min(s->layout.top_nodes, kTopStageBytes / (uint32_t)s->layout.record_bytes);
    c.stall_bytes = s->stall_bytes;
    switch (s->layout.node_stride) {
      case 4: e = dev::launch_trace_n4(sc, a, c, st); break;
      case 8: e = dev::launch_trace_n8(sc, a, c, st); break;
      case 12: e = dev::launch_trace_n12(sc, a, c, st); break;
      case 16: e = dev::launch_trace_n16(sc, a, c, st); break;
      default: return set_error(BVHGPU_ERR_UNSUPPORTED, "node width");
    }
    if (e != cudaSuccess) return cuda_error(e, "no-alloc trace launch");
  }
  return BVHGPU_OK;
}

}  // extern "C"
