/*
 * bvhgpu — GB300 (sm_103a) traversal of N-wide BVHs with L-wide leaves.
 *
 * C ABI of the drop-in boundary. All entry points return a status int
 * (BVHGPU_OK == 0); no C++ exception crosses this boundary. Buffers are
 * owned by the caller unless a function says otherwise. Calls that take a
 * `stream` are stream-ordered and do not synchronise unless noted; distinct
 * streams may call concurrently into distinct scenes.
 *
 * What each entry point replaces in the reference (Hengoo/BVHRaytracer):
 *   bvhgpu_bvh_build          Bvh::Bvh + Bvh::recursiveBvh + Bvh::bvhAnalysis
 *                             (src/accelerationStructure/bvh.cpp:28-40,
 *                              src/accelerationStructure/aabb.cpp:71-206,
 *                              src/rayTracer.cpp:604-623)
 *   bvhgpu_sah_factor         RayTracer::loadSahFactor (src/rayTracer.cpp:880-925)
 *   bvhgpu_bvh_import_compact the upload of a tree the reference built itself
 *                             (its CompactNodeManager arrays, compactNode.cpp:11-116)
 *   bvhgpu_bvh_export_compact CompactNodeManager<CompactNodeV3> constructor
 *                             (src/accelerationStructure/compactNode.cpp:11-116)
 *   bvhgpu_bvh_export_fast    FastNodeManager constructor
 *                             (src/accelerationStructure/fastNodeManager.h:1495-1688)
 *   bvhgpu_scene_create       the device-resident copy of the flat BVH (no
 *                             reference counterpart: the reference is CPU-only)
 *   bvhgpu_trace              FastNodeManager::intersect / intersectSecondary /
 *                             intersectWideAlternative / intersectSecondaryWideAlternative
 *                             (fastNodeManager.h:1328-1493, 835-1230) and the
 *                             instrumented CompactNodeManager::intersectImmediately /
 *                             intersectWideAlternative (compactNode.cpp:604-814, 357-601)
 *   bvhgpu_trace_steps        intersectWideAlternative with the per-step data of
 *                             CameraData's workgroup analysis (compactNode.cpp:357-601,
 *                             cameraData.h:660-1105)
 *   bvhgpu_trace_host[_batches] the same, on host buffers (copies in the call)
 *   bvhgpu_adjoint[_vertices|_hits] no reference counterpart: reverse pass of
 *                             triIntersect{L}'s Moller-Trumbore (rayTracerTemplate.ispc:35-76)
 *   bvhgpu_trace_jobs         many scenes in one persistent launch per ray kind (the refill
 *                             structure, fastNodeManager.h:92-156, across scenes)
 *   bvhgpu_camera_rays        Camera::getRayTargetPosition + FastRay (camera.h:82-98)
 *   bvhgpu_secondary_rays     getSurfaceNormalPosition + shadow / AO set-up
 *                             (fastNodeManager.h:1700-1713, cameraFast.h:366-381, 513-552,
 *                             camera.cpp:21-52)
 *   bvhgpu_ao_factor          the AO term of cameraData.h:403-406
 *   bvhgpu_gang_size / bvhgpu_aabb_intersect / bvhgpu_tri_intersect / bvhgpu_tri_any_hit
 *                             getGangSize / aabbIntersect{N} / triIntersect{L} / triAnyHit{L},
 *                             the ISPC C ABI (src/ISPC/rayTracerTemplate.ispc:3-233), batched
 *   bvhgpu_intersect_fastrays FastNodeManager::intersectWideAlternative on FastRay
 *                             records (fastNodeManager.h:835-1049; FastRay: src/fastRay.h:14-29)
 *   bvhgpu_intersect_secondary_fastrays
 *                             FastNodeManager::intersectSecondaryWideAlternative
 *                             (fastNodeManager.h:1051-1230)
 */
#ifndef BVHGPU_H
#define BVHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define BVHGPU_OK 0
#define BVHGPU_ERR_BAD_ARG 1        /* null pointer, size or option out of range */
#define BVHGPU_ERR_OOM 2            /* device or host allocation failed */
#define BVHGPU_ERR_CUDA 3           /* a CUDA runtime call failed */
#define BVHGPU_ERR_STACK_OVERFLOW 4 /* a ray needed more stack than the scene holds */
#define BVHGPU_ERR_TIMEOUT 5        /* a bounded device wait gave up */
#define BVHGPU_ERR_UNSUPPORTED 6    /* option combination not built */
#define BVHGPU_ERR_NO_DEVICE 7      /* no CUDA device visible */

/* ---- handles ----------------------------------------------------------- */
typedef struct bvhgpu_bvh* bvhgpu_bvh_t;     /* host BVH (builder output) */
typedef struct bvhgpu_scene* bvhgpu_scene_t; /* device-resident scene */

/* ---- host BVH build ---------------------------------------------------- */
/* Knobs of the reference's config.txt (minBranch..maxLeafSize, sortEachSplit,
 * leafSplitOption) and its per-(N, L) SAH node factor. */
typedef struct {
  int32_t branching;         /* N, 2..16 */
  int32_t leaf_size;         /* L, 1..16 */
  int32_t sort_each_split;   /* must be 1 (per-axis child orders) */
  int32_t leaf_split_option; /* 0, 1 or 2 */
  float sah_factor;          /* sahNodeFactor; see bvhgpu_sah_factor */
  int32_t drop_zero_area;    /* 1: skip zero-area triangles like the scene loader */
} bvhgpu_build_params_t;

typedef struct {
  uint64_t n_input_tris; /* triangles passed in */
  uint64_t n_tris;       /* triangles kept (zero-area ones dropped) */
  uint64_t n_nodes;      /* all nodes, leaves included (reference numbering) */
  uint64_t n_inner;
  uint64_t n_leaves;
  int32_t depth;         /* bvhDepth: deepest leaf depth + 1 */
  int32_t max_stack;     /* worst-case depth-first stack height */
  int32_t branching;
  int32_t leaf_size;
  float root_lo[3];
  float root_hi[3];
} bvhgpu_bvh_info_t;

/* tris: n_tris x 9 floats (p0, p1, p2), world space, in scene-loader order.
 * Primitive ids reported by traces are indices into this array. */
int bvhgpu_bvh_build(const float* tris, uint64_t n_tris, const bvhgpu_build_params_t* params,
                     bvhgpu_bvh_t* out);
int bvhgpu_bvh_info(bvhgpu_bvh_t bvh, bvhgpu_bvh_info_t* info);

/* A tree built elsewhere — typically by the reference's own builder — handed
 * over as its CompactNodeV3 arrays (the layout bvhgpu_bvh_export_compact
 * writes: CompactNodeManager's compactNodes and the primitive list,
 * compactNode.cpp:11-116): n_nodes nodes in reference numbering (root 0,
 * children consecutive and numbered after their parent, as customTreeOrder
 * gives), order48[node*48 + axis*16 + i] = traverseOrderEachAxis, leaves of
 * 1..leaf_size primitives; n_prims triangles (prim_tri9, 9 floats each, in
 * the primitive list's order) with their input ids. The arrays are copied and
 * validated; depths and the worst-case stack height are recomputed. The
 * result is used like a bvhgpu_bvh_build result. */
int bvhgpu_bvh_import_compact(uint64_t n_nodes, const float* lo3, const float* hi3,
                              const uint32_t* child_begin, const uint32_t* child_count,
                              const uint32_t* prim_begin, const uint32_t* prim_count,
                              const int8_t* order48, uint64_t n_prims, const uint32_t* prim_ids,
                              const float* prim_tri9, int32_t branching, int32_t leaf_size,
                              bvhgpu_bvh_t* out);
int bvhgpu_bvh_free(bvhgpu_bvh_t bvh);

/* sahNodeFactor for (N, L) from the reference's SSE table, with N and L
 * rounded up to the gang size; gang 8 returns 1 like the reference. */
int bvhgpu_sah_factor(int32_t branching, int32_t leaf_size, int32_t gang, float* out);

/* CompactNodeV3 view, reference node numbering (root = 0, customTreeOrder).
 * Arrays sized by bvhgpu_bvh_info: n_nodes entries each (lo3/hi3: 3 per node,
 * order48: 48 int8 per node, order[axis][i] at [axis*16+i]); prim_ids and
 * prim_tri9 are sized n_tris (prim_tri9: 9 floats each) in sorted order. */
int bvhgpu_bvh_export_compact(bvhgpu_bvh_t bvh, float* lo3, float* hi3, uint32_t* child_begin,
                              uint32_t* child_count, uint32_t* prim_begin, uint32_t* prim_count,
                              int8_t* order48, uint8_t* depth, uint32_t* prim_ids,
                              float* prim_tri9);

/* FastNode<node_memory> view and trianglePoints of FastNodeManager with the
 * given gang size (4 for SSE4, 8 for AVX2) and leaf memory. */
int bvhgpu_bvh_fast_sizes(bvhgpu_bvh_t bvh, int32_t gang, int32_t node_memory,
                          int32_t leaf_memory, uint64_t* n_nodes, uint64_t* n_tri_floats);
int bvhgpu_bvh_export_fast(bvhgpu_bvh_t bvh, int32_t gang, int32_t node_memory,
                           int32_t leaf_memory, float* bounds /* n_nodes*6*node_memory */,
                           uint32_t* begin /* childIdBegin or primIdBegin */,
                           int8_t* order /* n_nodes*3*node_memory */,
                           uint32_t* child_type /* bit j: child j is an inner node */,
                           float* tri_points);

/* ---- device scene ------------------------------------------------------ */
#define BVHGPU_NODES_FP32 0 /* float child boxes */
#define BVHGPU_NODES_Q8 1   /* 8-bit child boxes relative to the parent box */

typedef struct {
  int32_t gang;        /* 4 (SSE4 gang) or 8: leaf padding and fast-profile tie rule */
  int32_t leaf_memory; /* 0: L rounded up to the gang */
  int32_t node_format; /* BVHGPU_NODES_FP32 or BVHGPU_NODES_Q8 */
  int32_t top_levels;  /* inner levels laid out first, staged in shared memory (0..4) */
  int32_t device;      /* CUDA device ordinal */
} bvhgpu_scene_params_t;

int bvhgpu_scene_create(bvhgpu_bvh_t bvh, const bvhgpu_scene_params_t* params,
                        bvhgpu_scene_t* out);
int bvhgpu_scene_free(bvhgpu_scene_t scene);
/* Device bytes of the node array and of the leaf array. */
int bvhgpu_scene_bytes(bvhgpu_scene_t scene, uint64_t* node_bytes, uint64_t* leaf_bytes,
                       uint64_t* node_record_bytes, uint64_t* leaf_record_bytes);

/* ---- tracing ----------------------------------------------------------- */
typedef struct {
  float ox, oy, oz, tmax; /* origin and ray length limit */
  float dx, dy, dz, pad;  /* direction (see profiles) */
} bvhgpu_ray_t;           /* 32 bytes */

typedef struct {
  int32_t prim; /* input triangle index, -1 on miss */
  float t;      /* hit distance (profile units) */
  float u, v;   /* barycentric weights of p1 and p2 */
} bvhgpu_hit_t; /* 16 bytes */

#define BVHGPU_CLOSEST 0 /* closest hit (primary rays) */
#define BVHGPU_ANY 1     /* any hit (shadow / ambient-occlusion rays) */

#define BVHGPU_PER_RAY 0 /* depth-first traversal, one thread per ray */
#define BVHGPU_STREAM 1  /* ray-stream traversal over node / leaf work lists */
/* depth-first per ray, by persistent warps that refill finished lanes from a
 * global ray queue (same per-ray results as BVHGPU_PER_RAY) */
#define BVHGPU_PERSISTENT 2

/* Instrumented profile: CompactNodeManager + Ray + Triangle::intersect
 * semantics (direction normalised, watertight leaf test with the per-triangle
 * box pre-test, child order by the major axis for every ray).
 * Fast profile: FastNodeManager + FastRay + ISPC semantics (direction used as
 * given, Moller-Trumbore leaf test with gang-lane tie rule, index child order
 * for any-hit rays). */
#define BVHGPU_PROFILE_INSTRUMENTED 0
#define BVHGPU_PROFILE_FAST 1

typedef struct {
  int32_t kind;      /* BVHGPU_CLOSEST / BVHGPU_ANY */
  int32_t scheme;    /* BVHGPU_PER_RAY / BVHGPU_STREAM */
  int32_t profile;   /* BVHGPU_PROFILE_* */
  int32_t workgroup; /* stream scheme: packet = workgroup^2 rays (8, 16); 0 = 16 */
  int32_t block;     /* per-ray scheme: threads per block (32, 64, 128; 0 = 128) */
  int32_t policy;    /* persistent scheme: 0 while-while, 1 if-if, 2 while-while with
                        one leaf per lane set aside, 3 the same with up to two leaves per
                        lane, 4 as 3 with the warp's set-aside leaves tested as one pool
                        of (ray, triangle) pairs, 32 at a time (2 to 4: any-hit rays
                        without counters; else 0) */
  int32_t refill;    /* persistent scheme: idle lanes of a warp that trigger a refill
                        (1..32; 0 = 8) */
  int32_t save_distance; /* per-ray scheme, nonzero: the save-distance traversal of
                        FastNodeManager::intersectSaveDistance (fastNodeManager.h:1232-1326)
                        and intersectImmediately(ray, useDistance = true)
                        (compactNode.cpp:604-814): stack entries carry the box entry
                        distance, pops beyond the current tMax are skipped uncounted.
                        Any-hit rays are unaffected (their tMax never shrinks). Other
                        schemes: must be 0. */
  int32_t reorder;   /* 0: trace the rays in input order. K in 1..32: first group them
                        by direction into 6 K^2 cube-map cells (a counting sort of their
                        indices into stream-ordered scratch of about 6 bytes per ray),
                        trace them in that order and write every result to its input
                        slot; at most 2^32 - 1 rays per call. Results are identical
                        either way; incoherent rays (ambient occlusion) run faster
                        grouped. */
  int32_t stack_local; /* per-ray scheme, nonzero: each thread's traversal stack in local
                        memory (when the tree needs at most 64 entries; else shared
                        memory, the default placement). Same results. */
  int32_t any_order; /* 0: any-hit rays push the hit children of a node in the reference's
                        order (instrumented profile: traverseOrderEachAxis of the ray's
                        major axis; fast profile: child-index order). Nonzero: any-hit
                        rays without counters push them in child-index order in both
                        profiles. Same results (an any-hit ray's result does not depend
                        on the order in which its leaves are reached); short rays
                        (ambient occlusion) run faster, long rays toward a light slower. */
  int32_t fullness;  /* nonzero (with depth_hist): depth_hist holds 2 x 64 + 2 x 17 uint64;
                        after the per-depth rows come the reference's Ray::childFullness
                        and primitiveFullness (ray.h:36-37, compactNode.cpp:655,716)
                        summed over the rays: visits of nodes with c children
                        (entry 128 + c) and of leaves with c triangles (entry 145 + c),
                        c = 0..16. Instrumented and fast profile, every scheme. */
  int32_t one_launch; /* bvhgpu_trace_jobs: 0 one persistent launch per group of jobs with
                        one ray kind, node width and node format; nonzero: one launch for
                        all jobs, the closest-hit jobs' rays queued before the any-hit
                        jobs', each warp tracing one kind at a time (it takes any-hit
                        rays once the closest-hit queue is empty and its lanes are done).
                        Same results. */
} bvhgpu_trace_opts_t;

/* Counters per ray when `counters` is non-null (8 uint32 per ray):
 * node visits, leaf visits, box tests, box hits, triangle tests,
 * triangle hits, deepest stack, reserved. `depth_hist` (nullable):
 * 2 x 64 uint64, node visits then leaf visits per tree depth, accumulated;
 * with opts.fullness, 2 x 17 more: the fullness histograms. */
#define BVHGPU_COUNTERS_PER_RAY 8

/* Device pointers. Closest: writes hits[n]. Any: writes occluded[n] (0/1).
 * Rays whose origin x is NaN are skipped (miss / not occluded), like the
 * reference's inactive secondary rays. */
int bvhgpu_trace(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, uint64_t n,
                 const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                 uint32_t* counters, uint64_t* depth_hist, void* stream);

/* The stream scheme with counters and a step log, for CameraData's workgroup
 * analysis (cameraData.h:660-1109): for each packet (workgroup) p and step s
 * (step 0 = the state before the loop, compactNode.cpp:410-415), writes
 * step_stats[(p * step_cap + s) * 5 ..] = (rays doing node work, unique nodes
 * among them, rays doing leaf work, unique leaves among them, rays that
 * terminate) as intersectWideAlternative collects them
 * (compactNode.cpp:357-601), and step_count[p] = the packet's number of steps;
 * steps at or beyond step_cap are counted but not written. wide_alternative
 * 0 logs intersectWide's schedule instead (compactNode.cpp:118-356: a ray
 * whose node visit leaves a leaf on top visits that leaf in the same step).
 * opts: scheme BVHGPU_STREAM, no reorder; counters non-null; packets of
 * opts->workgroup^2 rays in ray order. Results and counters equal
 * bvhgpu_trace's. */
int bvhgpu_trace_steps(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, uint64_t n,
                       const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                       uint32_t* counters, uint64_t* depth_hist, int32_t step_cap,
                       int32_t wide_alternative, uint32_t* step_stats, uint32_t* step_count,
                       void* stream);

/* Host pointers: copies rays in, traces, copies results out, synchronises
 * `stream`. Device staging buffers are owned by the scene and reused. */
int bvhgpu_trace_host(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, uint64_t n,
                      const bvhgpu_trace_opts_t* opts, bvhgpu_hit_t* hits, uint8_t* occluded,
                      void* stream);

/* Several host-buffer batches of one scene (a frame's primary, shadow and
 * ambient-occlusion rays), each with its own options, in one call: the
 * chunked copies in, traces and copies out of all batches form one pipeline,
 * so a batch's first copy overlaps the previous batch's last trace. Results
 * equal bvhgpu_trace_host's per batch; synchronises `stream` once. */
typedef struct {
  const bvhgpu_ray_t* rays;         /* host */
  uint64_t n;
  const bvhgpu_trace_opts_t* opts;  /* kind, scheme, ... of this batch */
  bvhgpu_hit_t* hits;               /* host, closest */
  uint8_t* occluded;                /* host, any */
} bvhgpu_host_batch_t;

int bvhgpu_trace_host_batches(bvhgpu_scene_t scene, const bvhgpu_host_batch_t* batches,
                              int32_t n_batches, void* stream);

/* ---- many scenes in one launch ---------------------------------------- */
/* A job: one ray batch traced in one scene. bvhgpu_trace_jobs traces up to
 * BVHGPU_MAX_JOBS jobs (scenes of any N, L and node format, closest or any
 * hit, uneven sizes) in one persistent launch per group of jobs with the same
 * ray kind, node width and node format (each kernel compiled for its kind)
 * that pulls rays from a global queue spanning the group's jobs, scenes of
 * any size mixed (the GPU form of the reference's
 * workgroup refill, fastNodeManager.h:92-156, 277-450, extended across
 * scenes). Results per ray
 * equal bvhgpu_trace's. All scenes must live on the stream's device; the
 * options' profile and policy (0 or 2) apply to every job. Stream-ordered, no
 * synchronisation (so it can be recorded in a CUDA graph); no allocation
 * unless a job is reordered, whose scratch (about 6 bytes per ray) comes from
 * the stream-ordered allocator (cudaMallocAsync / cudaFreeAsync on the
 * stream, which graph capture records as memory nodes). */
#define BVHGPU_MAX_JOBS 192
typedef struct {
  bvhgpu_scene_t scene;
  const bvhgpu_ray_t* rays; /* device, 16-byte aligned */
  uint64_t n;               /* < 2^32 */
  int32_t kind;             /* BVHGPU_CLOSEST or BVHGPU_ANY */
  int32_t reorder;          /* 0, or K (1..32): trace the job's rays grouped into 6 K^2
                               direction bins (see bvhgpu_trace_opts_t.reorder); all
                               reordered jobs of a call use the same K */
  bvhgpu_hit_t* hits;       /* closest: device, 16-byte aligned */
  uint8_t* occluded;        /* any: device */
  int32_t any_order;        /* any: see bvhgpu_trace_opts_t.any_order (per job here) */
  int32_t pad;              /* 0 */
} bvhgpu_job_t;

int bvhgpu_trace_jobs(const bvhgpu_job_t* jobs, int32_t n_jobs, const bvhgpu_trace_opts_t* opts,
                      void* stream);

/* ---- the reference's ISPC kernels, batched ----------------------------- */
/* The extern "C" functions the ISPC compiler generates from
 * src/ISPC/rayTracerTemplate.ispc and fastNodeManager.h binds
 * (fastNodeManager.h:247-257), as batches of independent calls, one GPU
 * thread per call: where the reference calls aabbIntersect{N}(bounds,
 * distances, rayInfo) once per node visit, bvhgpu_aabb_intersect takes count
 * such calls. Device pointers; stream-ordered. `fastrays` are the reference's
 * FastRay records (10 floats: tMax, pos[3], invDirection[3], direction[3];
 * src/fastRay.h:14-29) used as given; rows of the node bounds and leaf blocks
 * are `width` floats long (padding 1), as in the FastNode / trianglePoints
 * arrays of bvhgpu_bvh_export_fast. */

/* getGangSize (rayTracerTemplate.ispc:3-6): the gang the fast profile uses
 * by default (4, the SSE4 build's programCount; scenes may use 8). */
int bvhgpu_gang_size(void);

/* aabbIntersect{N} (rayTracerTemplate.ispc:171-233), N = n in {4, 8, 12, 16}:
 * call i slab-tests fastrays[i] against the n boxes of bounds + offset[i]
 * (rows min x, min y, min z, max x, max y, max z); writes distances[i * n +
 * lane] = t0 for every hit lane (the other entries are left as they are) and
 * result[i] = 1 if any lane is hit. */
int bvhgpu_aabb_intersect(int32_t n, const float* bounds, const uint32_t* offset,
                          const float* fastrays, float* distances, uint8_t* result,
                          uint64_t count, void* stream);

/* triIntersect{L} (rayTracerTemplate.ispc:28-108), L = l in {4, 8, 12, 16}:
 * call i tests fastrays[i] against the l triangles of the leaf block at
 * tri + tri_id[i] (tri_id: the primIdBegin float offset) with the gang-lane
 * tie rule of a `gang`-wide ISPC gang (4 or 8); result[i] = the in-leaf index
 * of the hit or -1, and a hit lowers fastrays[i * 10] (tMax) to its t. */
int bvhgpu_tri_intersect(int32_t l, int32_t gang, const float* tri, const uint32_t* tri_id,
                         float* fastrays, int32_t* result, uint64_t count, void* stream);

/* triAnyHit{L} (rayTracerTemplate.ispc:112-168): result[i] = 1 if any of the
 * l triangles at tri + tri_id[i] is hit within tMax. */
int bvhgpu_tri_any_hit(int32_t l, const float* tri, const uint32_t* tri_id,
                       const float* fastrays, uint8_t* result, uint64_t count, void* stream);

/* ---- FastRay drop-in -------------------------------------------------- */
/* Host arrays of the reference's FastRay records (40 bytes each: tMax,
 * pos[3], invDirection[3], direction[3]; src/fastRay.h:14-29), fast profile.
 * Closest hit (intersect / intersectWideAlternative): for each hit ray, sets
 * tMax to the hit distance, leaf_index[i] to the leaf's primIdBegin (float
 * offset of its triangle block) and tri_index[i] to the in-leaf index; misses
 * keep tMax and get tri_index -1 (leaf_index untouched), like
 * fastNodeManager.h:1010-1015 after triIndex.fill(-1) (cameraFast.h:483).
 * Any hit (intersectSecondary[Wide]): result[i] += 1 for each occluded ray;
 * rays whose pos.x is NaN are skipped (fastNodeManager.h:1075-1082).
 * scheme: BVHGPU_PER_RAY or BVHGPU_STREAM (workgroup 16). Synchronises. */
int bvhgpu_intersect_fastrays(bvhgpu_scene_t scene, float* fastrays, uint64_t n, int32_t scheme,
                              uint32_t* leaf_index, int8_t* tri_index, void* stream);
int bvhgpu_intersect_secondary_fastrays(bvhgpu_scene_t scene, const float* fastrays, uint64_t n,
                                        int32_t scheme, uint16_t* result, void* stream);

/* ---- adjoint ---------------------------------------------------------- */
/* Backward pass of the closest-hit leaf intersection through a fixed
 * visibility set (fast profile: Moller-Trumbore of triIntersect{L},
 * rayTracerTemplate.ispc:35-76). For each ray the kernel re-traces the closest
 * hit (no stored hits are read) and, given grad_hits[i] = (unused, dL/dt,
 * dL/du, dL/dv), adds dL/dp0, dL/dp1, dL/dp2 of the hit triangle into
 * grad_tri9[prim*9 .. prim*9+8] (atomically: zero it first; sized by the input
 * triangle count) and writes grad_rays[i*8 ..] = (dL/do, 0, dL/dd, 0). Rays
 * that miss get zero gradients. FP32 node scenes only. Device pointers,
 * 16-byte aligned; stream-ordered. */
int bvhgpu_adjoint(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, uint64_t n,
                   const float* grad_hits, float* grad_tri9, float* grad_rays, void* stream);

/* The same backward pass for an indexed mesh: instead of grad_tri9, the
 * gradients of the hit triangle's three vertices are added (atomically: zero
 * first) into grad_verts[3 * v .. 3 * v + 2] for v = faces[3 * prim + k]
 * (int32 vertex ids of each input triangle, n_faces >= the input triangle
 * count). Vertex ids outside [0, n_verts) are skipped and recorded as
 * BVHGPU_ERR_BAD_ARG for bvhgpu_scene_status. */
int bvhgpu_adjoint_vertices(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, uint64_t n,
                            const float* grad_hits, const int32_t* faces, uint64_t n_faces,
                            uint64_t n_verts, float* grad_verts, float* grad_rays,
                            void* stream);

/* The same backward passes from the forward pass's closest hits instead of a
 * re-trace (no traversal: one thread per ray reads its hit, the triangle and
 * the ray), with the incoming gradients as separate per-ray arrays grad_t,
 * grad_u, grad_v (dL/dt, dL/du, dL/dv; NULL: zero) instead of grad_hits
 * records. hits[i] is bvhgpu_trace's record of ray i (fast profile for the
 * forward pass's hits to be the ones the gradients describe); its prim selects
 * the triangle, prim -1 gives zero gradients, an id the scene does not hold
 * gives zero gradients and is recorded as BVHGPU_ERR_BAD_ARG. With faces, the
 * vertex gradients go to grad_verts as in bvhgpu_adjoint_vertices (grad_tri9
 * NULL); without, to grad_tri9 as in bvhgpu_adjoint (grad_verts NULL). Any
 * node format. The first call uploads the scene's id -> leaf slot map. */
int bvhgpu_adjoint_hits(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, const bvhgpu_hit_t* hits,
                        uint64_t n, const float* grad_t, const float* grad_u,
                        const float* grad_v, const int32_t* faces, uint64_t n_faces,
                        uint64_t n_verts, float* grad_verts, float* grad_tri9, float* grad_rays,
                        void* stream);

/* ---- tracing without allocation --------------------------------------- */
/* No counterpart in the reference (its renderer allocates nothing on a GPU).
 * For callers that must not allocate GPU memory while they trace (a plugin
 * whose host application owns the memory budget, a frame loop that cannot
 * take the synchronisation an allocation may cause): traces up to 64 ray
 * batches with the persistent kernel, whose scratch (one ray-queue head per
 * batch) lives in a fixed 512-byte device array inside the library instead of
 * being allocated. More than 64 batches -> BVHGPU_ERR_BAD_ARG. The first call
 * on a device, and the first after that device's context was destroyed and
 * re-created (cudaDeviceReset), looks up that array's address: make it before
 * any stream capture. The first call with a given kind, profile, policy and
 * node width may also load that kernel variant (CUDA lazy loading), which can
 * take device memory for its code: warm up each combination once where no
 * change of free device memory may be seen. All calls share the array: calls
 * that overlap on the GPU race. opts: profile, policy, refill and any_order
 * are used; scheme is always persistent; reorder, save_distance and
 * stack_local -> BVHGPU_ERR_UNSUPPORTED. The top levels are staged in shared
 * memory as in the regular persistent launches. */
typedef struct {
  const bvhgpu_ray_t* rays; /* device, 16-byte aligned */
  uint64_t n;
  int32_t kind;             /* BVHGPU_CLOSEST or BVHGPU_ANY */
  int32_t pad;
  bvhgpu_hit_t* hits;       /* closest: device, n records, 16-byte aligned */
  uint8_t* occluded;        /* any: device, n bytes */
} bvhgpu_batch_t;

int bvhgpu_trace_batches_noalloc(bvhgpu_scene_t scene, const bvhgpu_batch_t* batches,
                                 int32_t n_batches, const bvhgpu_trace_opts_t* opts,
                                 void* stream);

/* ---- FP64 check ------------------------------------------------------- */
/* For each ray with a closest hit (hits[i].prim >= 0), recomputes the hit
 * record of the same ray / triangle pair in double precision (Moller-Trumbore
 * on the FP32 ray the kernels traced: normalised in the instrumented
 * profile) and writes out[i*4 ..] = (t64, b1_64, b2_64, |t - t64| / |t64|);
 * misses get NaN. The only kernel that computes in FP64. Device pointers
 * (rays, hits 16-byte aligned); stream-ordered. */
int bvhgpu_fp64_check(bvhgpu_scene_t scene, const bvhgpu_ray_t* rays, const bvhgpu_hit_t* hits,
                      uint64_t n, int32_t profile, double* out, void* stream);

/* ---- measurement ------------------------------------------------------- */
/* No counterpart in the reference. Read bandwidth of `device` in GB/s: a
 * buffer of `bytes` (allocated and freed inside the call) is read `passes`
 * times by one L2-cached, L1-bypassing streaming kernel, timed with CUDA
 * events `repeats` times; *gb_per_s is the median. A buffer that fits L2
 * (129 MB on GB300) gives the L2 read ceiling of the traversal kernels when
 * the BVH is L2-resident; a buffer far larger than L2 gives the HBM read
 * rate. Synchronous (default stream). */
int bvhgpu_read_bandwidth(int32_t device, uint64_t bytes, int32_t passes, int32_t repeats,
                          double* gb_per_s);

/* ---- ray generation on the GPU ----------------------------------------- */
/* Pinhole camera of Camera::getRayTargetPosition (camera.h:82-98): pixel (w, h)
 * with w = col - width/2, h = height/2 - row (integers) has the target
 * pos + transform * ((w, h, 0) / width + (0, 0, -focal)), and the ray is
 * FastRay(pos, target) (fastRay.cpp:3-20): direction = target - pos, not
 * normalised. Pixels are emitted tile by tile (workgroup x workgroup pixels,
 * row-major tiles, row-major inside a tile; edge tiles keep the pixels inside
 * the image), the order of CameraFast's workgroups (cameraFast.h:465-490). */
typedef struct {
  float pos[3];
  float transform[16]; /* camera to world, column-major (glm::inverse(glm::lookAt(..))) */
  uint32_t width, height;
  int32_t workgroup;   /* tile side in pixels (16) */
  float focal;         /* 0.866: 60 degree horizontal field of view */
  float tmax;          /* 222222: FastRay's default */
} bvhgpu_camera_t;

/* Replaces the ray set-up loops of CameraFast::renderImage
 * (cameraFast.h:484-490, 339-341). rays: width * height device records. */
int bvhgpu_camera_rays(const bvhgpu_camera_t* camera, bvhgpu_ray_t* rays, void* stream);

#define BVHGPU_AO_COSINE 0    /* cosine-distributed around the normal, hashed from (seed, ray, sample) */
#define BVHGPU_AO_REFERENCE 1 /* Camera::getAmbientDirection: FNV-1a-hashed (u, v), uniform
                                 hemisphere flipped to the normal side (camera.cpp:21-52) */
typedef struct {
  float light[3];      /* point light of the shadow rays */
  float offset;        /* origin offset along the normal: 0.001 (cameraFast.h:373) */
  int32_t ao_samples;  /* AO rays per primary ray (0: none) */
  float ao_length;     /* tMax of the AO rays (ambientDistance) */
  int32_t sampling;    /* BVHGPU_AO_* */
  int32_t pad;
  uint64_t seed;       /* cosine: hash seed; reference: pixel index of primary ray 0 */
} bvhgpu_secondary_t;

/* Secondary rays from closest hits, on the device: for primary ray i with a
 * hit, the geometric normal and ray-plane hit point of getSurfaceNormalPosition
 * (fastNodeManager.h:1700-1713), origin = point + normal * offset; shadow[i]
 * toward the light (unit direction, tMax = distance) when `shadow` is
 * non-null; ao[i * ao_samples + k] for k < ao_samples (unit directions, tMax =
 * ao_length). Rays of a missed primary get a NaN origin (inactive), as in
 * cameraFast.h:524-528. Replaces cameraFast.h:366-381 and 513-552. */
int bvhgpu_secondary_rays(bvhgpu_scene_t scene, const bvhgpu_ray_t* primary,
                          const bvhgpu_hit_t* hits, uint64_t n, const bvhgpu_secondary_t* params,
                          bvhgpu_ray_t* shadow, bvhgpu_ray_t* ao, void* stream);

/* factor[i] = 1 - (occluded AO samples of pixel i) / samples, the ambient
 * term of CameraData (cameraData.h:403-406); occluded holds n * samples bytes
 * in the layout of bvhgpu_secondary_rays. */
int bvhgpu_ao_factor(const uint8_t* occluded, uint64_t n, int32_t samples, float* factor,
                     void* stream);

/* ---- node records (no reference counterpart) --------------------------- */
/* Copies the scene's device node records (n_inner * record bytes; Q8 scenes
 * encode them on the device, and their push-sequence side array, n_inner *
 * 6 * (2, 4 or 8 for 4, 8 or 12-16 child slots) bytes, follows the records)
 * to `out`; *bytes gets the size (out may be null to query it). */
int bvhgpu_scene_node_records(bvhgpu_scene_t scene, void* out, uint64_t capacity,
                              uint64_t* bytes);
/* The same records as encoded on the host by the layout builder, for the
 * given scene parameters (the specification the device encoding matches). */
int bvhgpu_bvh_node_records(bvhgpu_bvh_t bvh, const bvhgpu_scene_params_t* params, void* out,
                            uint64_t capacity, uint64_t* bytes);

/* Caps the traversal stack at `entries` per ray (0: the tree's worst case,
 * the default, which never overflows). Rays that need more stop, report a
 * miss and record BVHGPU_ERR_STACK_OVERFLOW for bvhgpu_scene_status; the
 * reference's stacks are a fixed 48 entries (fastNodeManager.h:1333). */
int bvhgpu_scene_set_stack_limit(bvhgpu_scene_t scene, int32_t entries);

/* Failure-detection testing (no reference counterpart). With `on`, the
 * persistent kernels of this scene that stage top levels in shared memory
 * (scene top_levels > 0) wait for 16 bytes that no copy delivers; the wait
 * gives up after 0.5 s, the blocks stop without tracing and
 * bvhgpu_scene_status reports BVHGPU_ERR_TIMEOUT. No GPU fault is involved.
 * Call with 0 to restore normal operation. */
int bvhgpu_scene_inject_stall(bvhgpu_scene_t scene, int32_t on);

/* Synchronises `stream` and returns the first device-side error recorded by
 * this scene's kernels since the last call (and clears it). */
int bvhgpu_scene_status(bvhgpu_scene_t scene, void* stream);

/* Message for the last non-zero status returned on this thread. */
const char* bvhgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* BVHGPU_H */
