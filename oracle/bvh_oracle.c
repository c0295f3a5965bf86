/*
 * CPU oracle for the BVH traversal hot path — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
 * this file, and only to verify the GPU results or as the timed CPU baseline;
 * the product (libbvhgpu.so) never links or calls it.
 *
 * It restates, in plain C, the reference's (Hengoo/BVHRaytracer) scalar
 * algorithms for the path:
 *   instrumented profile (the reference's correctness renderer):
 *     Ray::Ray ............................ src/ray.cpp:4-36
 *     CompactNodeManager::aabbCheck ....... src/accelerationStructure/compactNode.h:247-278
 *     Triangle::intersect(Ray&) ........... src/primitives/triangle.cpp:52-249
 *     intersectImmediately (per ray) ...... src/accelerationStructure/compactNode.cpp:604-814
 *       (useDistance: pops whose box entry distance exceeds tMax are
 *       skipped, compactNode.cpp:623-645)
 *     intersectWideAlternative (stream) ... src/accelerationStructure/compactNode.cpp:357-601
 *   fast profile (the performance renderer, ISPC kernels with gang lanes):
 *     FastRay::FastRay .................... src/fastRay.cpp:3-20
 *     aabbIntersect{N} .................... src/ISPC/rayTracerTemplate.ispc:171-233
 *     triIntersect{L} / triAnyHit{L} ...... src/ISPC/rayTracerTemplate.ispc:26-168
 *     intersect / intersectSecondary ...... src/accelerationStructure/fastNodeManager.h:1328-1493
 *     intersectSaveDistance ............... fastNodeManager.h:1232-1326
 *     intersectWideAlternative /
 *     intersectSecondaryWideAlternative ... fastNodeManager.h:835-1230
 *   the ISPC kernels as single calls (oracle_*_calls) .. rayTracerTemplate.ispc:26-233
 *
 * Parity status of the instrumented profile: PINNED against the reference's
 * own code. oracle/ref/build_ref.py compiles the reference's SAH builder and
 * instrumented traversal (aabb.cpp, node.cpp, bvh.cpp, compactNode.cpp,
 * triangle.cpp, ray.cpp) here with g++ and a GLM stand-in; the tests compare
 * this restatement with it (trees node for node; hit triangle, t, hit point,
 * counters, per-depth and fullness histograms ray for ray) and with the
 * fixtures it generated (tests/golden/). The fast profile (the ISPC kernels
 * and FastNodeManager) needs the ISPC compiler, which is absent: it stays
 * checked against analytic known answers and hand-counted traversals.
 *
 * Deviations (both deliberate and documented):
 *   - the stream traversal of a tree whose root is a leaf tests that leaf
 *     (the reference's wide path would treat the root as an inner node);
 *   - fast-profile node tests cover only real children: the reference also
 *     slab-tests the zero padding boxes of a node, which matters only for
 *     rays through the exact world origin;
 *   - fast-profile stream traversal indexes the child order by the ray, not
 *     by the packet slot (fastNodeManager.h:913 uses rayMajorAxis[i]).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp (no FMA contraction,
 * IEEE float), see oracle/build_oracle.py.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAX_DEPTH 64
/* childFullness / primitiveFullness bins (Ray::childFullness[childCount],
 * ray.h:36-37): child or primitive counts 0..16. */
#define MAX_FULL 17

/* ---------------------------------------------------------------- views -- */
typedef struct {
  uint64_t n_nodes;
  const float* lo3;
  const float* hi3;
  const uint32_t* child_begin;
  const uint32_t* child_count;
  const uint32_t* prim_begin;
  const uint32_t* prim_count;
  const int8_t* order48; /* order[axis][i] at node*48 + axis*16 + i */
  const uint8_t* depth;
  const uint32_t* prim_ids;  /* sorted primitive -> input id */
  const float* prim_tri9;    /* sorted primitive points */
} oracle_compact_t;

typedef struct {
  uint64_t n_nodes;
  int32_t gang, node_memory, leaf_memory;
  const float* bounds;      /* n_nodes * 6 * node_memory */
  const uint32_t* begin;    /* childIdBegin / primIdBegin */
  const int8_t* order;      /* n_nodes * 3 * node_memory */
  const uint32_t* child_type;
  const float* tri_points;
} oracle_fast_t;

/* Ray input record: ox oy oz tmax dx dy dz pad (the bvhgpu_ray_t layout). */
typedef struct {
  float o[3], d[3], inv[3];
  float tmax;
  int code, reverse;
} oray_t;

/* Per-ray results: prim (input id or -1), t, u, v; counters[8]. */
typedef struct {
  int32_t prim;
  float t, u, v;
} ohit_t;

typedef struct {
  uint32_t node_visits, leaf_visits, box_tests, box_hits, tri_tests, tri_hits, max_stack, pad;
} octr_t;

static inline float rmin(float a, float b) { return (b < a) ? b : a; }
static inline float rmax(float a, float b) { return (a < b) ? b : a; }

/* maxAbsDimension (glmUtil.h:18-23). */
static inline int max_abs_dim(const float v[3]) {
  float x = fabsf(v[0]), y = fabsf(v[1]), z = fabsf(v[2]);
  return (x > y) ? ((x > z) ? 0 : 2) : ((y > z) ? 1 : 2);
}

/* Ray::Ray normalises (ray.cpp:12); FastRay keeps the direction as given. */
static void make_ray(const float* in, int normalise, oray_t* r) {
  float dx = in[4], dy = in[5], dz = in[6];
  r->o[0] = in[0]; r->o[1] = in[1]; r->o[2] = in[2];
  r->tmax = in[3];
  if (normalise) {
    volatile float dd = dx * dx + dy * dy + dz * dz;
    float s = 1.0f / sqrtf(dd);
    dx = dx * s; dy = dy * s; dz = dz * s;
  }
  r->d[0] = dx; r->d[1] = dy; r->d[2] = dz;
  r->inv[0] = 1.0f / dx; r->inv[1] = 1.0f / dy; r->inv[2] = 1.0f / dz;
  if (in[4] == 0) r->inv[0] = FLT_MAX;
  if (in[5] == 0) r->inv[1] = FLT_MAX;
  if (in[6] == 0) r->inv[2] = FLT_MAX;
  r->code = max_abs_dim(r->d);
  r->reverse = r->d[r->code] <= 0;
}

/* aabbCheck (compactNode.h:247-278) / one lane of aabbIntersect{N}. */
static int slab(const float lo[3], const float hi[3], const oray_t* r, float tmax) {
  float t0 = 0, t1 = tmax;
  for (int a = 0; a < 3; ++a) {
    float tn = (lo[a] - r->o[a]) * r->inv[a];
    float tf = (hi[a] - r->o[a]) * r->inv[a];
    if (tn > tf) { float t = tn; tn = tf; tf = t; }
    t0 = rmax(tn, t0);
    t1 = rmin(tf, t1);
  }
  return t0 <= t1;
}

/* aabbCheck(ray, id, distance) (compactNode.h:280-313) / aabbIntersect's
 * distances[] output: the same test, also returning the entry distance t0. */
static int slab_dist(const float lo[3], const float hi[3], const oray_t* r, float tmax,
                     float* dist) {
  float t0 = 0, t1 = tmax;
  for (int a = 0; a < 3; ++a) {
    float tn = (lo[a] - r->o[a]) * r->inv[a];
    float tf = (hi[a] - r->o[a]) * r->inv[a];
    if (tn > tf) { float t = tn; tn = tf; tf = t; }
    t0 = rmax(tn, t0);
    t1 = rmin(tf, t1);
  }
  *dist = t0;
  return t0 <= t1;
}

/* pbrt gamma(n), evaluated in double like MSVC does (util.h:13-17,44-48). */
static float gamma_n(int n) {
  double me = (double)FLT_EPSILON * 0.5;
  return (float)((n * me) / (1 - n * me));
}

/* Triangle::intersect(Ray&) (triangle.cpp:52-249) without its counters and
 * material lookup (the alpha test passes for opaque untextured meshes).
 * Returns 1 on a hit with *t, *b1, *b2. */
static int watertight_b0(const float* tri, const oray_t* r, float tmax, float* t_out,
                         float* b0_out, float* b1_out, float* b2_out) {
  const float* p0 = tri;
  const float* p1 = tri + 3;
  const float* p2 = tri + 6;
  /* box pre-test */
  float bmin[3], bmax[3];
  for (int a = 0; a < 3; ++a) {
    bmin[a] = rmin(rmin(p0[a], p1[a]), p2[a]);
    bmax[a] = rmax(rmax(p0[a], p1[a]), p2[a]);
  }
  float t1[3], t2[3], mn[3], mx[3];
  for (int a = 0; a < 3; ++a) {
    t1[a] = (bmin[a] - r->o[a]) * r->inv[a];
    t2[a] = (bmax[a] - r->o[a]) * r->inv[a];
    mn[a] = rmin(t1[a], t2[a]);
    mx[a] = rmax(t1[a], t2[a]);
  }
  float tmin = rmax(rmax(mn[0], mn[1]), mn[2]);
  float tmx = rmin(rmin(mx[0], mx[1]), mx[2]);
  if (tmx < 0) return 0;
  if (tmin > tmx) return 0;
  if (tmax < tmin) return 0;

  float p0t[3], p1t[3], p2t[3];
  for (int a = 0; a < 3; ++a) {
    p0t[a] = p0[a] - r->o[a];
    p1t[a] = p1[a] - r->o[a];
    p2t[a] = p2[a] - r->o[a];
  }
  float ad[3] = {fabsf(r->d[0]), fabsf(r->d[1]), fabsf(r->d[2])};
  int kz = (ad[0] > ad[1]) ? ((ad[0] > ad[2]) ? 0 : 2) : ((ad[1] > ad[2]) ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  float d[3] = {r->d[kx], r->d[ky], r->d[kz]};
  float q0[3] = {p0t[kx], p0t[ky], p0t[kz]};
  float q1[3] = {p1t[kx], p1t[ky], p1t[kz]};
  float q2[3] = {p2t[kx], p2t[ky], p2t[kz]};
  float sx = -d[0] / d[2];
  float sy = -d[1] / d[2];
  float sz = 1.f / d[2];
  q0[0] += sx * q0[2]; q0[1] += sy * q0[2];
  q1[0] += sx * q1[2]; q1[1] += sy * q1[2];
  q2[0] += sx * q2[2]; q2[1] += sy * q2[2];
  float e0 = q1[0] * q2[1] - q1[1] * q2[0];
  float e1 = q2[0] * q0[1] - q2[1] * q0[0];
  float e2 = q0[0] * q1[1] - q0[1] * q1[0];
  if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {
    double p2txp1ty = (double)q2[0] * (double)q1[1];
    double p2typ1tx = (double)q2[1] * (double)q1[0];
    e0 = (float)(p2typ1tx - p2txp1ty);
    double p0txp2ty = (double)q0[0] * (double)q2[1];
    double p0typ2tx = (double)q0[1] * (double)q2[0];
    e1 = (float)(p0typ2tx - p0txp2ty);
    double p1txp0ty = (double)q1[0] * (double)q0[1];
    double p1typ0tx = (double)q1[1] * (double)q0[0];
    e2 = (float)(p1typ0tx - p1txp0ty);
  }
  if ((e0 < 0 || e1 < 0 || e2 < 0) && (e0 > 0 || e1 > 0 || e2 > 0)) return 0;
  float det = e0 + e1 + e2;
  if (det == 0) return 0;
  q0[2] *= sz; q1[2] *= sz; q2[2] *= sz;
  float t_scaled = e0 * q0[2] + e1 * q1[2] + e2 * q2[2];
  if (det < 0 && (t_scaled >= 0 || t_scaled < tmax * det)) return 0;
  else if (det > 0 && (t_scaled <= 0 || t_scaled > tmax * det)) return 0;
  float inv_det = 1 / det;
  float b0 = e0 * inv_det;
  float b1 = e1 * inv_det;
  float b2 = e2 * inv_det;
  float t = t_scaled * inv_det;
  float max_zt = rmax(rmax(fabsf(q0[2]), fabsf(q1[2])), fabsf(q2[2]));
  float delta_z = gamma_n(3) * max_zt;
  float max_xt = rmax(rmax(fabsf(q0[0]), fabsf(q1[0])), fabsf(q2[0]));
  float max_yt = rmax(rmax(fabsf(q0[1]), fabsf(q1[1])), fabsf(q2[1]));
  float delta_x = gamma_n(5) * (max_xt + max_zt);
  float delta_y = gamma_n(5) * (max_yt + max_zt);
  float delta_e = 2 * (gamma_n(2) * max_xt * max_yt + delta_y * max_xt + delta_x * max_yt);
  float max_e = rmax(rmax(fabsf(e0), fabsf(e1)), fabsf(e2));
  float delta_t =
      3 * (gamma_n(3) * max_e * max_zt + delta_e * max_zt + delta_z * max_e) * fabsf(inv_det);
  if (t <= delta_t) return 0;
  *t_out = t;
  if (b0_out) *b0_out = b0;
  *b1_out = b1;
  *b2_out = b2;
  return 1;
}

static int watertight(const float* tri, const oray_t* r, float tmax, float* t_out, float* b1_out,
                      float* b2_out) {
  return watertight_b0(tri, r, tmax, t_out, NULL, b1_out, b2_out);
}

/* One lane of triIntersect{L} (rayTracerTemplate.ispc:35-76): p0/p1/p2 as
 * three-float points; the ray direction is used as given. */
static int moller_trumbore(const float p0[3], const float p1[3], const float p2[3],
                           const oray_t* r, float tmax, float* t_out, float* b1_out,
                           float* b2_out) {
  float e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  float e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  const float* dir = r->d;
  float s1[3] = {dir[1] * e2[2] - dir[2] * e2[1], dir[2] * e2[0] - dir[0] * e2[2],
                 dir[0] * e2[1] - dir[1] * e2[0]};
  float divisor = s1[0] * e1[0] + s1[1] * e1[1] + s1[2] * e1[2];
  int hit = 1;
  if (divisor == 0.) hit = 0;
  float inv_div = 1.f / divisor;
  float d[3] = {r->o[0] - p0[0], r->o[1] - p0[1], r->o[2] - p0[2]};
  float b1 = (d[0] * s1[0] + d[1] * s1[1] + d[2] * s1[2]) * inv_div;
  if (b1 < 0. || b1 > 1.) hit = 0;
  float s2[3] = {d[1] * e1[2] - d[2] * e1[1], d[2] * e1[0] - d[0] * e1[2],
                 d[0] * e1[1] - d[1] * e1[0]};
  float b2 = (dir[0] * s2[0] + dir[1] * s2[1] + dir[2] * s2[2]) * inv_div;
  if (b2 < 0. || b1 + b2 > 1.) hit = 0;
  float t = (e2[0] * s2[0] + e2[1] * s2[1] + e2[2] * s2[2]) * inv_div;
  if (t < 0 || t > tmax) hit = 0;
  *t_out = t;
  *b1_out = b1;
  *b2_out = b2;
  return hit;
}

/* ---------------------------------------------------- instrumented path -- */
typedef struct {
  oray_t r;
  int shadow;
  int alive;
  int32_t best_prim; /* sorted primitive index */
  float u, v;
  int hit;
  octr_t c;
  uint64_t* hist; /* [2][MAX_DEPTH], nullable */
  uint64_t* full; /* [2][MAX_FULL]: childFullness, primitiveFullness; nullable */
} ostate_t;

/* One leaf visit; returns 1 if any triangle was hit. */
static int leaf_visit(const oracle_compact_t* b, uint32_t id, ostate_t* s) {
  uint32_t pb = b->prim_begin[id], pc = b->prim_count[id];
  s->c.leaf_visits++;
  s->c.tri_tests += pc;
  if (s->hist) s->hist[MAX_DEPTH + (b->depth[id] < MAX_DEPTH ? b->depth[id] : MAX_DEPTH - 1)]++;
  /* ray.primitiveFullness[primCount]++ (compactNode.cpp:655) */
  if (s->full) s->full[MAX_FULL + (pc < MAX_FULL ? pc : MAX_FULL - 1)]++;
  int any = 0;
  for (uint32_t k = 0; k < pc; ++k) {
    float t, b1, b2;
    if (watertight(b->prim_tri9 + (size_t)(pb + k) * 9, &s->r, s->r.tmax, &t, &b1, &b2)) {
      s->c.tri_hits++;
      any = 1;
      if (!s->shadow) {
        s->r.tmax = t;
        s->best_prim = (int32_t)(pb + k);
        s->u = b1;
        s->v = b2;
      }
    }
  }
  return any;
}

/* Inner-node visit: test children in traverseOrderEachAxis order and push. */
static void node_visit(const oracle_compact_t* b, uint32_t id, ostate_t* s, int32_t* stack,
                       int* sp, int leaf_sign, float* dstack) {
  uint32_t cb = b->child_begin[id], cc = b->child_count[id];
  s->c.node_visits++;
  if (s->hist) s->hist[b->depth[id] < MAX_DEPTH ? b->depth[id] : MAX_DEPTH - 1]++;
  /* ray.childFullness[childCount]++ (compactNode.cpp:716) */
  if (s->full) s->full[cc < MAX_FULL ? cc : MAX_FULL - 1]++;
  const int8_t* ord = b->order48 + (size_t)id * 48 + s->r.code * 16;
  for (uint32_t k = 0; k < cc; ++k) {
    int i = s->r.reverse ? (int)k : (int)(cc - 1 - k);
    uint32_t ch = cb + (uint32_t)ord[i];
    s->c.box_tests++;
    float dist = 0;
    if (slab_dist(b->lo3 + (size_t)ch * 3, b->hi3 + (size_t)ch * 3, &s->r, s->r.tmax, &dist)) {
      s->c.box_hits++;
      int is_leaf = b->child_count[ch] == 0;
      if (dstack) dstack[*sp] = dist;
      stack[(*sp)++] = (leaf_sign && is_leaf) ? -(int32_t)ch : (int32_t)ch;
    }
  }
  if ((uint32_t)*sp > s->c.max_stack) s->c.max_stack = (uint32_t)*sp;
}

static void finish(const oracle_compact_t* b, const ostate_t* s, ohit_t* h, uint8_t* occ) {
  if (s->shadow) {
    if (occ) *occ = (uint8_t)(s->hit ? 1 : 0);
    return;
  }
  if (s->best_prim >= 0) {
    h->prim = (int32_t)b->prim_ids[s->best_prim];
    h->u = s->u;
    h->v = s->v;
  } else {
    h->prim = -1;
    h->u = 0;
    h->v = 0;
  }
  h->t = s->r.tmax;
}

static int stack_need(const oracle_compact_t* b) {
  /* Enough for any tree the builder makes: children of every node on a path. */
  (void)b;
  return 2048;
}

/* intersectImmediately(ray, useDistance) (compactNode.cpp:604-814). With
 * use_distance each stack entry carries its box's entry distance and a pop
 * whose distance exceeds the ray's current tMax is skipped uncounted
 * (compactNode.cpp:637-645); the root enters with distance 0. */
int oracle_trace_instrumented(const oracle_compact_t* b, const float* rays, uint64_t n, int shadow,
                              ohit_t* hits, uint8_t* occluded, octr_t* ctrs, uint64_t* hist,
                              int use_distance, uint64_t* fullness) {
  int cap = stack_need(b);
  int rc = 0;
#pragma omp parallel
  {
    int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
    float* dstack = use_distance ? (float*)malloc(sizeof(float) * (size_t)cap) : NULL;
    uint64_t* h = hist ? (uint64_t*)calloc(2 * MAX_DEPTH, sizeof(uint64_t)) : NULL;
    uint64_t* f = fullness ? (uint64_t*)calloc(2 * MAX_FULL, sizeof(uint64_t)) : NULL;
#pragma omp for schedule(dynamic, 64)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      ostate_t s;
      memset(&s, 0, sizeof(s));
      s.shadow = shadow;
      s.best_prim = -1;
      s.hist = h;
      s.full = f;
      make_ray(rays + i * 8, 1, &s.r);
      if (!isnan(rays[i * 8])) {
        int sp = 0;
        if (dstack) dstack[0] = 0;
        stack[sp++] = 0;
        while (sp > 0) {
          uint32_t id = (uint32_t)stack[--sp];
          if (dstack && dstack[sp] > s.r.tmax) continue;
          if (b->prim_count[id] != 0) {
            if (leaf_visit(b, id, &s)) {
              s.hit = 1;
              if (shadow) break;
            }
          }
          if (b->child_count[id] != 0) node_visit(b, id, &s, stack, &sp, 0, dstack);
          if (sp >= cap - 32) { rc = 4; break; }
        }
      }
      finish(b, &s, hits ? hits + i : NULL, occluded ? occluded + i : NULL);
      if (ctrs) ctrs[i] = s.c;
    }
    if (hist) {
#pragma omp critical
      for (int k = 0; k < 2 * MAX_DEPTH; ++k) hist[k] += h[k];
      free(h);
    }
    if (fullness) {
#pragma omp critical
      for (int k = 0; k < 2 * MAX_FULL; ++k) fullness[k] += f[k];
      free(f);
    }
    free(dstack);
    free(stack);
  }
  return rc;
}

/* intersectWideAlternative (compactNode.cpp:357-601) over packets of
 * `packet` consecutive rays. Per-ray results equal the per-ray traversal. */
static int cmp_i32(const void* x, const void* y) {
  int32_t a = *(const int32_t*)x, c = *(const int32_t*)y;
  return (a > c) - (a < c);
}

/* Number of distinct values among ids[0..k) (sorts ids). */
static uint32_t distinct(int32_t* ids, int k) {
  if (k == 0) return 0;
  qsort(ids, (size_t)k, sizeof(int32_t), cmp_i32);
  uint32_t d = 1;
  for (int i = 1; i < k; ++i) d += ids[i] != ids[i - 1];
  return d;
}

/* intersectWideAlternative with counters; with `steps`, also the per-step
 * data it collects for CameraData's workgroup analysis
 * (compactNode.cpp:357-601; wide_alt 0: the schedule of intersectWide,
 * compactNode.cpp:118-356, where a ray whose node visit leaves a leaf on
 * top visits that leaf in the same step's leaf loop): per packet p and step s, steps[(p * step_cap
 * + s) * 5 ..] = node work, unique nodes, leaf work, unique leaves,
 * terminations (step 0: the state before the loop, compactNode.cpp:410-415;
 * a root that is a leaf starts as leaf work), step_count[p] = steps used. */
static int stream_impl(const oracle_compact_t* b, const float* rays, uint64_t n, int shadow,
                       int packet, ohit_t* hits, uint8_t* occluded, octr_t* ctrs,
                       uint64_t* hist, int step_cap, uint32_t* steps, uint32_t* step_count,
                       int wide_alt, uint64_t* fullness) {
  int cap = stack_need(b);
  if (packet <= 0 || packet > 65535) return 1;
  int64_t npk = (int64_t)((n + (uint64_t)packet - 1) / (uint64_t)packet);
  int rc = 0;
#pragma omp parallel
  {
    int32_t* stacks = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap * (size_t)packet);
    int* sps = (int*)malloc(sizeof(int) * (size_t)packet);
    ostate_t* st = (ostate_t*)malloc(sizeof(ostate_t) * (size_t)packet);
    uint16_t* w1 = (uint16_t*)malloc(2 * (size_t)packet);
    uint16_t* w2 = (uint16_t*)malloc(2 * (size_t)packet);
    int32_t* ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)packet);
    uint16_t* ext = (uint16_t*)malloc(2 * (size_t)packet);
    uint64_t* h = hist ? (uint64_t*)calloc(2 * MAX_DEPTH, sizeof(uint64_t)) : NULL;
    uint64_t* f = fullness ? (uint64_t*)calloc(2 * MAX_FULL, sizeof(uint64_t)) : NULL;
#pragma omp for schedule(dynamic, 4)
    for (int64_t pk = 0; pk < npk; ++pk) {
      uint64_t first = (uint64_t)pk * (uint64_t)packet;
      int wide = (int)((n - first) < (uint64_t)packet ? (n - first) : (uint64_t)packet);
      uint16_t* cur = w1;
      uint16_t* nxt = w2;
      int node_rays = 0, leaf_rays = 0;
      int root_leaf = b->child_count[0] == 0;
      for (int j = 0; j < wide; ++j) {
        ostate_t* s = &st[j];
        memset(s, 0, sizeof(*s));
        s->shadow = shadow;
        s->best_prim = -1;
        s->hist = h;
        s->full = f;
        make_ray(rays + (first + (uint64_t)j) * 8, 1, &s->r);
        stacks[(size_t)j * cap] = root_leaf ? 0 : 0;
        sps[j] = 1;
        if (!isnan(rays[(first + (uint64_t)j) * 8])) {
          if (root_leaf) cur[wide - 1 - (leaf_rays++)] = (uint16_t)j;
          else cur[node_rays++] = (uint16_t)j;
        } else {
          sps[j] = 0;
        }
      }
      int next_node = 0, next_leaf = 0;
      int step = 1;
      if (steps && step_cap > 0) {
        uint32_t act = (uint32_t)(node_rays + leaf_rays);
        uint32_t* rec = steps + (size_t)pk * (size_t)step_cap * 5;
        rec[0] = root_leaf ? 0u : act;
        rec[1] = root_leaf ? 0u : 1u;
        rec[2] = root_leaf ? act : 0u;
        rec[3] = root_leaf ? (act ? 1u : 0u) : 0u;
        rec[4] = (uint32_t)wide - act;
      }
      while (node_rays != 0 || leaf_rays != 0) {
        uint32_t term = 0, un = 0, ul = 0;
        int n_ext = 0;
        for (int i = 0; i < node_rays; ++i) {
          int j = cur[i];
          ostate_t* s = &st[j];
          int32_t* stk = stacks + (size_t)j * cap;
          int32_t id = stk[--sps[j]];
          ids[i] = id;
          node_visit(b, (uint32_t)id, s, stk, &sps[j], 1, NULL);
          if (sps[j] >= cap - 32) rc = 4;
          if (sps[j] != 0) {
            if (stk[sps[j] - 1] >= 0) nxt[next_node++] = (uint16_t)j;
            else if (!wide_alt) ext[n_ext++] = (uint16_t)j;  /* intersectWide: leaf this step */
            else nxt[wide - 1 - (next_leaf++)] = (uint16_t)j;
          } else {
            term++;
          }
        }
        if (steps) un = distinct(ids, node_rays);
        for (int i = 0; i < leaf_rays + n_ext; ++i) {
          int j = i < leaf_rays ? cur[wide - 1 - i] : ext[i - leaf_rays];
          ostate_t* s = &st[j];
          int32_t* stk = stacks + (size_t)j * cap;
          int32_t id = -stk[--sps[j]];
          ids[i] = id;
          if (leaf_visit(b, (uint32_t)id, s)) {
            s->hit = 1;
            if (shadow) { sps[j] = 0; term++; continue; }
          }
          if (sps[j] != 0) {
            if (stk[sps[j] - 1] >= 0) nxt[next_node++] = (uint16_t)j;
            else nxt[wide - 1 - (next_leaf++)] = (uint16_t)j;
          } else {
            term++;
          }
        }
        if (steps) ul = distinct(ids, leaf_rays + n_ext);
        if (steps && step < step_cap) {
          uint32_t* rec = steps + ((size_t)pk * (size_t)step_cap + (size_t)step) * 5;
          rec[0] = (uint32_t)node_rays;
          rec[1] = un;
          rec[2] = (uint32_t)(leaf_rays + n_ext);
          rec[3] = ul;
          rec[4] = term;
        }
        ++step;
        leaf_rays = next_leaf;
        next_leaf = 0;
        node_rays = next_node;
        next_node = 0;
        uint16_t* t = cur; cur = nxt; nxt = t;
      }
      for (int j = 0; j < wide; ++j) {
        uint64_t i = first + (uint64_t)j;
        finish(b, &st[j], hits ? hits + i : NULL, occluded ? occluded + i : NULL);
        if (ctrs) ctrs[i] = st[j].c;
      }
      if (step_count) step_count[pk] = (uint32_t)step;
    }
    if (hist) {
#pragma omp critical
      for (int k = 0; k < 2 * MAX_DEPTH; ++k) hist[k] += h[k];
      free(h);
    }
    if (fullness) {
#pragma omp critical
      for (int k = 0; k < 2 * MAX_FULL; ++k) fullness[k] += f[k];
      free(f);
    }
    free(stacks); free(sps); free(st); free(w1); free(w2); free(ids); free(ext);
  }
  return rc;
}

int oracle_trace_instrumented_stream(const oracle_compact_t* b, const float* rays, uint64_t n,
                                     int shadow, int packet, ohit_t* hits, uint8_t* occluded,
                                     octr_t* ctrs, uint64_t* hist, uint64_t* fullness) {
  return stream_impl(b, rays, n, shadow, packet, hits, occluded, ctrs, hist, 0, NULL, NULL, 1,
                     fullness);
}

int oracle_trace_instrumented_stream_steps(const oracle_compact_t* b, const float* rays,
                                           uint64_t n, int shadow, int packet, ohit_t* hits,
                                           uint8_t* occluded, octr_t* ctrs, uint64_t* hist,
                                           int step_cap, uint32_t* steps, uint32_t* step_count,
                                           int wide_alternative, uint64_t* fullness) {
  return stream_impl(b, rays, n, shadow, packet, hits, occluded, ctrs, hist, step_cap, steps,
                     step_count, wide_alternative, fullness);
}

/* ------------------------------------------------------------ fast path -- */
/* Leaf loop count: the sentinel (stride, NaN) at the end of a block
 * (getLeafLoopCount, fastNodeManager.h:1728-1746). */
static int fast_leaf_stride(const oracle_fast_t* f, uint32_t begin) {
  if (f->leaf_memory == f->gang) return f->leaf_memory;
  const float* blk = f->tri_points + begin;
  int m = f->leaf_memory * 9;
  if (isnan(blk[m - 1])) return (int)blk[m - 2];
  return f->leaf_memory;
}

/* triIntersect{L} with gang lanes (rayTracerTemplate.ispc:28-108).
 * Returns the in-leaf index or -1; updates r->tmax; counts MT hits. */
static int tri_intersect(const oracle_fast_t* f, uint32_t begin, int stride, int real,
                         oray_t* r, float* u, float* v, octr_t* c) {
  float t_store[16];
  int orig[16];
  float us[16], vs[16];
  int gang = f->gang;
  int result = 0;
  for (int l = 0; l < gang; ++l) { t_store[l] = 1000000; orig[l] = -1; }
  const float* blk = f->tri_points + begin;
  const float tmax = r->tmax;
  for (int i = 0; i < stride; ++i) {
    int l = i % gang;
    float p0[3] = {blk[i], blk[i + stride], blk[i + stride * 2]};
    float p1[3] = {blk[i + stride * 3], blk[i + stride * 4], blk[i + stride * 5]};
    float p2[3] = {blk[i + stride * 6], blk[i + stride * 7], blk[i + stride * 8]};
    float t, b1, b2;
    int hit = moller_trumbore(p0, p1, p2, r, tmax, &t, &b1, &b2);
    if (hit && i < real && c) c->tri_hits++;
    if (hit) {
      if (t_store[l] > t) {
        result = 1;
        t_store[l] = t;
        orig[l] = i;
        us[l] = b1;
        vs[l] = b2;
      }
    }
  }
  if (!result) return -1;
  float best = t_store[0];
  for (int l = 1; l < gang; ++l) best = rmin(best, t_store[l]);
  int idx = -1, wl = -1;
  for (int l = 0; l < gang; ++l)
    if (t_store[l] == best && orig[l] > idx) { idx = orig[l]; wl = l; }
  r->tmax = best;
  *u = us[wl];
  *v = vs[wl];
  return idx;
}

static int tri_any_hit(const oracle_fast_t* f, uint32_t begin, int stride, int real,
                       const oray_t* r, octr_t* c) {
  const float* blk = f->tri_points + begin;
  int result = 0;
  for (int i = 0; i < stride; ++i) {
    float p0[3] = {blk[i], blk[i + stride], blk[i + stride * 2]};
    float p1[3] = {blk[i + stride * 3], blk[i + stride * 4], blk[i + stride * 5]};
    float p2[3] = {blk[i + stride * 6], blk[i + stride * 7], blk[i + stride * 8]};
    float t, b1, b2;
    if (moller_trumbore(p0, p1, p2, r, r->tmax, &t, &b1, &b2)) {
      result = 1;
      if (i < real && c) c->tri_hits++;
    }
  }
  return result;
}


#ifdef ORACLE_SIMD
/* ------------------------------------------- vectorised gang kernels -- */
/* The CPU baseline build (-DORACLE_SIMD -O3, oracle/build_oracle.py): the
 * ISPC kernels with their gang lanes as 4-wide GCC vectors (SSE on x86-64,
 * NEON on aarch64; the reference's SSE4 target has gang 4), each lane doing
 * exactly the scalar lane's float operations in the same order, so results
 * equal the scalar restatement's bit for bit. Used where the loop count is a
 * multiple of 4; the traversal loops around them are shared. */
typedef float v4f __attribute__((vector_size(16)));
typedef int32_t v4i __attribute__((vector_size(16)));

static inline v4f vld(const float* p) { v4f v; memcpy(&v, p, 16); return v; }
static inline v4f vsplat(float x) { v4f v = {x, x, x, x}; return v; }
static inline v4f vsel(v4i m, v4f a, v4f b) { /* m ? a : b */
  return (v4f)(((v4i)a & m) | ((v4i)b & ~m));
}
static inline v4i vseli(v4i m, v4i a, v4i b) { return (a & m) | (b & ~m); }
static inline int vany(v4i m) { return (m[0] | m[1] | m[2] | m[3]) != 0; }
static inline uint32_t vbits(v4i m) {
  return (uint32_t)((m[0] & 1) | (m[1] & 2) | (m[2] & 4) | (m[3] & 8));
}

/* Moller-Trumbore on 4 triangles (rows of a leaf block at column i). */
static inline v4i mt4(const float* blk, int i, int stride, const oray_t* r, float tmax,
                      v4f* t_out, v4f* b1_out, v4f* b2_out) {
  const v4f p0x = vld(blk + i), p0y = vld(blk + i + stride), p0z = vld(blk + i + stride * 2);
  const v4f p1x = vld(blk + i + stride * 3), p1y = vld(blk + i + stride * 4);
  const v4f p1z = vld(blk + i + stride * 5);
  const v4f p2x = vld(blk + i + stride * 6), p2y = vld(blk + i + stride * 7);
  const v4f p2z = vld(blk + i + stride * 8);
  const v4f d0 = vsplat(r->d[0]), d1 = vsplat(r->d[1]), d2 = vsplat(r->d[2]);
  const v4f e1x = p1x - p0x, e1y = p1y - p0y, e1z = p1z - p0z;
  const v4f e2x = p2x - p0x, e2y = p2y - p0y, e2z = p2z - p0z;
  const v4f s1x = d1 * e2z - d2 * e2y, s1y = d2 * e2x - d0 * e2z, s1z = d0 * e2y - d1 * e2x;
  const v4f divisor = s1x * e1x + s1y * e1y + s1z * e1z;
  v4i hit = ~(divisor == vsplat(0.f));
  const v4f inv_div = vsplat(1.f) / divisor;
  const v4f dx = vsplat(r->o[0]) - p0x, dy = vsplat(r->o[1]) - p0y, dz = vsplat(r->o[2]) - p0z;
  const v4f b1 = (dx * s1x + dy * s1y + dz * s1z) * inv_div;
  hit &= ~((b1 < vsplat(0.f)) | (b1 > vsplat(1.f)));
  const v4f s2x = dy * e1z - dz * e1y, s2y = dz * e1x - dx * e1z, s2z = dx * e1y - dy * e1x;
  const v4f b2 = (d0 * s2x + d1 * s2y + d2 * s2z) * inv_div;
  hit &= ~((b2 < vsplat(0.f)) | (b1 + b2 > vsplat(1.f)));
  const v4f t = (e2x * s2x + e2y * s2y + e2z * s2z) * inv_div;
  hit &= ~((t < vsplat(0.f)) | (t > vsplat(tmax)));
  *t_out = t;
  *b1_out = b1;
  *b2_out = b2;
  return hit;
}

static int tri_any_hit_v(const oracle_fast_t* f, uint32_t begin, int stride, int real,
                         const oray_t* r, octr_t* c) {
  const float* blk = f->tri_points + begin;
  v4i any = {0, 0, 0, 0};
  for (int i = 0; i < stride; i += 4) {
    v4f t, b1, b2;
    const v4i hit = mt4(blk, i, stride, r, r->tmax, &t, &b1, &b2);
    if (c) {
      const uint32_t bits = vbits(hit);
      for (int k = 0; k < 4; ++k)
        if ((bits >> k & 1u) && i + k < real) c->tri_hits++;
    }
    any |= hit;
  }
  return vany(any);
}

/* triIntersect{L}: lane i % gang keeps its first minimum below its running
 * value (rayTracerTemplate.ispc:28-101); gang 4 or 8 (one or two vectors of
 * lane state). */
static int tri_intersect_v(const oracle_fast_t* f, uint32_t begin, int stride, int real,
                           oray_t* r, float* u, float* v, octr_t* c) {
  const int gang = f->gang;
  v4f ts[2] = {vsplat(1000000.f), vsplat(1000000.f)};
  v4i orig[2] = {{-1, -1, -1, -1}, {-1, -1, -1, -1}};
  v4f us[2] = {vsplat(0.f), vsplat(0.f)}, vs[2] = {vsplat(0.f), vsplat(0.f)};
  v4i result = {0, 0, 0, 0};
  const float* blk = f->tri_points + begin;
  const float tmax = r->tmax;
  for (int i = 0; i < stride; i += 4) {
    const int g = (i % gang) / 4;
    v4f t, b1, b2;
    const v4i hit = mt4(blk, i, stride, r, tmax, &t, &b1, &b2);
    if (c) {
      const uint32_t bits = vbits(hit);
      for (int k = 0; k < 4; ++k)
        if ((bits >> k & 1u) && i + k < real) c->tri_hits++;
    }
    const v4i m = hit & (ts[g] > t);
    const v4i idx = {i, i + 1, i + 2, i + 3};
    ts[g] = vsel(m, t, ts[g]);
    orig[g] = vseli(m, idx, orig[g]);
    us[g] = vsel(m, b1, us[g]);
    vs[g] = vsel(m, b2, vs[g]);
    result |= m;
  }
  if (!vany(result)) return -1;
  float tl[8], ul[8], vl[8];
  int ol[8];
  for (int l = 0; l < gang; ++l) {
    tl[l] = ts[l / 4][l % 4];
    ol[l] = orig[l / 4][l % 4];
    ul[l] = us[l / 4][l % 4];
    vl[l] = vs[l / 4][l % 4];
  }
  float best = tl[0];
  for (int l = 1; l < gang; ++l) best = rmin(best, tl[l]);
  int idx = -1, wl = -1;
  for (int l = 0; l < gang; ++l)
    if (tl[l] == best && ol[l] > idx) { idx = ol[l]; wl = l; }
  r->tmax = best;
  *u = ul[wl];
  *v = vl[wl];
  return idx;
}

/* aabbIntersect over 4 children at a time; bits of the real children. */
static uint32_t aabb_intersect_v(const float* bd, int real, uint32_t cc, const oray_t* r,
                                 float* dist) {
  uint32_t mask = 0;
  const v4f ox = vsplat(r->o[0]), oy = vsplat(r->o[1]), oz = vsplat(r->o[2]);
  const v4f ix = vsplat(r->inv[0]), iy = vsplat(r->inv[1]), iz = vsplat(r->inv[2]);
  for (uint32_t j = 0; j < cc; j += 4) {
    v4f t0 = vsplat(0.f), t1 = vsplat(r->tmax);
    const v4f lo[3] = {vld(bd + j), vld(bd + j + real), vld(bd + j + real * 2)};
    const v4f hi[3] = {vld(bd + j + real * 3), vld(bd + j + real * 4),
                       vld(bd + j + real * 5)};
    const v4f o[3] = {ox, oy, oz}, inv[3] = {ix, iy, iz};
    for (int a = 0; a < 3; ++a) {
      v4f tn = (lo[a] - o[a]) * inv[a];
      v4f tf = (hi[a] - o[a]) * inv[a];
      const v4i sw = tn > tf;
      const v4f n2 = vsel(sw, tf, tn), f2 = vsel(sw, tn, tf);
      t0 = vsel(n2 < t0, t0, n2);   /* rmax(tn, t0) = (tn < t0) ? t0 : tn */
      t1 = vsel(t1 < f2, t1, f2);   /* rmin(tf, t1) = (t1 < tf) ? t1 : tf */
    }
    const uint32_t bits = vbits(t0 <= t1);
    for (uint32_t k = 0; k < 4 && j + k < cc; ++k) {
      if (bits >> k & 1u) {
        mask |= 1u << (j + k);
        if (dist) dist[j + k] = t0[k];
      }
    }
  }
  return mask;
}
#endif

/* aabbIntersect over the node's real children; bit j set if child j is hit. */
static uint32_t aabb_intersect(const oracle_fast_t* f, const oracle_compact_t* b, uint32_t id,
                               const oray_t* r, float* dist) {
  const float* bd = f->bounds + (size_t)id * 6 * f->node_memory;
  int real = f->node_memory;
  if (f->node_memory != f->gang && isnan(bd[f->node_memory * 6 - 1]))
    real = (int)bd[f->node_memory * 6 - 2];
  uint32_t cc = b->child_count[id];
#ifdef ORACLE_SIMD
  if (real % 4 == 0) return aabb_intersect_v(bd, real, cc, r, dist);
#endif
  uint32_t mask = 0;
  for (uint32_t j = 0; j < cc; ++j) {
    float lo[3] = {bd[j], bd[j + real], bd[j + real * 2]};
    float hi[3] = {bd[j + real * 3], bd[j + real * 4], bd[j + real * 5]};
    float t0 = 0;
    if (slab_dist(lo, hi, r, r->tmax, &t0)) {
      mask |= 1u << j;
      if (dist) dist[j] = t0;
    }
  }
  return mask;
}

typedef struct {
  oray_t r;
  int any;       /* any-hit ray */
  int hit;
  int32_t leaf_begin; /* primIdBegin float offset of the hit leaf */
  int lane;
  float u, v;
  octr_t c;
} fstate_t;

static void fast_leaf(const oracle_fast_t* f, const oracle_compact_t* b, uint32_t id,
                      fstate_t* s, uint64_t* hist) {
  uint32_t begin = f->begin[id];
  int stride = fast_leaf_stride(f, begin);
  int real = (int)b->prim_count[id];
  s->c.leaf_visits++;
  s->c.tri_tests += (uint32_t)real;
  if (hist) hist[MAX_DEPTH + (b->depth[id] < MAX_DEPTH ? b->depth[id] : MAX_DEPTH - 1)]++;
  if (s->any) {
#ifdef ORACLE_SIMD
    if (stride % 4 == 0) {
      if (tri_any_hit_v(f, begin, stride, real, &s->r, &s->c)) s->hit = 1;
      return;
    }
#endif
    if (tri_any_hit(f, begin, stride, real, &s->r, &s->c)) s->hit = 1;
  } else {
    float u, v;
#ifdef ORACLE_SIMD
    int idx = (stride % 4 == 0 && f->gang <= 8)
                  ? tri_intersect_v(f, begin, stride, real, &s->r, &u, &v, &s->c)
                  : tri_intersect(f, begin, stride, real, &s->r, &u, &v, &s->c);
#else
    int idx = tri_intersect(f, begin, stride, real, &s->r, &u, &v, &s->c);
#endif
    if (idx != -1) {
      s->hit = 1;
      s->leaf_begin = (int32_t)begin;
      s->lane = idx;
      s->u = u;
      s->v = v;
    }
  }
}

static void fast_node(const oracle_fast_t* f, const oracle_compact_t* b, uint32_t id,
                      fstate_t* s, int32_t* stack, int* sp, int leaf_sign, uint64_t* hist,
                      float* dstack) {
  float dist[16];
  uint32_t mask = aabb_intersect(f, b, id, &s->r, dist);
  uint32_t cc = b->child_count[id];
  uint32_t cbeg = f->begin[id];
  s->c.node_visits++;
  s->c.box_tests += cc;
  s->c.box_hits += (uint32_t)__builtin_popcount(mask);
  if (hist) hist[b->depth[id] < MAX_DEPTH ? b->depth[id] : MAX_DEPTH - 1]++;
  if (!mask) return;
  if (s->any) {
    for (uint32_t j = 0; j < cc; ++j)
      if (mask >> j & 1u) {
        int inner = (f->child_type[id] >> j) & 1u;
        if (dstack) dstack[*sp] = dist[j];
        stack[(*sp)++] = (leaf_sign && !inner) ? -(int32_t)(cbeg + j) : (int32_t)(cbeg + j);
      }
  } else {
    const int8_t* ord = f->order + ((size_t)id * 3 + (size_t)s->r.code) * f->node_memory;
    for (uint32_t k = 0; k < cc; ++k) {
      int i = s->r.reverse ? (int)k : (int)(cc - 1 - k);
      int j = ord[i];
      if (mask >> j & 1u) {
        int inner = (f->child_type[id] >> j) & 1u;
        if (dstack) dstack[*sp] = dist[j];
        stack[(*sp)++] = (leaf_sign && !inner) ? -(int32_t)(cbeg + j) : (int32_t)(cbeg + j);
      }
    }
  }
  if ((uint32_t)*sp > s->c.max_stack) s->c.max_stack = (uint32_t)*sp;
}

/* Per-leaf input ids for a fast hit: leaf_begin float offset -> leaf index. */
static int32_t fast_prim(const oracle_fast_t* f, const oracle_compact_t* b,
                         const uint32_t* leaf_node, int32_t leaf_begin, int lane) {
  uint32_t k = (uint32_t)leaf_begin / (uint32_t)(9 * f->leaf_memory);
  uint32_t id = leaf_node[k];
  return (int32_t)b->prim_ids[b->prim_begin[id] + (uint32_t)lane];
}

static void fast_finish(const oracle_fast_t* f, const oracle_compact_t* b, const uint32_t* ln,
                        const fstate_t* s, ohit_t* h, uint8_t* occ, int32_t* leaf_index,
                        int8_t* tri_index) {
  if (s->any) {
    if (occ) *occ = (uint8_t)s->hit;
    return;
  }
  if (h) {
    h->t = s->r.tmax;
    if (s->hit) {
      h->prim = fast_prim(f, b, ln, s->leaf_begin, s->lane);
      h->u = s->u;
      h->v = s->v;
    } else {
      h->prim = -1;
      h->u = 0;
      h->v = 0;
    }
  }
  if (leaf_index) *leaf_index = s->hit ? s->leaf_begin : -1;
  if (tri_index) *tri_index = (int8_t)(s->hit ? s->lane : -1);
}

static uint32_t* leaf_nodes(const oracle_fast_t* f, const oracle_compact_t* b) {
  (void)f;
  uint64_t nl = 0;
  for (uint64_t i = 0; i < b->n_nodes; ++i) nl += b->child_count[i] == 0;
  uint32_t* ln = (uint32_t*)malloc(sizeof(uint32_t) * (nl ? nl : 1));
  uint64_t k = 0;
  for (uint64_t i = 0; i < b->n_nodes; ++i)
    if (b->child_count[i] == 0) ln[k++] = (uint32_t)i;
  return ln;
}

/* FastNodeManager::intersect / intersectSecondary over n rays
 * (fastNodeManager.h:1328-1493), or, with packet > 0, the stream versions
 * intersectWideAlternative / intersectSecondaryWideAlternative over packets
 * of `packet` consecutive rays. threads <= 0: all available. use_distance
 * (per ray only): intersectSaveDistance (fastNodeManager.h:1232-1326), whose
 * stack entries carry aabbIntersect's t0 and whose pops with t0 > tMax are
 * skipped; the root enters with distance 0. */
int oracle_trace_fast(const oracle_fast_t* f, const oracle_compact_t* b, const float* rays,
                      uint64_t n, int any, int packet, int threads, ohit_t* hits,
                      uint8_t* occluded, int32_t* leaf_index, int8_t* tri_index, octr_t* ctrs,
                      uint64_t* hist, int use_distance) {
  const int cap = 2048;
  int rc = 0;
  uint32_t* ln = leaf_nodes(f, b);
#ifdef _OPENMP
  int nt = threads > 0 ? threads : omp_get_max_threads();
#else
  int nt = 1;
  (void)threads;
#endif
  if (packet <= 0) {
#pragma omp parallel num_threads(nt)
    {
      int32_t* stack = (int32_t*)malloc(sizeof(int32_t) * cap);
      float* dstack = use_distance ? (float*)malloc(sizeof(float) * cap) : NULL;
      uint64_t* h = hist ? (uint64_t*)calloc(2 * MAX_DEPTH, sizeof(uint64_t)) : NULL;
#pragma omp for schedule(dynamic, 64)
      for (int64_t i = 0; i < (int64_t)n; ++i) {
        fstate_t s;
        memset(&s, 0, sizeof(s));
        s.any = any;
        s.lane = -1;
        make_ray(rays + i * 8, 0, &s.r);
        if (!isnan(rays[i * 8])) {
          int sp = 0;
          if (dstack) dstack[0] = 0;
          stack[sp++] = 0;
          while (sp > 0) {
            uint32_t id = (uint32_t)stack[--sp];
            if (dstack && dstack[sp] > s.r.tmax) continue;
            if (b->child_count[id] == 0) {
              fast_leaf(f, b, id, &s, h);
              if (any && s.hit) break;
            } else {
              fast_node(f, b, id, &s, stack, &sp, 0, h, dstack);
            }
            if (sp >= cap - 32) { rc = 4; break; }
          }
        }
        fast_finish(f, b, ln, &s, hits ? hits + i : NULL, occluded ? occluded + i : NULL,
                    leaf_index ? leaf_index + i : NULL, tri_index ? tri_index + i : NULL);
        if (ctrs) ctrs[i] = s.c;
      }
      if (hist) {
#pragma omp critical
        for (int k = 0; k < 2 * MAX_DEPTH; ++k) hist[k] += h[k];
        free(h);
      }
      free(dstack);
      free(stack);
    }
  } else {
    if (use_distance) { free(ln); return 1; }
    int64_t npk = (int64_t)((n + (uint64_t)packet - 1) / (uint64_t)packet);
#pragma omp parallel num_threads(nt)
    {
      int32_t* stacks = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap * (size_t)packet);
      int* sps = (int*)malloc(sizeof(int) * (size_t)packet);
      fstate_t* st = (fstate_t*)malloc(sizeof(fstate_t) * (size_t)packet);
      uint16_t* w1 = (uint16_t*)malloc(2 * (size_t)packet);
      uint16_t* w2 = (uint16_t*)malloc(2 * (size_t)packet);
      uint64_t* h = hist ? (uint64_t*)calloc(2 * MAX_DEPTH, sizeof(uint64_t)) : NULL;
#pragma omp for schedule(dynamic, 4)
      for (int64_t pk = 0; pk < npk; ++pk) {
        uint64_t first = (uint64_t)pk * (uint64_t)packet;
        int wide = (int)((n - first) < (uint64_t)packet ? (n - first) : (uint64_t)packet);
        uint16_t* cur = w1;
        uint16_t* nxt = w2;
        int node_rays = 0, leaf_rays = 0;
        int root_leaf = b->child_count[0] == 0;
        for (int j = 0; j < wide; ++j) {
          fstate_t* s = &st[j];
          memset(s, 0, sizeof(*s));
          s->any = any;
          s->lane = -1;
          make_ray(rays + (first + (uint64_t)j) * 8, 0, &s->r);
          stacks[(size_t)j * cap] = 0;
          sps[j] = 1;
          if (!isnan(rays[(first + (uint64_t)j) * 8])) {
            if (root_leaf) cur[wide - 1 - (leaf_rays++)] = (uint16_t)j;
            else cur[node_rays++] = (uint16_t)j;
          } else {
            sps[j] = 0;
          }
        }
        int next_node = 0, next_leaf = 0;
        while (node_rays != 0 || leaf_rays != 0) {
          for (int i = 0; i < node_rays; ++i) {
            int j = cur[i];
            int32_t* stk = stacks + (size_t)j * cap;
            int32_t id = stk[--sps[j]];
            fast_node(f, b, (uint32_t)id, &st[j], stk, &sps[j], 1, h, NULL);
            if (sps[j] != 0) {
              if (stk[sps[j] - 1] >= 0 && !(stk[sps[j] - 1] == 0 && root_leaf))
                nxt[next_node++] = (uint16_t)j;
              else
                nxt[wide - 1 - (next_leaf++)] = (uint16_t)j;
            }
          }
          for (int i = 0; i < leaf_rays; ++i) {
            int j = cur[wide - 1 - i];
            int32_t* stk = stacks + (size_t)j * cap;
            int32_t id = -stk[--sps[j]];
            fast_leaf(f, b, (uint32_t)id, &st[j], h);
            if (any && st[j].hit) { sps[j] = 0; continue; }
            if (sps[j] != 0) {
              if (stk[sps[j] - 1] >= 0) nxt[next_node++] = (uint16_t)j;
              else nxt[wide - 1 - (next_leaf++)] = (uint16_t)j;
            }
          }
          leaf_rays = next_leaf;
          next_leaf = 0;
          node_rays = next_node;
          next_node = 0;
          uint16_t* t = cur; cur = nxt; nxt = t;
        }
        for (int j = 0; j < wide; ++j) {
          uint64_t i = first + (uint64_t)j;
          fast_finish(f, b, ln, &st[j], hits ? hits + i : NULL, occluded ? occluded + i : NULL,
                      leaf_index ? leaf_index + i : NULL, tri_index ? tri_index + i : NULL);
          if (ctrs) ctrs[i] = st[j].c;
        }
      }
      if (hist) {
#pragma omp critical
        for (int k = 0; k < 2 * MAX_DEPTH; ++k) hist[k] += h[k];
        free(h);
      }
      free(stacks); free(sps); free(st); free(w1); free(w2);
    }
  }
  free(ln);
  return rc;
}

/* ----------------------------------------------------------- FP64 check -- */
/* Double-precision Moller-Trumbore of each (ray, triangle) pair, for the
 * error statement of float results: out[i] = {t, b1, b2} (NaN when the
 * pair does not intersect in double). normalise: 1 to normalise the
 * direction first (instrumented profile). */
void oracle_fp64_pairs(const float* rays, const float* tri9, uint64_t n, int normalise,
                       double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    const float* r = rays + i * 8;
    const float* t = tri9 + i * 9;
    double o[3] = {r[0], r[1], r[2]}, d[3] = {r[4], r[5], r[6]};
    if (normalise) {
      /* The float-normalised direction is the ray the float path traces. */
      float dx = r[4], dy = r[5], dz = r[6];
      volatile float dd = dx * dx + dy * dy + dz * dz;
      float s = 1.0f / sqrtf(dd);
      d[0] = (double)(dx * s); d[1] = (double)(dy * s); d[2] = (double)(dz * s);
    }
    double p0[3] = {t[0], t[1], t[2]}, p1[3] = {t[3], t[4], t[5]}, p2[3] = {t[6], t[7], t[8]};
    double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    double s1[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2],
                    d[0] * e2[1] - d[1] * e2[0]};
    double div = s1[0] * e1[0] + s1[1] * e1[1] + s1[2] * e1[2];
    double* o3 = out + i * 3;
    if (div == 0.0) { o3[0] = o3[1] = o3[2] = NAN; continue; }
    double inv = 1.0 / div;
    double dd[3] = {o[0] - p0[0], o[1] - p0[1], o[2] - p0[2]};
    double b1 = (dd[0] * s1[0] + dd[1] * s1[1] + dd[2] * s1[2]) * inv;
    double s2[3] = {dd[1] * e1[2] - dd[2] * e1[1], dd[2] * e1[0] - dd[0] * e1[2],
                    dd[0] * e1[1] - dd[1] * e1[0]};
    double b2 = (d[0] * s2[0] + d[1] * s2[1] + d[2] * s2[2]) * inv;
    double tt = (e2[0] * s2[0] + e2[1] * s2[1] + e2[2] * s2[2]) * inv;
    o3[0] = tt;
    o3[1] = b1;
    o3[2] = b2;
  }
}

/* The instrumented profile's hit point of each (ray, triangle) pair:
 * Triangle::intersect's pHit = b0 * p0 + b1 * p1 + b2 * p2 (triangle.cpp:201,
 * glm vec3 operations, left to right), which the reference stores as
 * Ray::surfacePosition. Recomputes the watertight test for the given triangle
 * (its barycentrics do not depend on tMax); pairs it does not hit get NaN. */
void oracle_hit_points(const float* rays, const float* tri9, uint64_t n, float* out_pos) {
  for (uint64_t i = 0; i < n; ++i) {
    oray_t r;
    make_ray(rays + i * 8, 1, &r);
    const float* p = tri9 + i * 9;
    float t, b0, b1, b2;
    float* o = out_pos + i * 3;
    if (!watertight_b0(p, &r, INFINITY, &t, &b0, &b1, &b2)) {
      o[0] = o[1] = o[2] = NAN;
      continue;
    }
    for (int a = 0; a < 3; ++a) {
      float x = b0 * p[a];
      float y = b1 * p[3 + a];
      float z = b2 * p[6 + a];
      o[a] = (x + y) + z;
    }
  }
}

/* --------------------------------------------- ISPC calls, one by one -- */
/* The reference's exported ISPC kernels as independent calls, for the
 * batched GPU entry points. FastRay records (10 floats: tMax, pos[3],
 * invDirection[3], direction[3]; fastRay.h:14-29) are used as given: the
 * slab test reads invDirection, Moller-Trumbore reads pos and direction.
 * Rows are `width` long (padding 1, raytracerTemplateGen.py:10). */
static void fastray_state(const float* fr, oray_t* r) {
  r->tmax = fr[0];
  for (int a = 0; a < 3; ++a) {
    r->o[a] = fr[1 + a];
    r->inv[a] = fr[4 + a];
    r->d[a] = fr[7 + a];
  }
  r->code = max_abs_dim(r->d);
  r->reverse = r->d[r->code] <= 0;
}

/* aabbIntersect{N} (rayTracerTemplate.ispc:171-233) over all `n` lanes of
 * bounds + offset[i]: distances[i * n + lane] = t0 for each hit lane (other
 * entries untouched), result[i] = 1 if any lane is hit. */
void oracle_aabb_intersect_calls(int32_t n, const float* bounds, const uint32_t* offset,
                                 const float* fastrays, float* distances, uint8_t* result,
                                 uint64_t count) {
  for (uint64_t i = 0; i < count; ++i) {
    oray_t r;
    fastray_state(fastrays + i * 10, &r);
    const float* bd = bounds + offset[i];
    int any = 0;
    for (int j = 0; j < n; ++j) {
      float lo[3] = {bd[j], bd[j + n], bd[j + n * 2]};
      float hi[3] = {bd[j + n * 3], bd[j + n * 4], bd[j + n * 5]};
      float t0 = 0;
      if (slab_dist(lo, hi, &r, r.tmax, &t0)) {
        any = 1;
        distances[i * n + j] = t0;
      }
    }
    result[i] = (uint8_t)any;
  }
}

/* triIntersect{L} (rayTracerTemplate.ispc:28-108) on the leaf block at
 * tri + tri_id[i] with `l` lanes of a `gang`-wide ISPC gang: result[i] = the
 * in-leaf index of the hit (or -1); a hit lowers fastrays[i * 10] (tMax). */
void oracle_tri_intersect_calls(int32_t l, int32_t gang, const float* tri,
                                const uint32_t* tri_id, float* fastrays, int32_t* result,
                                uint64_t count) {
  oracle_fast_t f;
  memset(&f, 0, sizeof f);
  f.gang = gang;
  f.leaf_memory = l;
  f.tri_points = tri;
  for (uint64_t i = 0; i < count; ++i) {
    oray_t r;
    fastray_state(fastrays + i * 10, &r);
    float u, v;
    result[i] = tri_intersect(&f, tri_id[i], l, l, &r, &u, &v, NULL);
    fastrays[i * 10] = r.tmax;
  }
}

/* triAnyHit{L} (rayTracerTemplate.ispc:112-168): result[i] = 1 if any of
 * the `l` triangles at tri + tri_id[i] is hit within tMax. */
void oracle_tri_any_hit_calls(int32_t l, const float* tri, const uint32_t* tri_id,
                              const float* fastrays, uint8_t* result, uint64_t count) {
  oracle_fast_t f;
  memset(&f, 0, sizeof f);
  f.gang = 4;
  f.leaf_memory = l;
  f.tri_points = tri;
  for (uint64_t i = 0; i < count; ++i) {
    oray_t r;
    fastray_state(fastrays + i * 10, &r);
    result[i] = (uint8_t)tri_any_hit(&f, tri_id[i], l, l, &r, NULL);
  }
}

int oracle_abi_version(void) { return 1; }
