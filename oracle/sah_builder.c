/*
 * SAH builder restated in plain C — TEST INFRASTRUCTURE ONLY.
 *
 * Builds the reference's BVH (CompactNodeManager<CompactNodeV3> records in
 * customTreeOrder) from world-space triangles, so that the CPU baseline and
 * the reference arm of bench.py need nothing from the product library. Only
 * tests/ and bench.py's CPU-baseline / reference legs use it; the tests
 * check it node for node against the product builder and, where the
 * reference's sources are present, against the reference's own builder.
 *
 * Follows, in this order:
 *   GameObject::iterateGo: zero-area triangles dropped ... gameobject.h:110-146
 *   Triangle bounds and centre max*0.5 + min*0.5 ........ triangle.cpp:41-50
 *   RayTracer::preparePrimitives: one initial sort ...... rayTracer.cpp:747-754
 *   chooseAxisAndSort (stable here; see below) .......... aabb.h:40-67
 *   Aabb::calculateBounds / getSurfaceArea .............. aabb.h:113-134
 *   Node::sah, step variant ............................. node.h:66-91
 *   PrimIntervall::computerBestSplitSort ................ aabb.cpp:4-69
 *     (the left sweep reads one element ahead: Node::sweepRight advances
 *     the end iterator before reading it, aabb.h:205-213)
 *   Aabb::recursiveBvh .................................. aabb.cpp:71-206
 *   Node::calculateTraverseOrderEachAxis with the child
 *     centre (max + min) + 0.5 .......................... node.cpp:254-275, aabb.h:142-146
 *   customTreeOrder ..................................... compactNode.cpp:997-1008
 *
 * The reference sorts with std::sort(par_unseq), which leaves triangles
 * with equal centres in an unspecified order; this builder (like the product
 * builder) uses a stable sort. Build: see oracle/build_oracle.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
  float p[3][3];
  float bmin[3], bmax[3], center[3];
  uint32_t id;
} stri_t;

typedef struct snode {
  uint32_t begin, end; /* primitive range (leaves) */
  float bmin[3], bmax[3];
  uint8_t depth;
  int n_children;
  struct snode* children[16];
  int8_t order[3][16];
} snode_t;

typedef struct {
  int branching, leaf_size, leaf_split_option;
  float sah_factor;
  stri_t* tris;
  uint32_t* prims;
  uint32_t* scratch; /* merge-sort buffer */
  int axis;          /* sort key of the current sort */
  size_t n_nodes;
} sbuild_t;

static inline float fmin_ref(float a, float b) { return (b < a) ? b : a; }
static inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }

/* glmUtil.h:7-11 maxDimension (not on absolute values). */
static int max_dimension(const float v[3]) {
  return (v[0] > v[1]) ? ((v[0] > v[2]) ? 0 : 2) : ((v[1] > v[2]) ? 1 : 2);
}

typedef struct { float lo[3], hi[3]; } sbox_t;

static void box_reset(sbox_t* b) {
  for (int i = 0; i < 3; ++i) { b->lo[i] = 222222.0f; b->hi[i] = -222222.0f; }
}
static void box_grow(sbox_t* b, const stri_t* t) {
  for (int i = 0; i < 3; ++i) {
    b->lo[i] = fmin_ref(b->lo[i], t->bmin[i]);
    b->hi[i] = fmax_ref(b->hi[i], t->bmax[i]);
  }
}
static float box_area(const sbox_t* b) {
  float dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
  return 2.0f * (dx * dy + dx * dz + dy * dz);
}

/* Node::sah(invArea, leafTarget), step variant. */
static float sah_step(size_t count, const sbox_t* b, float inv_area, int leaf_target) {
  if (count != 0) {
    size_t steps = ((count - 1) / (size_t)leaf_target) + 1;
    return (float)steps * box_area(b) * inv_area * (float)leaf_target;
  }
  return box_area(b) * inv_area * 1.0f;
}

/* Stable merge sort of prims[begin, end) by centre[axis]. */
static void msort(sbuild_t* s, uint32_t begin, uint32_t end) {
  if (end - begin < 2) return;
  uint32_t mid = begin + (end - begin) / 2;
  msort(s, begin, mid);
  msort(s, mid, end);
  const int ax = s->axis;
  if (!(s->tris[s->prims[mid]].center[ax] < s->tris[s->prims[mid - 1]].center[ax])) return;
  uint32_t i = begin, j = mid, k = 0;
  while (i < mid && j < end) {
    /* take from the right only when strictly smaller: stable */
    if (s->tris[s->prims[j]].center[ax] < s->tris[s->prims[i]].center[ax])
      s->scratch[k++] = s->prims[j++];
    else
      s->scratch[k++] = s->prims[i++];
  }
  while (i < mid) s->scratch[k++] = s->prims[i++];
  while (j < end) s->scratch[k++] = s->prims[j++];
  memcpy(s->prims + begin, s->scratch, sizeof(uint32_t) * k);
}

/* chooseAxisAndSort (aabb.h:40-67). */
static int choose_axis_and_sort(sbuild_t* s, uint32_t begin, uint32_t end) {
  float mn[3] = {222222.0f, 222222.0f, 222222.0f};
  float mx[3] = {-222222.0f, -222222.0f, -222222.0f};
  for (uint32_t i = begin; i < end; ++i) {
    const float* c = s->tris[s->prims[i]].center;
    for (int k = 0; k < 3; ++k) { mn[k] = fmin_ref(mn[k], c[k]); mx[k] = fmax_ref(mx[k], c[k]); }
  }
  float d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  int axis = max_dimension(d);
  int sorted = 1;
  for (uint32_t i = begin + 1; i < end && sorted; ++i)
    if (s->tris[s->prims[i]].center[axis] < s->tris[s->prims[i - 1]].center[axis]) sorted = 0;
  if (!sorted) {
    s->axis = axis;
    msort(s, begin, end);
  }
  return axis;
}

/* PrimIntervall::computerBestSplitSort (aabb.cpp:4-69). */
static uint32_t best_split(sbuild_t* s, uint32_t begin, uint32_t end, float inv_area,
                           float* cost, float* metric) {
  choose_axis_and_sort(s, begin, end);
  size_t size = end - begin;
  for (size_t j = 0; j + 1 < size; ++j) metric[j] = 0.0f;
  sbox_t box;
  box_reset(&box);
  for (size_t j = 0; j + 1 < size; ++j) {
    box_grow(&box, &s->tris[s->prims[begin + j + 1]]);
    metric[j] += sah_step(j + 1, &box, inv_area, s->leaf_size);
  }
  box_reset(&box);
  for (size_t jj = size - 1; jj-- > 0;) {
    box_grow(&box, &s->tris[s->prims[begin + jj + 1]]);
    metric[jj] += sah_step(size - 1 - jj, &box, inv_area, s->leaf_size);
  }
  size_t best = 0;
  for (size_t j = 1; j + 1 < size; ++j)
    if (metric[j] < metric[best]) best = j;
  *cost = metric[best];
  return begin + (uint32_t)best + 1;
}

static void bounds_of(sbuild_t* s, snode_t* n) {
  sbox_t b;
  box_reset(&b);
  for (uint32_t i = n->begin; i < n->end; ++i) box_grow(&b, &s->tris[s->prims[i]]);
  for (int k = 0; k < 3; ++k) { n->bmin[k] = b.lo[k]; n->bmax[k] = b.hi[k]; }
}

/* Node::calculateTraverseOrderEachAxis: children sorted by (centre, index). */
static void traverse_order(snode_t* n) {
  for (int face = 0; face < 3; ++face) {
    float key[16];
    int idx[16];
    for (int i = 0; i < n->n_children; ++i) {
      key[i] = (n->children[i]->bmax[face] + n->children[i]->bmin[face]) + 0.5f;
      idx[i] = i;
    }
    for (int i = 1; i < n->n_children; ++i) { /* insertion sort: lexicographic on (key, idx) */
      float k = key[i];
      int v = idx[i], j = i - 1;
      while (j >= 0 && (k < key[j] || (!(key[j] < k) && v < idx[j]))) {
        key[j + 1] = key[j];
        idx[j + 1] = idx[j];
        --j;
      }
      key[j + 1] = k;
      idx[j + 1] = v;
    }
    for (int i = 0; i < n->n_children; ++i) n->order[face][i] = (int8_t)idx[i];
  }
}

typedef struct { uint32_t b, e; } sint_t;

/* Aabb::recursiveBvh (aabb.cpp:71-206). Returns 0, or -1 when out of memory. */
static int recurse(sbuild_t* s, snode_t* n, float* metric) {
  const unsigned N = (unsigned)s->branching, L = (unsigned)s->leaf_size;
  size_t count = n->end - n->begin;
  if (count <= L && (s->leaf_split_option == 0 || s->leaf_split_option == 2)) return 0;
  choose_axis_and_sort(s, n->begin, n->end);
  sint_t work[16];
  int nw = 1;
  work[0].b = n->begin;
  work[0].e = n->end;
  int best_i = 0;
  sbox_t nb;
  for (int k = 0; k < 3; ++k) { nb.lo[k] = n->bmin[k]; nb.hi[k] = n->bmax[k]; }
  float inv_area = 1 / box_area(&nb);
  for (unsigned b = 0; b < N - 1; ++b) {
    size_t prim_counter = 0;
    for (int i = 0; i < nw; ++i)
      if (prim_counter < work[i].e - work[i].b) { prim_counter = work[i].e - work[i].b; best_i = i; }
    if (prim_counter <= L) break;
    float cost;
    uint32_t split = best_split(s, work[best_i].b, work[best_i].e, inv_area, &cost, metric);
    for (int i = nw; i > best_i + 1; --i) work[i] = work[i - 1];
    work[best_i + 1].b = split;
    work[best_i + 1].e = work[best_i].e;
    work[best_i].e = split;
    ++nw;
  }
  if (s->leaf_split_option == 1 || s->leaf_split_option == 2) {
    for (size_t b = (size_t)nw - 1; b < N - 1; ++b) {
      float best_imp = 0;
      int best_id = -1;
      uint32_t best_at = 0;
      for (int i = 0; i < nw; ++i) {
        int cnt = (int)(work[i].e - work[i].b);
        if (cnt == 1) continue;
        float leaf_cost = (float)cnt;
        float split_cost = 0.f;
        uint32_t split = best_split(s, work[i].b, work[i].e, inv_area, &split_cost, metric);
        split_cost += s->sah_factor;
        if (leaf_cost - split_cost > best_imp) {
          best_imp = leaf_cost - split_cost;
          best_id = i;
          best_at = split;
        }
      }
      if (best_imp == 0) break;
      for (int i = nw; i > best_id + 1; --i) work[i] = work[i - 1];
      work[best_id + 1].b = best_at;
      work[best_id + 1].e = work[best_id].e;
      work[best_id].e = best_at;
      ++nw;
    }
  }
  if (nw == 1) return 0; /* leaf */
  for (int i = 0; i < nw; ++i) {
    snode_t* c = (snode_t*)calloc(1, sizeof(snode_t));
    if (!c) return -1;
    c->begin = work[i].b;
    c->end = work[i].e;
    c->depth = (uint8_t)(n->depth + 1);
    bounds_of(s, c);
    n->children[n->n_children++] = c;
  }
  traverse_order(n);
  n->begin = n->end; /* inner nodes keep no primitives */
  s->n_nodes += (size_t)nw;
  for (int i = 0; i < n->n_children; ++i)
    if (recurse(s, n->children[i], metric)) return -1;
  return 0;
}

static void free_tree(snode_t* n) {
  for (int i = 0; i < n->n_children; ++i) free_tree(n->children[i]);
  free(n);
}

static int stack_extra(const snode_t* n) {
  if (n->n_children == 0) return 0;
  int m = 0;
  for (int i = 0; i < n->n_children; ++i) {
    int e = stack_extra(n->children[i]);
    if (e > m) m = e;
  }
  return n->n_children - 1 + m;
}

typedef struct {
  uint64_t n_nodes, n_prims;
  int32_t depth, max_stack;
  float *lo3, *hi3;
  uint32_t *child_begin, *child_count, *prim_begin, *prim_count;
  int8_t* order48;
  uint8_t* depth_of;
  uint32_t* prim_ids;
  float* prim_tri9;
} otree_t;

/* customTreeOrder: the children of a node receive consecutive ids when they
 * are emitted, then each child's subtree follows. */
static void emit(const snode_t* n, uint32_t my_id, uint32_t* next, snode_t** by_id,
                 uint32_t* first_child) {
  uint32_t base = *next;
  first_child[my_id] = base;
  *next += (uint32_t)n->n_children;
  for (int i = 0; i < n->n_children; ++i) by_id[base + (uint32_t)i] = n->children[i];
  for (int i = 0; i < n->n_children; ++i)
    emit(n->children[i], base + (uint32_t)i, next, by_id, first_child);
}

void oracle_tree_free(otree_t* t) {
  if (!t) return;
  free(t->lo3); free(t->hi3); free(t->child_begin); free(t->child_count);
  free(t->prim_begin); free(t->prim_count); free(t->order48); free(t->depth_of);
  free(t->prim_ids); free(t->prim_tri9);
  memset(t, 0, sizeof(*t));
}

/* Builds the tree of n triangles (tri9: n x 9 floats). Returns 0 on success,
 * 1 for bad arguments, 2 when no triangle has an area, -1 when out of memory. */
int oracle_build_tree(const float* tri9, uint64_t n, int32_t branching, int32_t leaf_size,
                      int32_t leaf_split_option, float sah_factor, otree_t* out) {
  if (!tri9 || !out || n == 0 || branching < 2 || branching > 16 || leaf_size < 1 ||
      leaf_size > 16 || leaf_split_option < 0 || leaf_split_option > 2)
    return 1;
  memset(out, 0, sizeof(*out));
  sbuild_t s;
  memset(&s, 0, sizeof(s));
  s.branching = branching;
  s.leaf_size = leaf_size;
  s.leaf_split_option = leaf_split_option;
  s.sah_factor = sah_factor;
  s.tris = (stri_t*)malloc(sizeof(stri_t) * n);
  if (!s.tris) return -1;
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i) {
    stri_t t;
    for (int v = 0; v < 3; ++v)
      for (int k = 0; k < 3; ++k) t.p[v][k] = tri9[i * 9 + v * 3 + k];
    /* calcTriangleSurfaceArea != 0 (glmUtil.h:57-62), glm::cross order */
    float ax = t.p[1][0] - t.p[0][0], ay = t.p[1][1] - t.p[0][1], az = t.p[1][2] - t.p[0][2];
    float bx = t.p[2][0] - t.p[0][0], by = t.p[2][1] - t.p[0][1], bz = t.p[2][2] - t.p[0][2];
    float cx = ay * bz - by * az, cy = az * bx - bz * ax, cz = ax * by - bx * ay;
    float dd = cx * cx + cy * cy + cz * cz;
    if (0.5f * sqrtf(dd) == 0.0f) continue;
    for (int k = 0; k < 3; ++k) {
      float mn = fmin_ref(t.p[0][k], t.p[1][k]), mx = fmax_ref(t.p[0][k], t.p[1][k]);
      t.bmin[k] = fmin_ref(mn, t.p[2][k]);
      t.bmax[k] = fmax_ref(mx, t.p[2][k]);
      t.center[k] = t.bmax[k] * 0.5f + t.bmin[k] * 0.5f;
    }
    t.id = (uint32_t)i;
    s.tris[m++] = t;
  }
  if (m == 0) { free(s.tris); return 2; }
  s.prims = (uint32_t*)malloc(sizeof(uint32_t) * m);
  s.scratch = (uint32_t*)malloc(sizeof(uint32_t) * m);
  float* metric = (float*)malloc(sizeof(float) * m);
  snode_t* root = (snode_t*)calloc(1, sizeof(snode_t));
  int rc = 0;
  if (!s.prims || !s.scratch || !metric || !root) rc = -1;
  if (!rc) {
    for (uint64_t i = 0; i < m; ++i) s.prims[i] = (uint32_t)i;
    choose_axis_and_sort(&s, 0, (uint32_t)m);
    root->begin = 0;
    root->end = (uint32_t)m;
    bounds_of(&s, root);
    s.n_nodes = 1;
    rc = recurse(&s, root, metric);
  }
  snode_t** by_id = NULL;
  uint32_t* first_child = NULL;
  if (!rc) {
    const size_t nn = s.n_nodes;
    by_id = (snode_t**)malloc(sizeof(snode_t*) * nn);
    first_child = (uint32_t*)calloc(nn, sizeof(uint32_t));
    out->lo3 = (float*)malloc(sizeof(float) * 3 * nn);
    out->hi3 = (float*)malloc(sizeof(float) * 3 * nn);
    out->child_begin = (uint32_t*)calloc(nn, 4);
    out->child_count = (uint32_t*)calloc(nn, 4);
    out->prim_begin = (uint32_t*)calloc(nn, 4);
    out->prim_count = (uint32_t*)calloc(nn, 4);
    out->order48 = (int8_t*)calloc(nn * 48, 1);
    out->depth_of = (uint8_t*)calloc(nn, 1);
    out->prim_ids = (uint32_t*)malloc(sizeof(uint32_t) * m);
    out->prim_tri9 = (float*)malloc(sizeof(float) * 9 * m);
    if (!by_id || !first_child || !out->lo3 || !out->hi3 || !out->child_begin ||
        !out->child_count || !out->prim_begin || !out->prim_count || !out->order48 ||
        !out->depth_of || !out->prim_ids || !out->prim_tri9)
      rc = -1;
  }
  if (!rc) {
    uint32_t next = 1;
    by_id[0] = root;
    emit(root, 0, &next, by_id, first_child);
    int depth = 0;
    for (size_t id = 0; id < s.n_nodes; ++id) {
      const snode_t* nd = by_id[id];
      for (int k = 0; k < 3; ++k) {
        out->lo3[id * 3 + k] = nd->bmin[k];
        out->hi3[id * 3 + k] = nd->bmax[k];
      }
      out->depth_of[id] = nd->depth;
      if (nd->n_children) {
        out->child_begin[id] = first_child[id];
        out->child_count[id] = (uint32_t)nd->n_children;
        for (int a = 0; a < 3; ++a)
          for (int j = 0; j < nd->n_children; ++j) out->order48[id * 48 + a * 16 + j] = nd->order[a][j];
      } else {
        out->prim_begin[id] = nd->begin;
        out->prim_count[id] = nd->end - nd->begin;
        if (nd->depth + 1 > depth) depth = nd->depth + 1;
      }
    }
    for (uint64_t i = 0; i < m; ++i) {
      const stri_t* t = &s.tris[s.prims[i]];
      out->prim_ids[i] = t->id;
      for (int v = 0; v < 3; ++v)
        for (int k = 0; k < 3; ++k) out->prim_tri9[i * 9 + v * 3 + k] = t->p[v][k];
    }
    out->n_nodes = s.n_nodes;
    out->n_prims = m;
    out->depth = depth;
    out->max_stack = 1 + stack_extra(root);
  } else {
    oracle_tree_free(out);
  }
  free(by_id);
  free(first_child);
  if (root) free_tree(root);
  free(metric);
  free(s.scratch);
  free(s.prims);
  free(s.tris);
  return rc;
}
