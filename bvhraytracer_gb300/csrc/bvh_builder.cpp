// SAH builder: restatement of the reference's Aabb::recursiveBvh.
// Float expressions keep the reference's evaluation order; this file must be
// compiled with -ffp-contract=off so x86-64 and aarch64 build the same tree.
#include "bvh_builder.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <thread>

#include "bvhgpu_status.hpp"

namespace bvhgpu {
namespace {

// glm::min / std::min and glm::max / std::max for floats.
inline float ref_min(float a, float b) { return (b < a) ? b : a; }
inline float ref_max(float a, float b) { return (a < b) ? b : a; }

// glmUtil.h:7-11 maxDimension (not on absolute values).
inline int max_dimension(const float v[3]) {
  return (v[0] > v[1]) ? ((v[0] > v[2]) ? 0 : 2) : ((v[1] > v[2]) ? 1 : 2);
}

struct Box {
  float lo[3], hi[3];
  // Aabb::calculateBounds starting values (aabb.h:116).
  void reset() {
    for (int i = 0; i < 3; ++i) { lo[i] = 222222.0f; hi[i] = -222222.0f; }
  }
  void grow(const Triangle& t) {
    for (int i = 0; i < 3; ++i) {
      lo[i] = ref_min(lo[i], t.bmin[i]);
      hi[i] = ref_max(hi[i], t.bmax[i]);
    }
  }
  // Aabb::getSurfaceArea (aabb.h:130-134).
  float area() const {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0f * (dx * dy + dx * dz + dy * dz);
  }
};

// Node::sah(invArea, leafTarget), step variant "c" (node.h:66-91).
inline float sah_step(size_t count, const Box& b, float inv_area, int leaf_target) {
  if (count != 0) {
    size_t steps = ((count - 1) / (size_t)leaf_target) + 1;
    return (float)steps * b.area() * inv_area * (float)leaf_target;
  }
  return b.area() * inv_area * 1.0f;
}

struct Builder {
  const BuildParams& p;
  std::vector<Triangle>& tris;
  std::vector<uint32_t>& prims;
  std::atomic<int> threads_left{0};

  Builder(const BuildParams& params, std::vector<Triangle>& t, std::vector<uint32_t>& pr)
      : p(params), tris(t), prims(pr) {
    unsigned hc = std::thread::hardware_concurrency();
    threads_left = hc > 1 ? (int)hc - 1 : 0;
  }

  bool center_less(uint32_t a, uint32_t b, int axis) const {
    return tris[a].center[axis] < tris[b].center[axis];
  }

  // chooseAxisAndSort (aabb.h:40-67).
  int choose_axis_and_sort(uint32_t begin, uint32_t end) {
    float mn[3] = {222222.0f, 222222.0f, 222222.0f};
    float mx[3] = {-222222.0f, -222222.0f, -222222.0f};
    for (uint32_t i = begin; i < end; ++i) {
      const float* c = tris[prims[i]].center;
      for (int k = 0; k < 3; ++k) { mn[k] = ref_min(mn[k], c[k]); mx[k] = ref_max(mx[k], c[k]); }
    }
    float d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    int axis = max_dimension(d);
    auto cmp = [&](uint32_t a, uint32_t b) { return center_less(a, b, axis); };
    if (!std::is_sorted(prims.begin() + begin, prims.begin() + end, cmp))
      std::stable_sort(prims.begin() + begin, prims.begin() + end, cmp);
    return axis;
  }

  // PrimIntervall::computerBestSplit[Sort] (aabb.cpp:4-69). The left sweep
  // keeps the reference's Node::sweepRight order: it advances the end
  // iterator and then reads the element at the new end, so after k steps the
  // left box holds primitives begin+1 .. begin+k while its count is k.
  uint32_t best_split(uint32_t begin, uint32_t end, bool sort, float inv_area, float& cost) {
    if (sort) choose_axis_and_sort(begin, end);
    size_t size = end - begin;
    std::vector<float> metric(size - 1, 0.0f);
    Box box;
    box.reset();
    for (size_t j = 0; j + 1 < size; ++j) {
      box.grow(tris[prims[begin + j + 1]]);
      metric[j] += sah_step(j + 1, box, inv_area, p.leaf_size);
    }
    box.reset();
    for (size_t jj = size - 1; jj-- > 0;) {
      box.grow(tris[prims[begin + jj + 1]]);
      metric[jj] += sah_step(size - 1 - jj, box, inv_area, p.leaf_size);
    }
    size_t best = 0;
    for (size_t j = 1; j < metric.size(); ++j)
      if (metric[j] < metric[best]) best = j;
    cost = metric[best];
    return begin + (uint32_t)best + 1;
  }

  void bounds_of(BuildNode& n) {
    Box b;
    b.reset();
    for (uint32_t i = n.begin; i < n.end; ++i) b.grow(tris[prims[i]]);
    for (int k = 0; k < 3; ++k) { n.bmin[k] = b.lo[k]; n.bmax[k] = b.hi[k]; }
  }

  // Aabb::recursiveBvh (aabb.cpp:71-206).
  void recurse(BuildNode& n) {
    const unsigned N = (unsigned)p.branching;
    const unsigned L = (unsigned)p.leaf_size;
    size_t count = n.end - n.begin;
    if (count <= L && (p.leaf_split_option == 0 || p.leaf_split_option == 2)) return;

    choose_axis_and_sort(n.begin, n.end);
    struct Interval { uint32_t b, e; size_t count() const { return e - b; } };
    std::vector<Interval> work{{n.begin, n.end}};
    int best_i = 0;
    Box nb;
    for (int k = 0; k < 3; ++k) { nb.lo[k] = n.bmin[k]; nb.hi[k] = n.bmax[k]; }
    float inv_area = 1 / nb.area();
    const bool sort = p.sort_each_split != 0;

    for (size_t b = 0; b < N - 1; ++b) {
      size_t prim_counter = 0;
      for (size_t i = 0; i < work.size(); ++i) {
        if (prim_counter < work[i].count()) { prim_counter = work[i].count(); best_i = (int)i; }
      }
      if (prim_counter <= L) break;
      float cost;
      uint32_t split = best_split(work[best_i].b, work[best_i].e, sort, inv_area, cost);
      Interval p2{split, work[best_i].e};
      work[best_i].e = split;
      work.insert(work.begin() + best_i + 1, p2);
    }
    if (p.leaf_split_option == 1 || p.leaf_split_option == 2) {
      for (size_t b = work.size() - 1; b < N - 1; ++b) {
        float best_imp = 0;
        int best_id = -1;
        uint32_t best_at = 0;
        for (size_t i = 0; i < work.size(); ++i) {
          int cnt = (int)work[i].count();
          if (cnt == 1) continue;
          float leaf_cost = (float)cnt;
          float split_cost = 0.f;
          uint32_t split = best_split(work[i].b, work[i].e, sort, inv_area, split_cost);
          split_cost += p.sah_factor;
          if (leaf_cost - split_cost > best_imp) {
            best_imp = leaf_cost - split_cost;
            best_id = (int)i;
            best_at = split;
          }
        }
        if (best_imp == 0) break;
        Interval p2{best_at, work[best_id].e};
        work[best_id].e = best_at;
        work.insert(work.begin() + best_id + 1, p2);
      }
    }
    if (work.size() == 1) return;  // leaf

    for (auto& iv : work) {
      auto c = std::make_unique<BuildNode>();
      c->begin = iv.b;
      c->end = iv.e;
      c->depth = (uint8_t)(n.depth + 1);
      bounds_of(*c);
      n.children.push_back(std::move(c));
    }
    if (sort) calc_traverse_order(n);
    n.begin = n.end;  // inner nodes keep no primitives

    // Node::recursiveBvh recurses children (par_unseq over disjoint ranges).
    std::vector<std::thread> pool;
    for (auto& c : n.children) {
      size_t cc = c->end - c->begin;
      if (cc > 20000 && threads_left.fetch_sub(1) > 0) {
        BuildNode* cp = c.get();
        pool.emplace_back([this, cp] { recurse(*cp); threads_left.fetch_add(1); });
      } else {
        if (cc > 20000) threads_left.fetch_add(1);
        recurse(*c);
      }
    }
    for (auto& t : pool) t.join();
  }

  // Node::calculateTraverseOrderEachAxis (node.cpp:254-275); the child centre
  // is Aabb::getCenter, (max + min) + 0.5 (aabb.h:142-146).
  void calc_traverse_order(BuildNode& n) {
    size_t c = n.children.size();
    for (int face = 0; face < 3; ++face) {
      std::vector<std::pair<float, int>> v;
      v.reserve(c);
      for (size_t i = 0; i < c; ++i) {
        float center = (n.children[i]->bmax[face] + n.children[i]->bmin[face]) + 0.5f;
        v.emplace_back(center, (int)i);
      }
      std::sort(v.begin(), v.end());
      n.order[face].clear();
      for (auto& t : v) n.order[face].push_back((int8_t)t.second);
    }
  }
};

void custom_tree_order(BuildNode* n, std::vector<BuildNode*>& out) {
  for (auto& c : n->children) out.push_back(c.get());
  for (auto& c : n->children) custom_tree_order(c.get(), out);
}

int stack_extra(const BuildNode* n) {
  if (n->children.empty()) return 0;
  int m = 0;
  for (auto& c : n->children) m = std::max(m, stack_extra(c.get()));
  return (int)n->children.size() - 1 + m;
}

}  // namespace

int Bvh::build(const float* tri9, uint64_t n_tris, const BuildParams& prm) {
  params = prm;
  if (prm.branching < 2 || prm.branching > 16) return BVHGPU_ERR_BAD_ARG;
  if (prm.leaf_size < 1 || prm.leaf_size > 16) return BVHGPU_ERR_BAD_ARG;
  if (prm.leaf_split_option < 0 || prm.leaf_split_option > 2) return BVHGPU_ERR_BAD_ARG;
  if (!prm.sort_each_split) return BVHGPU_ERR_UNSUPPORTED;  // traversal needs per-axis orders
  if (n_tris == 0 || tri9 == nullptr) return BVHGPU_ERR_BAD_ARG;
  if (n_tris > (1ull << 31)) return BVHGPU_ERR_BAD_ARG;

  tris.clear();
  tris.reserve(n_tris);
  for (uint64_t i = 0; i < n_tris; ++i) {
    Triangle t;
    for (int v = 0; v < 3; ++v)
      for (int k = 0; k < 3; ++k) t.p[v][k] = tri9[i * 9 + v * 3 + k];
    for (int k = 0; k < 3; ++k) {
      if (!std::isfinite(t.p[0][k]) || !std::isfinite(t.p[1][k]) || !std::isfinite(t.p[2][k]))
        return BVHGPU_ERR_BAD_ARG;
    }
    if (prm.drop_zero_area) {
      // calcTriangleSurfaceArea != 0 (glmUtil.h:57-62), glm::cross order.
      float ax = t.p[1][0] - t.p[0][0], ay = t.p[1][1] - t.p[0][1], az = t.p[1][2] - t.p[0][2];
      float bx = t.p[2][0] - t.p[0][0], by = t.p[2][1] - t.p[0][1], bz = t.p[2][2] - t.p[0][2];
      float cx = ay * bz - by * az, cy = az * bx - bz * ax, cz = ax * by - bx * ay;
      float dd = cx * cx + cy * cy + cz * cz;
      if (0.5f * std::sqrt(dd) == 0.0f) continue;
    }
    for (int k = 0; k < 3; ++k) {
      float mn = ref_min(t.p[0][k], t.p[1][k]);
      float mx = ref_max(t.p[0][k], t.p[1][k]);
      t.bmin[k] = ref_min(mn, t.p[2][k]);
      t.bmax[k] = ref_max(mx, t.p[2][k]);
      t.center[k] = t.bmax[k] * 0.5f + t.bmin[k] * 0.5f;
    }
    t.id = (uint32_t)i;
    tris.push_back(t);
  }
  if (tris.empty()) return BVHGPU_ERR_BAD_ARG;

  prims.resize(tris.size());
  for (size_t i = 0; i < prims.size(); ++i) prims[i] = (uint32_t)i;

  Builder b(params, tris, prims);
  // RayTracer::preparePrimitives sorts once before any build (rayTracer.cpp:747-754).
  b.choose_axis_and_sort(0, (uint32_t)prims.size());

  root = std::make_unique<BuildNode>();
  root->begin = 0;
  root->end = (uint32_t)prims.size();
  root->depth = 0;
  b.bounds_of(*root);
  b.recurse(*root);

  // Flatten in customTreeOrder (compactNode.cpp:27-28, 997-1008).
  node_ptr.clear();
  node_ptr.push_back(root.get());
  custom_tree_order(root.get(), node_ptr);
  nodes.assign(node_ptr.size(), CompactNode{});
  leaf_count = inner_count = 0;
  bvh_depth = 0;
  // Replay customTreeOrder: the children of a node receive consecutive ids at
  // the moment they are emitted, so the first-child id follows from a walk
  // with the same recursion.
  std::vector<uint32_t> first_child(node_ptr.size(), 0);
  struct Rec {
    static void run(const BuildNode* n, uint32_t& next, std::vector<uint32_t>& fc, uint32_t my_id) {
      uint32_t base = next;
      fc[my_id] = base;
      next += (uint32_t)n->children.size();
      for (size_t i = 0; i < n->children.size(); ++i)
        run(n->children[i].get(), next, fc, base + (uint32_t)i);
    }
  };
  uint32_t next_id = 1;
  Rec::run(root.get(), next_id, first_child, 0);
  for (size_t id = 0; id < node_ptr.size(); ++id) {
    BuildNode* n = node_ptr[id];
    CompactNode& c = nodes[id];
    for (int k = 0; k < 3; ++k) { c.bmin[k] = n->bmin[k]; c.bmax[k] = n->bmax[k]; }
    c.depth = n->depth;
    std::fill(&c.order[0][0], &c.order[0][0] + 48, (int8_t)0);
    if (!n->children.empty()) {
      c.child_begin = first_child[id];
      c.child_count = (uint32_t)n->children.size();
      c.prim_begin = 0;
      c.prim_count = 0;
      for (int a = 0; a < 3; ++a)
        for (size_t j = 0; j < n->order[a].size(); ++j) c.order[a][j] = n->order[a][j];
      ++inner_count;
    } else {
      c.child_begin = 0;
      c.child_count = 0;
      c.prim_begin = n->begin;
      c.prim_count = n->end - n->begin;
      ++leaf_count;
      bvh_depth = std::max(bvh_depth, (int)n->depth + 1);
    }
  }
  max_stack = 1 + stack_extra(root.get());
  return BVHGPU_OK;
}

int Bvh::import_compact(uint64_t n_nodes, const float* lo3, const float* hi3,
                        const uint32_t* child_begin, const uint32_t* child_count,
                        const uint32_t* prim_begin, const uint32_t* prim_count,
                        const int8_t* order48, uint64_t n_prims, const uint32_t* prim_ids,
                        const float* prim_tri9, int branching, int leaf_size) {
  if (!lo3 || !hi3 || !child_begin || !child_count || !prim_begin || !prim_count || !order48 ||
      !prim_ids || !prim_tri9)
    return BVHGPU_ERR_BAD_ARG;
  if (n_nodes == 0 || n_nodes > (1ull << 27) || n_prims == 0 || n_prims > (1ull << 31))
    return BVHGPU_ERR_BAD_ARG;
  if (branching < 2 || branching > 16 || leaf_size < 1 || leaf_size > 16) return BVHGPU_ERR_BAD_ARG;
  params = BuildParams();
  params.branching = branching;
  params.leaf_size = leaf_size;
  // Structure: children after their parent, in range, one parent each; leaf
  // ranges inside the primitive array; per-axis orders are permutations.
  std::vector<uint8_t> parents(n_nodes, 0);
  std::vector<uint8_t> depth(n_nodes, 0);
  for (uint64_t id = 0; id < n_nodes; ++id) {
    const uint32_t cc = child_count[id], pc = prim_count[id];
    if (cc > 0) {
      if (pc != 0 || cc < 1 || (int)cc > branching) return BVHGPU_ERR_BAD_ARG;
      const uint64_t cb = child_begin[id];
      if (cb <= id || cb + cc > n_nodes) return BVHGPU_ERR_BAD_ARG;
      for (int a = 0; a < 3; ++a) {
        uint32_t seen = 0;
        for (uint32_t i = 0; i < cc; ++i) {
          const int v = order48[id * 48 + a * 16 + i];
          if (v < 0 || (uint32_t)v >= cc || (seen >> v) & 1u) return BVHGPU_ERR_BAD_ARG;
          seen |= 1u << v;
        }
      }
      for (uint32_t j = 0; j < cc; ++j) {
        if (parents[cb + j]++) return BVHGPU_ERR_BAD_ARG;
        if (depth[id] >= 255) return BVHGPU_ERR_BAD_ARG;
        depth[cb + j] = (uint8_t)(depth[id] + 1);
      }
    } else {
      if (pc < 1 || (int)pc > leaf_size || (uint64_t)prim_begin[id] + pc > n_prims)
        return BVHGPU_ERR_BAD_ARG;
    }
  }
  for (uint64_t id = 1; id < n_nodes; ++id)
    if (parents[id] != 1) return BVHGPU_ERR_BAD_ARG;
  // Triangles in sorted order.
  tris.assign(n_prims, Triangle{});
  prims.resize(n_prims);
  for (uint64_t i = 0; i < n_prims; ++i) {
    Triangle& t = tris[i];
    for (int v = 0; v < 3; ++v)
      for (int k = 0; k < 3; ++k) {
        t.p[v][k] = prim_tri9[i * 9 + v * 3 + k];
        if (!std::isfinite(t.p[v][k])) return BVHGPU_ERR_BAD_ARG;
      }
    for (int k = 0; k < 3; ++k) {
      t.bmin[k] = std::min(std::min(t.p[0][k], t.p[1][k]), t.p[2][k]);
      t.bmax[k] = std::max(std::max(t.p[0][k], t.p[1][k]), t.p[2][k]);
      t.center[k] = t.bmax[k] * 0.5f + t.bmin[k] * 0.5f;
    }
    t.id = prim_ids[i];
    prims[i] = (uint32_t)i;
  }
  nodes.assign(n_nodes, CompactNode{});
  node_ptr.assign(n_nodes, nullptr);
  imported_.clear();
  imported_.reserve(n_nodes);
  root.reset();
  leaf_count = inner_count = 0;
  bvh_depth = 0;
  for (uint64_t id = 0; id < n_nodes; ++id) {
    CompactNode& c = nodes[id];
    for (int k = 0; k < 3; ++k) {
      c.bmin[k] = lo3[id * 3 + k];
      c.bmax[k] = hi3[id * 3 + k];
    }
    c.depth = depth[id];
    std::fill(&c.order[0][0], &c.order[0][0] + 48, (int8_t)0);
    auto bn = std::make_unique<BuildNode>();
    for (int k = 0; k < 3; ++k) {
      bn->bmin[k] = c.bmin[k];
      bn->bmax[k] = c.bmax[k];
    }
    bn->depth = c.depth;
    if (child_count[id] > 0) {
      c.child_begin = child_begin[id];
      c.child_count = child_count[id];
      for (int a = 0; a < 3; ++a)
        for (uint32_t i = 0; i < c.child_count; ++i) {
          c.order[a][i] = order48[id * 48 + a * 16 + i];
          bn->order[a].push_back(c.order[a][i]);
        }
      ++inner_count;
    } else {
      c.prim_begin = prim_begin[id];
      c.prim_count = prim_count[id];
      bn->begin = c.prim_begin;
      bn->end = c.prim_begin + c.prim_count;
      ++leaf_count;
      bvh_depth = std::max(bvh_depth, (int)c.depth + 1);
    }
    node_ptr[id] = bn.get();
    imported_.push_back(std::move(bn));
  }
  // Worst-case depth-first stack: 1 + max over root-to-leaf paths of the sum
  // of (children - 1); children are numbered after their parents.
  std::vector<int> extra(n_nodes, 0);
  for (uint64_t id = n_nodes; id-- > 0;) {
    if (child_count[id] == 0) continue;
    int m = 0;
    for (uint32_t j = 0; j < child_count[id]; ++j) m = std::max(m, extra[child_begin[id] + j]);
    extra[id] = (int)child_count[id] - 1 + m;
  }
  max_stack = 1 + extra[0];
  return BVHGPU_OK;
}

}  // namespace bvhgpu
