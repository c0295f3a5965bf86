// Driver around the reference's own instrumented renderer code —
// TEST INFRASTRUCTURE. Compiled only by oracle/ref/build_ref.py, together with
// the reference's sources (src/ray.cpp, src/primitives/triangle.cpp,
// src/accelerationStructure/{aabb,node,bvh,compactNode}.cpp), into
// oracle/_ref/libbvhref.so. Only tests/ and tests/golden/make_golden.py load
// it, to pin the oracle (oracle/bvh_oracle.c) and the CUDA kernels against the
// reference's results on the same triangles and rays.
//
// What it calls, in the reference's order (rayTracer.cpp:604-623, 711-716,
// 747-754; gameobject.h:110-146):
//   1. one Triangle per input triangle with its world-space points
//      (Triangle(gameObject, mesh, index, points), triangle.cpp:19-23) over a
//      Mesh holding those points as vertices, untextured, colour (1,1,1,1);
//      zero-area triangles are skipped as GameObject::iterateGo does;
//   2. chooseAxisAndSort over all primitives (aabb.h:40-67);
//   3. Bvh(primitives, N, L, sortEachSplit, leafSplitOption) and
//      Bvh::recursiveBvh(sahFactor) (bvh.cpp:28-40, aabb.cpp:71-206);
//   4. Bvh::bvhAnalysis with saving, performance test and images off
//      (bvh.cpp:337-364), which builds the NodeAnalysis tree;
//   5. CompactNodeManager<CompactNodeV3>(bvh, nodeOrder) (compactNode.cpp:11-104);
//   6. per ray Ray(pos, dir, bvh, shadow) (ray.cpp:4-35) with tMax set to the
//      given limit, then CompactNodeManager::intersectImmediately(ray,
//      useDistance) (compactNode.cpp:604-814), or intersectWideAlternative
//      over packets (compactNode.cpp:357-601).
// The hit primitive is observed by wrapping Triangle::intersect (a subclass
// that forwards to it and notes which triangle accepted the ray); nothing of
// the reference's arithmetic is replaced.
#include <cstdint>
#include <cstring>
#include <iostream>
#include <memory>
#include <sstream>
#include <unordered_map>
#include <vector>

#include "accelerationStructure/aabb.h"
#include "accelerationStructure/bvh.h"
#include "accelerationStructure/compactNode.h"
#include "accelerationStructure/nodeAnalysis.h"
#include "glmUtil.h"
#include "mesh.h"
#include "primitives/triangle.h"
#include "ray.h"

namespace {

// Last triangle that accepted each ray (keyed by the Ray's address, which is
// stable while a traversal runs).
thread_local std::unordered_map<const Ray*, int32_t>* g_hits = nullptr;

// Triangle that remembers its input index and reports accepting hits.
class TracedTriangle : public Triangle {
 public:
  TracedTriangle(const Mesh* mesh, int index, std::array<glm::vec3, 3> points, int32_t id)
      : Triangle(nullptr, mesh, index, points), id_(id) {}
  bool intersect(Ray& ray) override {
    const bool hit = Triangle::intersect(ray);
    if (hit && g_hits) (*g_hits)[&ray] = id_;
    return hit;
  }
  bool intersect(Node* node) override { return Triangle::intersect(node); }
  int32_t id() const { return id_; }

 private:
  int32_t id_;
};

struct Silence {  // the reference logs to std::cout while it builds
  std::streambuf* old;
  std::ostringstream sink;
  Silence() : old(std::cout.rdbuf(sink.rdbuf())) {}
  ~Silence() { std::cout.rdbuf(old); }
};

}  // namespace

struct bvhref {
  std::shared_ptr<Mesh> mesh;
  std::unique_ptr<Bvh> bvh;
  std::unique_ptr<CompactNodeManager<CompactNodeV3>> manager;
  std::vector<NodeAnalysis*> by_id;  // analysis node of each compact node id
  int depth = 0;
};

extern "C" {

// Builds the reference's BVH and CompactNodeManager over n triangles
// (tri9: n x 9 floats, world space). Returns 0 on success.
int bvhref_build(const float* tri9, uint64_t n, int32_t branching, int32_t leaf_size,
                 int32_t leaf_split_option, int32_t sort_each_split, float sah_factor,
                 int32_t node_order, bvhref** out) {
  if (!tri9 || !out || n == 0) return 1;
  Silence quiet;
  auto h = std::make_unique<bvhref>();
  auto verts = std::make_shared<std::vector<Vertex>>();
  auto idx = std::make_shared<std::vector<uint32_t>>();
  verts->reserve(n * 3);
  idx->reserve(n * 3);
  for (uint64_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      const float* p = tri9 + i * 9 + k * 3;
      verts->push_back(Vertex(glm::vec3(p[0], p[1], p[2]), glm::vec3(0, 1, 0), glm::vec2(0)));
      idx->push_back((uint32_t)(i * 3 + k));
    }
  h->mesh = std::make_shared<Mesh>(verts, idx, Color(1.f, 1.f, 1.f, 1.f), "input");
  primPointVector prims;
  for (uint64_t i = 0; i < n; ++i) {
    std::array<glm::vec3, 3> pts = {(*verts)[i * 3].pos, (*verts)[i * 3 + 1].pos,
                                     (*verts)[i * 3 + 2].pos};
    if (calcTriangleSurfaceArea(pts[0], pts[1], pts[2]) != 0)
      prims.push_back(std::make_shared<TracedTriangle>(h->mesh.get(), (int)(i * 3), pts, (int32_t)i));
  }
  if (prims.empty()) return 2;
  chooseAxisAndSort(prims.begin(), prims.end());
  h->bvh = std::make_unique<Bvh>(prims, branching, leaf_size, sort_each_split != 0,
                                 leaf_split_option);
  h->bvh->recursiveBvh(sah_factor);
  h->bvh->bvhAnalysis("", false, false, false, "ref", "", 1.f, 1.f, true);
  h->manager = std::make_unique<CompactNodeManager<CompactNodeV3>>(*h->bvh, node_order);
  // The manager numbered the analysis nodes (NodeAnalysis::id) in its order.
  std::vector<NodeAnalysis*> stack{h->bvh->getAnalysisRoot()};
  size_t count = 0;
  while (!stack.empty()) {
    NodeAnalysis* a = stack.back();
    stack.pop_back();
    ++count;
    if ((size_t)a->id >= h->by_id.size()) h->by_id.resize(a->id + 1, nullptr);
    h->by_id[a->id] = a;
    for (auto& c : a->children) stack.push_back(c.get());
  }
  if (count != h->by_id.size()) return 3;
  h->depth = h->bvh->bvhDepth;
  *out = h.release();
  return 0;
}

void bvhref_free(bvhref* h) { delete h; }

// Node count, primitive count (after zero-area removal), tree depth.
void bvhref_sizes(const bvhref* h, uint64_t* n_nodes, uint64_t* n_prims, int32_t* depth) {
  *n_nodes = h->by_id.size();
  *n_prims = h->bvh->primitives->size();
  *depth = h->depth;
}

// The CompactNodeV3 records in the manager's order, as the manager's
// constructor fills them (compactNode.cpp:77-102): bounds, first child id and
// child count (0 for a leaf), first primitive slot and primitive count, the
// three per-axis push sequences (order_stride entries each, -1 padded), depth;
// and prim_ids[slot] = input triangle index of each primitive slot.
void bvhref_export(const bvhref* h, float* lo3, float* hi3, uint32_t* child_begin,
                   uint32_t* child_count, uint32_t* prim_begin, uint32_t* prim_count,
                   int8_t* order, int32_t order_stride, uint32_t* depth, uint32_t* prim_ids) {
  const auto& prims = *h->bvh->primitives;
  for (size_t i = 0; i < h->by_id.size(); ++i) {
    const NodeAnalysis* a = h->by_id[i];
    const Aabb* box = static_cast<const Aabb*>(a->node);
    for (int k = 0; k < 3; ++k) {
      lo3[i * 3 + k] = box->boundMin[k];
      hi3[i * 3 + k] = box->boundMax[k];
    }
    child_begin[i] = a->children.empty() ? 0 : (uint32_t)a->children.front()->id;
    child_count[i] = (uint32_t)a->children.size();
    const size_t pc = a->node->getPrimCount();
    prim_begin[i] = pc ? (uint32_t)std::distance(h->bvh->primitives->begin(),
                                                 a->node->primitiveBegin) : 0;
    prim_count[i] = (uint32_t)pc;
    for (int ax = 0; ax < 3; ++ax)
      for (int k = 0; k < order_stride; ++k) {
        const auto& seq = a->node->traverseOrderEachAxis[ax];
        order[(i * 3 + ax) * order_stride + k] = k < (int)seq.size() ? seq[k] : (int8_t)-1;
      }
    depth[i] = a->depth;
  }
  for (size_t s = 0; s < prims.size(); ++s)
    prim_ids[s] = (uint32_t)static_cast<const TracedTriangle*>(prims[s].get())->id();
}

// Per ray (rays: n x 8 floats = origin, tMax, direction, unused):
//   prim[i]   input index of the triangle that last accepted the ray (-1: none);
//   t[i]      Ray::tMax after the traversal;
//   pos3/normal3  Ray::surfacePosition / surfaceNormal (closest-hit rays);
//   occluded[i]   the traversal's result (per ray: intersectImmediately's
//                 return value; ray stream: tMax set to NaN for shadow rays,
//                 a surface position for closest-hit rays);
//   counters[i*6..] nodes visited, leaves visited, box tests, box hits,
//                   triangle tests, triangle hits (Ray's counters);
// and summed over the rays: node and leaf visits per depth (hist, 2 x
// hist_len), childFullness (child_full, N + 1 entries) and primitiveFullness
// (prim_full, L + 1 entries). packet > 0: intersectWideAlternative over
// packets of that many consecutive rays instead of intersectImmediately per
// ray, with the per-step data of each packet in steps[packet][step][5] (node
// work, unique nodes, leaf work, unique leaves, terminations; step_cap steps
// at most) and step_count[packet].
int bvhref_trace(const bvhref* h, const float* rays, uint64_t n, int32_t shadow,
                 int32_t use_distance, int32_t packet, int32_t* prim, float* t, float* pos3,
                 float* normal3, uint8_t* occluded, uint32_t* counters, uint64_t* hist,
                 int32_t hist_len, uint64_t* child_full, uint64_t* prim_full, uint32_t* steps,
                 uint32_t* step_count, int32_t step_cap) {
  if (!h || (!rays && n)) return 1;
  const Bvh& bvh = *h->bvh;
  std::unordered_map<const Ray*, int32_t> hits;
  g_hits = &hits;
  auto make = [&](uint64_t i) {
    const float* r = rays + i * 8;
    Ray ray(glm::vec3(r[0], r[1], r[2]), glm::vec3(r[4], r[5], r[6]), bvh, shadow != 0);
    ray.tMax = r[3];
    return ray;
  };
  auto store = [&](uint64_t i, const Ray& ray, bool res) {
    auto it = hits.find(&ray);
    if (prim) prim[i] = it == hits.end() ? -1 : it->second;
    if (t) t[i] = ray.tMax;
    if (occluded) occluded[i] = res ? 1 : 0;
    for (int k = 0; k < 3; ++k) {
      if (pos3) pos3[i * 3 + k] = ray.surfacePosition[k];
      if (normal3) normal3[i * 3 + k] = ray.surfaceNormal[k];
    }
    if (counters) {
      uint32_t nodes = 0, leaves = 0;
      for (auto c : ray.nodeIntersectionCount) nodes += c;
      for (auto c : ray.leafIntersectionCount) leaves += c;
      uint32_t* c = counters + i * 6;
      c[0] = nodes;
      c[1] = leaves;
      c[2] = ray.aabbIntersectionCount;
      c[3] = ray.successfulAabbIntersectionCount;
      c[4] = ray.primitiveIntersectionCount;
      c[5] = ray.successfulPrimitiveIntersectionCount;
    }
    if (hist)
      for (size_t d = 0; d < ray.nodeIntersectionCount.size() && (int)d < hist_len; ++d) {
        hist[d] += ray.nodeIntersectionCount[d];
        hist[hist_len + d] += ray.leafIntersectionCount[d];
      }
    if (child_full)
      for (size_t k = 0; k < ray.childFullness.size(); ++k) child_full[k] += ray.childFullness[k];
    if (prim_full)
      for (size_t k = 0; k < ray.primitiveFullness.size(); ++k) prim_full[k] += ray.primitiveFullness[k];
  };
  if (packet <= 0) {
    for (uint64_t i = 0; i < n; ++i) {
      Ray ray = make(i);
      hits.clear();
      const bool res = h->manager->intersectImmediately(ray, use_distance != 0);
      store(i, ray, res);
    }
    g_hits = nullptr;
    return 0;
  }
  std::vector<uint32_t> a, b, c, d, e;
  for (uint64_t s = 0, pk = 0; s < n; s += (uint64_t)packet, ++pk) {
    const uint64_t m = std::min<uint64_t>((uint64_t)packet, n - s);
    std::vector<Ray> batch;
    batch.reserve(m);
    for (uint64_t i = 0; i < m; ++i) batch.push_back(make(s + i));
    hits.clear();
    a.clear(); b.clear(); c.clear(); d.clear(); e.clear();
    h->manager->intersectWideAlternative(batch, a, b, c, d, e);
    for (uint64_t i = 0; i < m; ++i) {
      const Ray& ray = batch[i];
      store(s + i, ray, shadow ? std::isnan(ray.tMax) : !std::isnan(ray.surfacePosition.x));
    }
    if (step_count) step_count[pk] = (uint32_t)a.size();
    if (steps)
      for (size_t k = 0; k < a.size() && (int)k < step_cap; ++k) {
        uint32_t* o = steps + (pk * (size_t)step_cap + k) * 5;
        o[0] = a[k]; o[1] = c[k]; o[2] = b[k]; o[3] = d[k]; o[4] = e[k];
      }
  }
  g_hits = nullptr;
  return 0;
}

}  // extern "C"
