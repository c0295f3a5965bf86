// Flat exports of a built BVH (compile with -ffp-contract=off).
#include "bvh_export.hpp"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>

#include "bvhgpu_status.hpp"

namespace bvhgpu {

// ---------------------------------------------------------------------------
// FastNodeManager constructor (fastNodeManager.h:1495-1673).
int export_fast(const Bvh& bvh, int gang, int node_memory, int leaf_memory, FastView& out) {
  if (gang != 4 && gang != 8) return BVHGPU_ERR_BAD_ARG;
  if (node_memory < bvh.params.branching || node_memory % gang) return BVHGPU_ERR_BAD_ARG;
  if (leaf_memory < bvh.params.leaf_size || leaf_memory % gang) return BVHGPU_ERR_BAD_ARG;
  if (node_memory > 32) return BVHGPU_ERR_BAD_ARG;
  out.gang = gang;
  out.node_memory = node_memory;
  out.leaf_memory = leaf_memory;
  const size_t n = bvh.nodes.size();
  out.bounds.assign(n * 6 * node_memory, 0.0f);
  out.begin.assign(n, 0);
  out.order.assign(n * 3 * node_memory, 0);
  out.child_type.assign(n, 0);
  out.tri_points.clear();
  out.tri_points.reserve((size_t)bvh.leaf_count * leaf_memory * 9);
  const float qnan = std::numeric_limits<float>::quiet_NaN();

  for (size_t id = 0; id < n; ++id) {
    const CompactNode& c = bvh.nodes[id];
    const BuildNode* bn = bvh.node_ptr[id];
    float* bounds = &out.bounds[id * 6 * node_memory];
    if (c.child_count > 0) {
      int real = (((int)c.child_count - 1) / gang + 1) * gang;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < real; ++j)
          if (j < (int)c.child_count) bounds[i * real + j] = bvh.nodes[c.child_begin + j].bmin[i];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < real; ++j)
          if (j < (int)c.child_count)
            bounds[real * 3 + i * real + j] = bvh.nodes[c.child_begin + j].bmax[i];
      if (real != node_memory) {
        bounds[node_memory * 6 - 2] = (float)real;
        bounds[node_memory * 6 - 1] = qnan;
      }
      uint32_t type = 0;
      for (uint32_t j = 0; j < c.child_count; ++j)
        if (bvh.nodes[c.child_begin + j].child_count != 0) type |= 1u << j;
      out.child_type[id] = type;
      out.begin[id] = c.child_begin;
      for (int a = 0; a < 3; ++a)
        for (int i = 0; i < node_memory; ++i)
          out.order[(id * 3 + a) * node_memory + i] =
              (i < (int)bn->order[0].size()) ? bn->order[a][i] : (int8_t)0;
    }
    if (c.prim_count > 0) {
      if (c.prim_count > (uint32_t)leaf_memory) return BVHGPU_ERR_BAD_ARG;
      int real = (((int)c.prim_count - 1) / gang + 1) * gang;
      size_t p_begin = out.tri_points.size();
      size_t p_tmp = p_begin + real;
      for (int v = 0; v < 3; ++v) {
        for (int i = 0; i < 3; ++i) {
          for (uint32_t k = 0; k < c.prim_count; ++k)
            out.tri_points.push_back(bvh.tris[bvh.prims[c.prim_begin + k]].p[v][i]);
          out.tri_points.resize(p_tmp, 0.0f);
          p_tmp += real;
        }
      }
      out.tri_points.resize(p_begin + (size_t)leaf_memory * 9, 0.0f);
      if (real != leaf_memory) {
        out.tri_points[p_begin + leaf_memory * 9 - 2] = (float)real;
        out.tri_points[p_begin + leaf_memory * 9 - 1] = qnan;
      }
      bounds[0] = qnan;
      out.begin[id] = (uint32_t)p_begin;
    }
  }
  return BVHGPU_OK;
}

// ---------------------------------------------------------------------------
// Q8 helpers: power-of-two steps make q*step exact; the frame origin plus
// that offset is rounded down (lower bounds) or up (upper bounds), which the
// device reproduces with __fadd_rd / __fadd_ru.
namespace {

// a + b rounded toward -inf / +inf, via Knuth's TwoSum error term.
float add_round(float a, float b, bool up) {
  volatile float s = a + b;
  float bb = s - a;
  float err = (a - (s - bb)) + (b - bb);
  float r = s;
  if (up && err > 0.0f) r = std::nextafter(s, std::numeric_limits<float>::infinity());
  if (!up && err < 0.0f) r = std::nextafter(s, -std::numeric_limits<float>::infinity());
  return r;
}

float step_of(int e) { return std::ldexp(1.0f, e); }

}  // namespace

int build_device_layout(const Bvh& bvh, int gang, int leaf_memory, int node_format,
                        int top_levels, DeviceLayout& out) {
  const int N = bvh.params.branching;
  if (gang != 4 && gang != 8) return BVHGPU_ERR_BAD_ARG;
  if (leaf_memory == 0) leaf_memory = round_up(bvh.params.leaf_size, gang);
  if (leaf_memory < bvh.params.leaf_size || leaf_memory % gang || leaf_memory > 16)
    return BVHGPU_ERR_BAD_ARG;
  if (node_format != 0 && node_format != 1) return BVHGPU_ERR_BAD_ARG;
  if (top_levels < 0 || top_levels > 8) return BVHGPU_ERR_BAD_ARG;
  const int nm = round_up(N, 4);
  out.branching = N;
  out.node_stride = nm;
  out.leaf_memory = leaf_memory;
  out.gang = gang;
  out.node_format = node_format;
  out.record_bytes = node_format == 0 ? fp32_record_bytes(nm) : q8_record_bytes(nm);
  out.boxes_ordered = node_format == 0;

  const size_t n = bvh.nodes.size();
  // Leaf numbering: order of leaves in the reference's customTreeOrder.
  std::vector<int64_t> leaf_id(n, -1), inner_id(n, -1);
  uint32_t nl = 0;
  for (size_t id = 0; id < n; ++id)
    if (bvh.nodes[id].child_count == 0) leaf_id[id] = nl++;
  if (nl > kLeafIndexMask) return BVHGPU_ERR_UNSUPPORTED;

  // Inner numbering: level order for depth < top_levels, then customTreeOrder
  // below; siblings stay consecutive in both parts.
  std::vector<uint32_t> inner_order;
  uint32_t top = 0;
  if (bvh.nodes[0].child_count != 0) {
    std::vector<uint32_t> frontier{0};
    int level = 0;
    while (level < top_levels && !frontier.empty()) {
      std::vector<uint32_t> next;
      for (uint32_t f : frontier) {
        inner_order.push_back(f);
        const CompactNode& c = bvh.nodes[f];
        for (uint32_t j = 0; j < c.child_count; ++j)
          if (bvh.nodes[c.child_begin + j].child_count != 0) next.push_back(c.child_begin + j);
      }
      frontier.swap(next);
      ++level;
    }
    top = (uint32_t)inner_order.size();
    for (uint32_t f : frontier) inner_order.push_back(f);
    // customTreeOrder restricted to inner nodes below each frontier node.
    std::vector<uint32_t> work;
    struct Walk {
      static void run(const Bvh& b, uint32_t id, std::vector<uint32_t>& o) {
        const CompactNode& c = b.nodes[id];
        for (uint32_t j = 0; j < c.child_count; ++j)
          if (b.nodes[c.child_begin + j].child_count != 0) o.push_back(c.child_begin + j);
        for (uint32_t j = 0; j < c.child_count; ++j)
          if (b.nodes[c.child_begin + j].child_count != 0) run(b, c.child_begin + j, o);
      }
    };
    for (uint32_t f : frontier) Walk::run(bvh, f, inner_order);
  }
  for (size_t i = 0; i < inner_order.size(); ++i) inner_id[inner_order[i]] = (int64_t)i;
  out.n_inner = (uint32_t)inner_order.size();
  out.n_leaves = nl;
  out.top_nodes = top;

  auto entry_of = [&](uint32_t id) -> uint32_t {
    const CompactNode& c = bvh.nodes[id];
    if (c.child_count == 0)
      return kLeafBit | ((c.prim_count - 1) << kLeafCountShift) | (uint32_t)leaf_id[id];
    return (uint32_t)inner_id[id];
  };
  out.root_entry = entry_of(0);

  // Inner records.
  out.nodes.assign((size_t)out.n_inner * out.record_bytes, 0);
  const int pbytes = q8_perm_bytes(nm);
  if (node_format != 0) out.q8_perm.assign((size_t)out.n_inner * pbytes, 0);
  out.child_entry.assign((size_t)out.n_inner * nm, 0u);
  for (uint32_t g = 0; g < out.n_inner; ++g) {
    const uint32_t id = inner_order[g];
    const CompactNode& c = bvh.nodes[id];
    const BuildNode* bn = bvh.node_ptr[id];
    uint8_t* rec = &out.nodes[(size_t)g * out.record_bytes];
    uint32_t inner_base = 0, leaf_base = 0;
    bool have_inner = false, have_leaf = false;
    uint16_t leaf_mask = 0;
    for (uint32_t j = 0; j < c.child_count; ++j) {
      uint32_t ch = c.child_begin + j;
      if (bvh.nodes[ch].child_count == 0) {
        leaf_mask |= (uint16_t)(1u << j);
        if (!have_leaf) { leaf_base = (uint32_t)leaf_id[ch]; have_leaf = true; }
      } else if (!have_inner) {
        inner_base = (uint32_t)inner_id[ch];
        have_inner = true;
      }
    }
    for (uint32_t j = 0; j < c.child_count; ++j)
      out.child_entry[(size_t)g * nm + j] = entry_of(c.child_begin + j);
    // Sibling contiguity in both numberings.
    {
      uint32_t li = leaf_base, ii = inner_base;
      for (uint32_t j = 0; j < c.child_count; ++j) {
        uint32_t ch = c.child_begin + j;
        if (bvh.nodes[ch].child_count == 0) {
          if ((uint32_t)leaf_id[ch] != li++) return BVHGPU_ERR_UNSUPPORTED;
        } else if ((uint32_t)inner_id[ch] != ii++) {
          return BVHGPU_ERR_UNSUPPORTED;
        }
      }
    }
    uint8_t* meta;
    if (node_format == 0) {
      float* box = reinterpret_cast<float*>(rec);
      for (uint32_t j = 0; j < c.child_count; ++j) {
        const CompactNode& ch = bvh.nodes[c.child_begin + j];
        for (int k = 0; k < 3; ++k) {
          box[k * nm + j] = ch.bmin[k];
          box[(3 + k) * nm + j] = ch.bmax[k];
          if (!(std::isfinite(ch.bmin[k]) && std::isfinite(ch.bmax[k]) && ch.bmin[k] <= ch.bmax[k]))
            out.boxes_ordered = false;
        }
      }
      meta = rec + 24 * nm;
    } else {
      // Frame: this node's own box.
      float origin[3];
      int8_t ex[3];
      for (int k = 0; k < 3; ++k) {
        origin[k] = c.bmin[k];
        float ext = c.bmax[k] - c.bmin[k];
        int e = -126;
        if (ext > 0.0f) {
          int fe;
          std::frexp((double)ext / 255.0, &fe);  // ext/255 in [2^(fe-1), 2^fe)
          e = std::max(-126, fe - 1);
        }
        while (e < 127 && add_round(origin[k], 255.0f * step_of(e), true) < c.bmax[k]) ++e;
        ex[k] = (int8_t)e;
      }
      float* o = reinterpret_cast<float*>(rec);
      o[0] = origin[0];
      o[1] = origin[1];
      o[2] = origin[2];
      rec[12] = (uint8_t)ex[0];
      rec[13] = (uint8_t)ex[1];
      rec[14] = (uint8_t)ex[2];
      uint8_t* q = rec + q8_box_offset(nm);
      for (uint32_t j = 0; j < c.child_count; ++j) {
        const CompactNode& ch = bvh.nodes[c.child_begin + j];
        for (int k = 0; k < 3; ++k) {
          float step = step_of(ex[k]);
          double fl = std::floor(((double)ch.bmin[k] - (double)origin[k]) / (double)step);
          int ql = (int)std::min(255.0, std::max(0.0, fl));
          while (ql > 0 && add_round(origin[k], (float)ql * step, false) > ch.bmin[k]) --ql;
          while (ql < 255 && add_round(origin[k], (float)(ql + 1) * step, false) <= ch.bmin[k]) ++ql;
          double ce = std::ceil(((double)ch.bmax[k] - (double)origin[k]) / (double)step);
          int qh = (int)std::min(255.0, std::max(0.0, ce));
          while (qh < 255 && add_round(origin[k], (float)qh * step, true) < ch.bmax[k]) ++qh;
          while (qh > 0 && add_round(origin[k], (float)(qh - 1) * step, true) >= ch.bmax[k]) --qh;
          if (add_round(origin[k], (float)ql * step, false) > ch.bmin[k] ||
              add_round(origin[k], (float)qh * step, true) < ch.bmax[k])
            return BVHGPU_ERR_UNSUPPORTED;
          q[k * nm + j] = (uint8_t)ql;
          q[(3 + k) * nm + j] = (uint8_t)qh;
        }
      }
      meta = rec + 16;
    }
    std::memcpy(meta + 0, &inner_base, 4);
    std::memcpy(meta + 4, &leaf_base, 4);
    std::memcpy(meta + 8, &leaf_mask, 2);
    meta[10] = (uint8_t)c.child_count;
    meta[11] = c.depth;
    // Per axis: the push sequence of rays whose direction[axis] <= 0 (the
    // traverseOrderEachAxis order, one child per nibble) and its inverse
    // (the position of each child in it). The other direction pushes the
    // same children in the opposite order.
    const int wb = perm_word_bytes(nm);
    uint8_t* perm = node_format == 0 ? meta + 12 : &out.q8_perm[(size_t)g * pbytes];
    for (int a = 0; a < 3; ++a) {
      const size_t c_n = bn->order[a].size();
      uint64_t up = 0, inv = 0;
      for (size_t k = 0; k < c_n; ++k) {
        up |= (uint64_t)(uint8_t)bn->order[a][k] << (4 * k);
        inv |= (uint64_t)k << (4 * (uint8_t)bn->order[a][k]);
      }
      std::memcpy(perm + (a * 2 + 0) * wb, &up, wb);
      std::memcpy(perm + (a * 2 + 1) * wb, &inv, wb);
    }
    if (node_format == 0) {
      uint8_t* lcnt = meta + 12 + 6 * wb;
      for (uint32_t j = 0; j < c.child_count; ++j) {
        const CompactNode& ch = bvh.nodes[c.child_begin + j];
        lcnt[j] = ch.child_count == 0 ? (uint8_t)ch.prim_count : 0;
      }
    } else {
      uint8_t* nib = meta + 12;  // (count - 1) per leaf child, 4 bits
      for (uint32_t j = 0; j < c.child_count; ++j) {
        const CompactNode& ch = bvh.nodes[c.child_begin + j];
        if (ch.child_count == 0)
          nib[j / 2] |= (uint8_t)(((ch.prim_count - 1) & 15u) << (4 * (j & 1)));
      }
    }
  }

  // Leaf blocks: the reference's trianglePoints blocks, plus ids and depths.
  out.leaves.assign((size_t)nl * 9 * leaf_memory, 0.0f);
  out.leaf_prim.assign((size_t)nl * leaf_memory, 0xFFFFFFFFu);
  out.leaf_depth.assign(nl, 0);
  out.leaf_bounds.assign((size_t)nl * 6 * leaf_memory, 0.0f);
  const float qnan = std::numeric_limits<float>::quiet_NaN();
  for (size_t id = 0; id < n; ++id) {
    const CompactNode& c = bvh.nodes[id];
    if (c.child_count != 0) continue;
    if (c.prim_count > (uint32_t)leaf_memory) return BVHGPU_ERR_BAD_ARG;
    const size_t k = (size_t)leaf_id[id];
    float* blk = &out.leaves[k * 9 * leaf_memory];
    const int real = (((int)c.prim_count - 1) / gang + 1) * gang;
    for (uint32_t i = 0; i < c.prim_count; ++i) {
      const Triangle& t = bvh.tris[bvh.prims[c.prim_begin + i]];
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) blk[(v * 3 + a) * real + i] = t.p[v][a];
      out.leaf_prim[k * leaf_memory + i] = t.id;
      float* bnd = &out.leaf_bounds[k * 6 * leaf_memory];
      for (int a = 0; a < 3; ++a) {
        bnd[a * leaf_memory + i] = std::fmin(std::fmin(t.p[0][a], t.p[1][a]), t.p[2][a]);
        bnd[(3 + a) * leaf_memory + i] = std::fmax(std::fmax(t.p[0][a], t.p[1][a]), t.p[2][a]);
      }
    }
    if (real != leaf_memory) {
      blk[leaf_memory * 9 - 2] = (float)real;
      blk[leaf_memory * 9 - 1] = qnan;
    }
    out.leaf_depth[k] = c.depth;
  }
  return BVHGPU_OK;
}

// sahFactorConfigSse.txt:2-17 and RayTracer::loadSahFactor (rayTracer.cpp:880-925).
float sah_factor_sse(int branching, int leaf_size, int gang) {
  if (gang == 8) return 1.0f;  // the reference returns 1 for the AVX table
  // Float literals: the reference parses the text with std::stof, which
  // rounds the decimal straight to float.
  static const float table[4][4] = {
      {0.9790158394920848f, 0.6019200777645688f, 0.46148535855892625f, 0.38099865799955585f},
      {1.3129201663140904f, 0.8089449478051558f, 0.6356877674077516f, 0.5431092069456159f},
      {1.5611955563121058f, 0.9667477491937599f, 0.7477536713402126f, 0.638505587529224f},
      {1.8033700927282266f, 1.1369639789217003f, 0.8735301252614894f, 0.7655054621988963f}};
  int tn = (int)std::ceil(branching / (float)gang) * gang;
  int tl = (int)std::ceil(leaf_size / (float)gang) * gang;
  if (tn < 4 || tn > 16 || tl < 4 || tl > 16 || tn % 4 || tl % 4) return 1.0f;
  return table[tn / 4 - 1][tl / 4 - 1];
}

}  // namespace bvhgpu
