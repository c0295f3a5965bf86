// Adjoint of the leaf intersection: gradients of (t, b1, b2) of each ray's
// closest hit with respect to the three triangle vertices and the ray origin
// and direction, through a fixed visibility set.
//
// adjoint_kernel re-traces each ray (per-ray depth-first, fast profile, so
// the hit is the forward pass's); adjoint_hits_kernel takes the forward
// pass's stored hits instead. Both then run the reverse pass of the
// Moller-Trumbore expressions of triIntersect{L}
// (rayTracerTemplate.ispc:35-76):
//   e1 = p1 - p0, e2 = p2 - p0, s1 = d x e2, div = s1.e1, inv = 1/div,
//   s = o - p0, b1 = (s.s1) inv, s2 = s x e1, b2 = (d.s2) inv,
//   t = (e2.s2) inv.
// The reverse pass runs in double-float arithmetic (pairs of floats, see
// below), so the FP32 gradients it returns are the correctly rounded values
// of a ~48-bit evaluation even for grazing rays, where a float evaluation of
// s1.e1 cancels. Vertex gradients are summed per triangle within each warp,
// then added with atomics per triangle (9 floats, scattered to shared
// vertices by the caller) or per vertex through the face indices.
#include "adjoint.cuh"

namespace bvhgpu {
namespace dev {

// ---- double-float arithmetic -------------------------------------------
// A value is an unevaluated sum hi + lo of two floats (about 48 significant
// bits). Error-free transformations: Knuth's TwoSum, Dekker's TwoProduct by
// fused multiply-add; df_add / df_mul / df_recip follow the double-double
// algorithms of Hida, Li and Bailey (2001) with float components. The kernels
// are compiled without FMA contraction, so the compensations are not folded.
struct df {
  float hi, lo;
};

BVHGPU_DEV df df_of(float a) { return df{a, 0.f}; }
BVHGPU_DEV df quick_two_sum(float a, float b) {
  const float s = a + b;
  return df{s, b - (s - a)};
}
BVHGPU_DEV df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return df{s, (a - (s - bb)) + (b - bb)};
}
BVHGPU_DEV df two_prod(float a, float b) {
  const float p = a * b;
  return df{p, __fmaf_rn(a, b, -p)};
}
BVHGPU_DEV df df_add(df x, df y) {
  df s = two_sum(x.hi, y.hi);
  const df t = two_sum(x.lo, y.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}
BVHGPU_DEV df df_neg(df x) { return df{-x.hi, -x.lo}; }
BVHGPU_DEV df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
BVHGPU_DEV df df_mul(df x, df y) {
  df p = two_prod(x.hi, y.hi);
  p.lo += x.hi * y.lo + x.lo * y.hi;
  return quick_two_sum(p.hi, p.lo);
}
BVHGPU_DEV df df_recip(df x) {
  // One Newton step from the float reciprocal: r + r (1 - x r).
  const float r = 1.f / x.hi;
  const df e = df_sub(df_of(1.f), df_mul(x, df_of(r)));
  return df_add(df_of(r), df_mul(df_of(r), e));
}
BVHGPU_DEV float df_float(df x) { return x.hi + x.lo; }

struct df3 {
  df x, y, z;
};
BVHGPU_DEV df3 d3(df x, df y, df z) { return df3{x, y, z}; }
BVHGPU_DEV df3 d3f(float x, float y, float z) { return df3{df_of(x), df_of(y), df_of(z)}; }
// a - b of float vectors, exact.
BVHGPU_DEV df3 sub3f(float3 a, float3 b) {
  return df3{two_sum(a.x, -b.x), two_sum(a.y, -b.y), two_sum(a.z, -b.z)};
}
BVHGPU_DEV df3 add3(df3 a, df3 b) { return d3(df_add(a.x, b.x), df_add(a.y, b.y), df_add(a.z, b.z)); }
BVHGPU_DEV df3 mul3(df3 a, df s) { return d3(df_mul(a.x, s), df_mul(a.y, s), df_mul(a.z, s)); }
BVHGPU_DEV df dot3(df3 a, df3 b) {
  return df_add(df_add(df_mul(a.x, b.x), df_mul(a.y, b.y)), df_mul(a.z, b.z));
}
BVHGPU_DEV df3 cross3(df3 a, df3 b) {
  return d3(df_sub(df_mul(a.y, b.z), df_mul(a.z, b.y)), df_sub(df_mul(a.z, b.x), df_mul(a.x, b.z)),
            df_sub(df_mul(a.x, b.y), df_mul(a.y, b.x)));
}
BVHGPU_DEV float3 to_f3(df3 a) { return make_float3(df_float(a.x), df_float(a.y), df_float(a.z)); }

// Gradients of one hit triangle's three vertices (dL/dp0, dL/dp1, dL/dp2).
struct TriGrad {
  float v[9];
};

// Reverse pass for ray rid whose closest hit is lane `i` of leaf `leaf`:
// writes the ray gradients and returns the vertex gradients.
BVHGPU_DEV TriGrad adjoint_reverse(const SceneDev& sc, const AdjointArgs& a, uint64_t rid,
                                   const bvhgpu_ray_t& in, uint32_t leaf, int i) {
  float* gr = a.grad_rays + rid * 8;
  // Vertices of the hit triangle from its leaf block (original axes).
  const float* blk = sc.leaves + (size_t)leaf * 9 * sc.leaf_memory;
  // Stride = leaf count rounded up to the gang: recover it from the sentinel.
  int stride_l = sc.leaf_memory;
  {
    const float last = blk[sc.leaf_memory * 9 - 1];
    if (isnan(last)) stride_l = (int)blk[sc.leaf_memory * 9 - 2];
  }
  const float3 p0 = make_float3(blk[0 * stride_l + i], blk[1 * stride_l + i], blk[2 * stride_l + i]);
  const float3 p1 = make_float3(blk[3 * stride_l + i], blk[4 * stride_l + i], blk[5 * stride_l + i]);
  const float3 p2 = make_float3(blk[6 * stride_l + i], blk[7 * stride_l + i], blk[8 * stride_l + i]);
  // The fast profile's ray: origin and direction as given (FastRay).
  const float3 of = make_float3(in.ox, in.oy, in.oz);
  const df3 d = d3f(in.dx, in.dy, in.dz);

  // Forward intermediates in double-float: the differences of float inputs
  // are exact, so a grazing ray (small s1.e1) loses no bits to cancellation
  // before the reverse pass divides by it.
  const df3 e1 = sub3f(p1, p0), e2 = sub3f(p2, p0);
  const df3 s1 = cross3(d, e2);
  const df div = dot3(s1, e1);
  const df inv = df_recip(div);
  const df3 s = sub3f(of, p0);
  const df n1 = dot3(s, s1);
  const df3 s2 = cross3(s, e1);
  const df n2 = dot3(d, s2);
  const df n3 = dot3(e2, s2);

  // Reverse pass.
  float4 g;
  if (a.grad_hits) {
    g = a.grad_hits[rid];
  } else {
    // Separate per-ray arrays dL/dt, dL/du, dL/dv (null: zero).
    g = make_float4(0.f, a.grad_t ? __ldg(a.grad_t + rid) : 0.f,
                    a.grad_u ? __ldg(a.grad_u + rid) : 0.f, a.grad_v ? __ldg(a.grad_v + rid) : 0.f);
  }
  const df gt = df_of(g.y), gb1 = df_of(g.z), gb2 = df_of(g.w);
  const df g_n1 = df_mul(gb1, inv), g_n2 = df_mul(gb2, inv), g_n3 = df_mul(gt, inv);
  const df g_inv = df_add(df_add(df_mul(gb1, n1), df_mul(gb2, n2)), df_mul(gt, n3));
  const df g_div = df_neg(df_mul(df_mul(g_inv, inv), inv));
  df3 g_s = mul3(s1, g_n1);
  const df3 g_s1 = add3(mul3(s, g_n1), mul3(e1, g_div));
  df3 g_d = mul3(s2, g_n2);
  const df3 g_s2 = add3(mul3(d, g_n2), mul3(e2, g_n3));
  df3 g_e2 = mul3(s2, g_n3);
  df3 g_e1 = mul3(s1, g_div);
  // s1 = d x e2
  g_d = add3(g_d, cross3(e2, g_s1));
  g_e2 = add3(g_e2, cross3(g_s1, d));
  // s2 = s x e1
  g_s = add3(g_s, cross3(e1, g_s2));
  g_e1 = add3(g_e1, cross3(g_s2, s));
  // s = o - p0, e1 = p1 - p0, e2 = p2 - p0
  const float3 g_o = to_f3(g_s);
  const float3 g_dd = to_f3(g_d);
  const float3 g_p1 = to_f3(g_e1), g_p2 = to_f3(g_e2);
  const float3 g_p0 = to_f3(df3{df_neg(df_add(df_add(g_s.x, g_e1.x), g_e2.x)),
                                df_neg(df_add(df_add(g_s.y, g_e1.y), g_e2.y)),
                                df_neg(df_add(df_add(g_s.z, g_e1.z), g_e2.z))});
  reinterpret_cast<float4*>(gr)[0] = make_float4(g_o.x, g_o.y, g_o.z, 0.f);
  reinterpret_cast<float4*>(gr)[1] = make_float4(g_dd.x, g_dd.y, g_dd.z, 0.f);
  return TriGrad{{g_p0.x, g_p0.y, g_p0.z, g_p1.x, g_p1.y, g_p1.z, g_p2.x, g_p2.y, g_p2.z}};
}

BVHGPU_DEV void zero_ray_grad(const AdjointArgs& a, uint64_t rid) {
  float4* gr = reinterpret_cast<float4*>(a.grad_rays + rid * 8);
  gr[0] = make_float4(0.f, 0.f, 0.f, 0.f);
  gr[1] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Adds the vertex gradients of the warp's hits. Neighbouring rays often hit
// the same triangle (a large triangle close to the camera takes thousands of
// rays), so lanes with the same triangle first sum their gradients through
// shuffles and one lane per triangle issues the atomics: same-address
// atomics would serialise in L2. Every lane of the warp must call this
// (valid = false: nothing to add).
BVHGPU_DEV void scatter_grads(const SceneDev& sc, const AdjointArgs& a, bool valid,
                              uint32_t prim, TriGrad g) {
  constexpr unsigned FULL = 0xFFFFFFFFu;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long key = valid ? (unsigned long long)prim : (1ull << 32) | lane;
  const unsigned peers = __match_any_sync(FULL, key);
  const int leader = __ffs(peers) - 1;
  unsigned donors = __ballot_sync(FULL, valid && (int)lane != leader);
  TriGrad sum = g;
  while (donors) {
    const int k = __ffs(donors) - 1;
    donors &= donors - 1u;
    const int to = __shfl_sync(FULL, leader, k);
#pragma unroll
    for (int c = 0; c < 9; ++c) {
      const float x = __shfl_sync(FULL, g.v[c], k);
      if ((int)lane == to) sum.v[c] += x;
    }
  }
  if (!valid || (int)lane != leader) return;
  if (a.faces) {
    const int32_t* fv = a.faces + (size_t)prim * 3;
    const uint32_t v0 = (uint32_t)__ldg(fv + 0), v1 = (uint32_t)__ldg(fv + 1);
    const uint32_t v2 = (uint32_t)__ldg(fv + 2);
    if (v0 >= a.n_verts || v1 >= a.n_verts || v2 >= a.n_verts) {
      record_error(sc.status, BVHGPU_ERR_BAD_ARG);
      return;
    }
    const uint32_t vid[3] = {v0, v1, v2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float* gv = a.grad_verts + (size_t)vid[k] * 3;
      atomicAdd(gv + 0, sum.v[3 * k + 0]);
      atomicAdd(gv + 1, sum.v[3 * k + 1]);
      atomicAdd(gv + 2, sum.v[3 * k + 2]);
    }
  } else {
    float* gt9 = a.grad_tri9 + (size_t)prim * 9;
#pragma unroll
    for (int c = 0; c < 9; ++c) atomicAdd(gt9 + c, sum.v[c]);
  }
}

// Re-trace, then the reverse pass. Lanes past the end or without a hit stay
// in the warp until the gradient scatter.
template <int N>
__global__ void __launch_bounds__(128) adjoint_kernel(SceneDev sc, AdjointArgs a) {
  extern __shared__ uint32_t smem[];
  const int stride = blockDim.x;
  uint32_t* stack = smem + threadIdx.x;
  const uint64_t rid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = false;
  uint32_t prim = 0;
  TriGrad g{};
  if (rid < a.n) {
    const bvhgpu_ray_t in = load_ray(a.rays, rid);
    Best best;
    bool ok = !isnan(in.ox);
    if (ok) {
      // Re-trace: closest hit, fast profile, depth-first.
      const Ray r = make_ray<BVHGPU_PROFILE_FAST>(in);
      float tmax = r.tmax;
      Counters ctr;
      int sp = 1;
      stack[0] = sc.root_entry;
      while (sp > 0) {
        --sp;
        const uint32_t e = stack[sp * stride];
        if (e & kLeafBit) {
          leaf_step<BVHGPU_PROFILE_FAST, BVHGPU_CLOSEST, false>(sc, e, r, tmax, best, ctr);
        } else {
          int depth;
          if (!node_step<N, BVHGPU_PROFILE_FAST, BVHGPU_CLOSEST, false, kFmtFP32>(
                  sc, e, nullptr, 0u, r, tmax, stack, stride, sp, a.stack_cap, ctr, depth)) {
            record_error(sc.status, kDevErrStackOverflow);
            ok = false;
            break;
          }
        }
      }
    }
    if (ok && best.lane >= 0) {
      prim = __ldg(sc.leaf_prim + (size_t)best.leaf * sc.leaf_memory + best.lane);
      g = adjoint_reverse(sc, a, rid, in, best.leaf, best.lane);
      valid = true;
    } else {
      zero_ray_grad(a, rid);
    }
  }
  scatter_grads(sc, a, valid, prim, g);
}

// The reverse pass from stored closest hits (the forward pass's records):
// no traversal. A hit's prim selects the triangle through the input id ->
// leaf slot map; misses (prim -1) get zero gradients, unknown ids too (and
// are recorded as a bad argument).
__global__ void __launch_bounds__(128) adjoint_hits_kernel(SceneDev sc, AdjointArgs a) {
  const uint64_t rid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool valid = false;
  uint32_t prim = 0;
  TriGrad g{};
  if (rid < a.n) {
    const bvhgpu_ray_t in = load_ray(a.rays, rid);
    prim = __float_as_uint(__ldg(a.hits + rid).x);
    uint32_t slot = 0xFFFFFFFFu;
    if (!isnan(in.ox) && prim != 0xFFFFFFFFu) {
      slot = prim < a.n_prims ? __ldg(a.prim_slot + prim) : 0xFFFFFFFFu;
      if (slot == 0xFFFFFFFFu) record_error(sc.status, BVHGPU_ERR_BAD_ARG);
    }
    if (slot != 0xFFFFFFFFu) {
      const uint32_t lm = (uint32_t)sc.leaf_memory;
      g = adjoint_reverse(sc, a, rid, in, slot / lm, (int)(slot % lm));
      valid = true;
    } else {
      zero_ray_grad(a, rid);
    }
  }
  scatter_grads(sc, a, valid, prim, g);
}

cudaError_t launch_adjoint(const SceneDev& sc, int nm, const AdjointArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const int bs = 128;
  if (a.hits) {
    adjoint_hits_kernel<<<(unsigned)((a.n + bs - 1) / bs), bs, 0, s>>>(sc, a);
    return cudaGetLastError();
  }
  const size_t smem = (size_t)a.stack_cap * bs * 4;
  const uint64_t grid = (a.n + bs - 1) / bs;
  auto pick = [&](auto k) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)grid, bs, smem, s>>>(sc, a);
    return cudaGetLastError();
  };
  switch (nm) {
    case 4: return pick(adjoint_kernel<4>);
    case 8: return pick(adjoint_kernel<8>);
    case 12: return pick(adjoint_kernel<12>);
    case 16: return pick(adjoint_kernel<16>);
  }
  return cudaErrorInvalidValue;
}

}  // namespace dev
}  // namespace bvhgpu
