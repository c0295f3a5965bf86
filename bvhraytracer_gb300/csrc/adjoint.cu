// Adjoint of the leaf intersection: gradients of (t, b1, b2) of each ray's
// closest hit with respect to the three triangle vertices and the ray origin
// and direction, through a fixed visibility set.
//
// The kernel does not read stored hits: it re-traces each ray (per-ray
// depth-first, fast profile, so the hit is the forward pass's), then runs the
// reverse pass of the Moller-Trumbore expressions of triIntersect{L}
// (rayTracerTemplate.ispc:35-76):
//   e1 = p1 - p0, e2 = p2 - p0, s1 = d x e2, div = s1.e1, inv = 1/div,
//   s = o - p0, b1 = (s.s1) inv, s2 = s x e1, b2 = (d.s2) inv,
//   t = (e2.s2) inv.
// Vertex gradients are accumulated per triangle (9 floats) with atomics; the
// caller scatters them to shared vertices.
#include "adjoint.cuh"

namespace bvhgpu {
namespace dev {

BVHGPU_DEV float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
BVHGPU_DEV float3 sub3(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
BVHGPU_DEV float3 add3(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
BVHGPU_DEV float3 mul3(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
BVHGPU_DEV float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
BVHGPU_DEV float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

template <int N>
__global__ void __launch_bounds__(128) adjoint_kernel(SceneDev sc, AdjointArgs a) {
  extern __shared__ uint32_t smem[];
  const int stride = blockDim.x;
  uint32_t* stack = smem + threadIdx.x;
  const uint64_t rid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (rid >= a.n) return;
  float* gr = a.grad_rays + rid * 8;
  const bvhgpu_ray_t in = load_ray(a.rays, rid);
  if (isnan(in.ox)) {
    for (int k = 0; k < 8; ++k) gr[k] = 0.f;
    return;
  }
  // Re-trace: closest hit, fast profile, depth-first.
  const Ray r = make_ray<BVHGPU_PROFILE_FAST>(in);
  float tmax = r.tmax;
  Best best;
  Counters ctr;
  int sp = 1;
  stack[0] = sc.root_entry;
  bool ok = true;
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
  if (!ok || best.lane < 0) {
    for (int k = 0; k < 8; ++k) gr[k] = 0.f;
    return;
  }
  // Vertices of the hit triangle from its leaf block (original axes).
  const float* blk = sc.leaves + (size_t)best.leaf * 9 * sc.leaf_memory;
  // Stride = leaf count rounded up to the gang: recover it from the sentinel.
  int stride_l = sc.leaf_memory;
  {
    const float last = blk[sc.leaf_memory * 9 - 1];
    if (isnan(last)) stride_l = (int)blk[sc.leaf_memory * 9 - 2];
  }
  const int i = best.lane;
  const float3 p0 = f3(blk[0 * stride_l + i], blk[1 * stride_l + i], blk[2 * stride_l + i]);
  const float3 p1 = f3(blk[3 * stride_l + i], blk[4 * stride_l + i], blk[5 * stride_l + i]);
  const float3 p2 = f3(blk[6 * stride_l + i], blk[7 * stride_l + i], blk[8 * stride_l + i]);
  const uint32_t prim = __ldg(sc.leaf_prim + (size_t)best.leaf * sc.leaf_memory + i);
  const float3 o = f3(r.o[0], r.o[1], r.o[2]);
  const float3 d = f3(r.d[0], r.d[1], r.d[2]);

  // Forward intermediates.
  const float3 e1 = sub3(p1, p0), e2 = sub3(p2, p0);
  const float3 s1 = cross3(d, e2);
  const float div = dot3(s1, e1);
  const float inv = 1.f / div;
  const float3 s = sub3(o, p0);
  const float n1 = dot3(s, s1);
  const float3 s2 = cross3(s, e1);
  const float n2 = dot3(d, s2);
  const float n3 = dot3(e2, s2);

  // Reverse pass.
  const float4 g = a.grad_hits[rid];
  const float gt = g.y, gb1 = g.z, gb2 = g.w;
  const float g_n1 = gb1 * inv, g_n2 = gb2 * inv, g_n3 = gt * inv;
  const float g_inv = gb1 * n1 + gb2 * n2 + gt * n3;
  const float g_div = -g_inv * inv * inv;
  float3 g_s = mul3(s1, g_n1);
  float3 g_s1 = add3(mul3(s, g_n1), mul3(e1, g_div));
  float3 g_d = mul3(s2, g_n2);
  float3 g_s2 = add3(mul3(d, g_n2), mul3(e2, g_n3));
  float3 g_e2 = mul3(s2, g_n3);
  float3 g_e1 = mul3(s1, g_div);
  // s1 = d x e2
  g_d = add3(g_d, cross3(e2, g_s1));
  g_e2 = add3(g_e2, cross3(g_s1, d));
  // s2 = s x e1
  g_s = add3(g_s, cross3(e1, g_s2));
  g_e1 = add3(g_e1, cross3(g_s2, s));
  // s = o - p0, e1 = p1 - p0, e2 = p2 - p0
  const float3 g_o = g_s;
  const float3 g_p1 = g_e1, g_p2 = g_e2;
  const float3 g_p0 = f3(-(g_s.x + g_e1.x + g_e2.x), -(g_s.y + g_e1.y + g_e2.y),
                         -(g_s.z + g_e1.z + g_e2.z));
  float* gt9 = a.grad_tri9 + (size_t)prim * 9;
  atomicAdd(gt9 + 0, g_p0.x); atomicAdd(gt9 + 1, g_p0.y); atomicAdd(gt9 + 2, g_p0.z);
  atomicAdd(gt9 + 3, g_p1.x); atomicAdd(gt9 + 4, g_p1.y); atomicAdd(gt9 + 5, g_p1.z);
  atomicAdd(gt9 + 6, g_p2.x); atomicAdd(gt9 + 7, g_p2.y); atomicAdd(gt9 + 8, g_p2.z);
  reinterpret_cast<float4*>(gr)[0] = make_float4(g_o.x, g_o.y, g_o.z, 0.f);
  reinterpret_cast<float4*>(gr)[1] = make_float4(g_d.x, g_d.y, g_d.z, 0.f);
}

cudaError_t launch_adjoint(const SceneDev& sc, int nm, const AdjointArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const int bs = 128;
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
