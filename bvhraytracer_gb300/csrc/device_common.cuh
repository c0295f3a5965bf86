// Device-side building blocks shared by every traversal kernel: ray set-up,
// the N-wide slab test and the two L-wide leaf tests.
//
// Bit-exactness: this code must be compiled with -fmad=false, -prec-div=true,
// -prec-sqrt=true and -ftz=false (the build script does so). Every float
// expression keeps the reference's evaluation order, so results match the
// reference's scalar / ISPC code (compiled without FMA contraction)
// operation for operation.
#pragma once
#include <cfloat>
#include <cstdint>

#include "bvhgpu.h"

namespace bvhgpu {
namespace dev {

#define BVHGPU_DEV __device__ __forceinline__

constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kLeafCountShift = 27;
constexpr uint32_t kLeafIndexMask = (1u << 27) - 1;

// Device error codes recorded in the scene's status word.
constexpr int kDevErrStackOverflow = BVHGPU_ERR_STACK_OVERFLOW;
constexpr int kDevErrTimeout = BVHGPU_ERR_TIMEOUT;
constexpr int kDevErrQ8Encode = BVHGPU_ERR_UNSUPPORTED;

// pbrt gamma(n) = (n*eps/2) / (1 - n*eps/2), evaluated in double and rounded
// to float as MSVC does for the reference (src/util.h:13-17, 44-48).
constexpr float kGamma2 = (float)((2 * (FLT_EPSILON * 0.5)) / (1 - 2 * (FLT_EPSILON * 0.5)));
constexpr float kGamma3 = (float)((3 * (FLT_EPSILON * 0.5)) / (1 - 3 * (FLT_EPSILON * 0.5)));
constexpr float kGamma5 = (float)((5 * (FLT_EPSILON * 0.5)) / (1 - 5 * (FLT_EPSILON * 0.5)));

// std::min / std::max (and glm::min / glm::max) on floats.
BVHGPU_DEV float rmin(float a, float b) { return (b < a) ? b : a; }
BVHGPU_DEV float rmax(float a, float b) { return (a < b) ? b : a; }

// maxDimension on |v| (glmUtil.h:18-23); also pbrt's kz.
BVHGPU_DEV int max_abs_dim(float x, float y, float z) {
  float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
  return (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
}

BVHGPU_DEV float sel3(int k, float x, float y, float z) { return k == 0 ? x : (k == 1 ? y : z); }

// Per-ray state held in registers.
struct Ray {
  float o[3];   // origin
  float d[3];   // direction (normalised for the instrumented profile)
  float inv[3]; // 1 / direction; FLT_MAX where the input component is 0
  float tmax;
  int code;     // major axis of |direction|
  bool reverse; // direction[code] <= 0: children are pushed in ascending order
  // Watertight test: permutation (kz == code) and shear (triangle.cpp:110-125),
  // which depend on the ray only.
  int kx, ky;
  float sx, sy, sz;
  // True when a NaN can appear in the box tests (non-finite origin, tMax or
  // 1/direction). Such rays take the reference's comparison forms exactly;
  // all others use IEEE min/max (see slab_mm).
  bool exact;
};

// Ray::Ray (src/ray.cpp:4-36) for the instrumented profile (normalise), and
// FastRay::FastRay (src/fastRay.cpp:3-20) for the fast profile.
template <int PROFILE>
BVHGPU_DEV Ray make_ray(const bvhgpu_ray_t& in) {
  Ray r;
  r.o[0] = in.ox; r.o[1] = in.oy; r.o[2] = in.oz;
  r.tmax = in.tmax;
  float dx = in.dx, dy = in.dy, dz = in.dz;
  if (PROFILE == BVHGPU_PROFILE_INSTRUMENTED) {
    // glm::normalize: v * (1 / sqrt((x*x + y*y) + z*z)).
    float dd = dx * dx + dy * dy + dz * dz;
    float s = 1.0f / sqrtf(dd);
    dx = dx * s; dy = dy * s; dz = dz * s;
  }
  r.d[0] = dx; r.d[1] = dy; r.d[2] = dz;
  r.inv[0] = in.dx == 0.0f ? FLT_MAX : 1.0f / dx;
  r.inv[1] = in.dy == 0.0f ? FLT_MAX : 1.0f / dy;
  r.inv[2] = in.dz == 0.0f ? FLT_MAX : 1.0f / dz;
  r.code = max_abs_dim(dx, dy, dz);
  r.reverse = sel3(r.code, dx, dy, dz) <= 0.0f;
  int kz = r.code;
  r.kx = kz + 1 == 3 ? 0 : kz + 1;
  r.ky = r.kx + 1 == 3 ? 0 : r.kx + 1;
  float pdx = sel3(r.kx, dx, dy, dz), pdy = sel3(r.ky, dx, dy, dz), pdz = sel3(kz, dx, dy, dz);
  r.sx = -pdx / pdz;
  r.sy = -pdy / pdz;
  r.sz = 1.f / pdz;
  r.exact = !(isfinite(r.o[0]) && isfinite(r.o[1]) && isfinite(r.o[2]) && isfinite(r.tmax) &&
              isfinite(r.inv[0]) && isfinite(r.inv[1]) && isfinite(r.inv[2]));
  return r;
}

// Slab test of one child box: CompactNodeManager::aabbCheck (compactNode.h:247-278)
// and aabbIntersect{N} (rayTracerTemplate.ispc:171-233).
BVHGPU_DEV bool slab(float lx, float ly, float lz, float hx, float hy, float hz, const Ray& r,
                     float tmax) {
  float t0 = 0.0f, t1 = tmax;
  float tn = (lx - r.o[0]) * r.inv[0], tf = (hx - r.o[0]) * r.inv[0];
  if (tn > tf) { float t = tn; tn = tf; tf = t; }
  t0 = rmax(tn, t0);
  t1 = rmin(tf, t1);
  tn = (ly - r.o[1]) * r.inv[1]; tf = (hy - r.o[1]) * r.inv[1];
  if (tn > tf) { float t = tn; tn = tf; tf = t; }
  t0 = rmax(tn, t0);
  t1 = rmin(tf, t1);
  tn = (lz - r.o[2]) * r.inv[2]; tf = (hz - r.o[2]) * r.inv[2];
  if (tn > tf) { float t = tn; tn = tf; tf = t; }
  t0 = rmax(tn, t0);
  t1 = rmin(tf, t1);
  return t0 <= t1;
}

// The same slab test with IEEE min / max. When no operand is NaN the two
// forms return the same boolean: they can differ only in the sign of a zero
// t0 / t1, and t0 <= t1 does not observe it. Rays that could produce a NaN
// (Ray::exact) use `slab`.
BVHGPU_DEV bool slab_mm(float lx, float ly, float lz, float hx, float hy, float hz, const Ray& r,
                        float tmax) {
  float tn = (lx - r.o[0]) * r.inv[0], tf = (hx - r.o[0]) * r.inv[0];
  float t0 = fmaxf(fminf(tn, tf), 0.0f), t1 = fminf(fmaxf(tn, tf), tmax);
  tn = (ly - r.o[1]) * r.inv[1]; tf = (hy - r.o[1]) * r.inv[1];
  t0 = fmaxf(fminf(tn, tf), t0);
  t1 = fminf(fmaxf(tn, tf), t1);
  tn = (lz - r.o[2]) * r.inv[2]; tf = (hz - r.o[2]) * r.inv[2];
  t0 = fmaxf(fminf(tn, tf), t0);
  t1 = fminf(fmaxf(tn, tf), t1);
  return t0 <= t1;
}

template <bool MM>
BVHGPU_DEV bool slab_t(float lx, float ly, float lz, float hx, float hy, float hz, const Ray& r,
                       float tmax) {
  return MM ? slab_mm(lx, ly, lz, hx, hy, hz, r, tmax) : slab(lx, ly, lz, hx, hy, hz, r, tmax);
}

// The slab test that also returns the box's entry distance t0: the
// `distance` of aabbCheck(ray, id, distance) (compactNode.h:280-313) and the
// distances[] of aabbIntersect{N}, kept on the stack by the save-distance
// traversals. For NaN-free rays the IEEE form gives the same t0 up to the
// sign of a zero, which the later `t0 > tMax` test does not observe.
template <bool MM>
BVHGPU_DEV bool slab_dist(float lx, float ly, float lz, float hx, float hy, float hz,
                          const Ray& r, float tmax, float& t0_out) {
  float t0, t1;
  if (MM) {
    float tn = (lx - r.o[0]) * r.inv[0], tf = (hx - r.o[0]) * r.inv[0];
    t0 = fmaxf(fminf(tn, tf), 0.0f);
    t1 = fminf(fmaxf(tn, tf), tmax);
    tn = (ly - r.o[1]) * r.inv[1]; tf = (hy - r.o[1]) * r.inv[1];
    t0 = fmaxf(fminf(tn, tf), t0);
    t1 = fminf(fmaxf(tn, tf), t1);
    tn = (lz - r.o[2]) * r.inv[2]; tf = (hz - r.o[2]) * r.inv[2];
    t0 = fmaxf(fminf(tn, tf), t0);
    t1 = fminf(fmaxf(tn, tf), t1);
  } else {
    t0 = 0.0f;
    t1 = tmax;
    float tn = (lx - r.o[0]) * r.inv[0], tf = (hx - r.o[0]) * r.inv[0];
    if (tn > tf) { float t = tn; tn = tf; tf = t; }
    t0 = rmax(tn, t0);
    t1 = rmin(tf, t1);
    tn = (ly - r.o[1]) * r.inv[1]; tf = (hy - r.o[1]) * r.inv[1];
    if (tn > tf) { float t = tn; tn = tf; tf = t; }
    t0 = rmax(tn, t0);
    t1 = rmin(tf, t1);
    tn = (lz - r.o[2]) * r.inv[2]; tf = (hz - r.o[2]) * r.inv[2];
    if (tn > tf) { float t = tn; tn = tf; tf = t; }
    t0 = rmax(tn, t0);
    t1 = rmin(tf, t1);
  }
  t0_out = t0;
  return t0 <= t1;
}

// min / max of the reference (MM false) or IEEE min / max (MM true).
template <bool MM> BVHGPU_DEV float tmin2(float a, float b) { return MM ? fminf(a, b) : rmin(a, b); }
template <bool MM> BVHGPU_DEV float tmax2(float a, float b) { return MM ? fmaxf(a, b) : rmax(a, b); }

// Watertight ray-triangle test of Triangle::intersect(Ray&)
// (src/primitives/triangle.cpp:52-249), on points given in the ray's
// permuted axes (x' = kx, y' = ky, z' = kz). Returns true on a hit with
// t <= tmax; b1 / b2 are the weights of p1 / p2. PRE false: the caller ran
// the box pre-test and it passed.
template <bool MM, bool PRE = true>
BVHGPU_DEV bool watertight(const float (&p)[3][3], const Ray& r, float tmax, float& t_out,
                           float& b1_out, float& b2_out) {
  const float ox = sel3(r.kx, r.o[0], r.o[1], r.o[2]);
  const float oy = sel3(r.ky, r.o[0], r.o[1], r.o[2]);
  const float oz = sel3(r.code, r.o[0], r.o[1], r.o[2]);
  // Translate to the ray origin (triangle.cpp:98-101).
  float p0x = p[0][0] - ox, p0y = p[0][1] - oy, p0z = p[0][2] - oz;
  float p1x = p[1][0] - ox, p1y = p[1][1] - oy, p1z = p[1][2] - oz;
  float p2x = p[2][0] - ox, p2y = p[2][1] - oy, p2z = p[2][2] - oz;
  if (PRE) {
    // Per-triangle box pre-test (triangle.cpp:55-79) in the permuted axes
    // (the max / min of three values does not depend on the axis order).
    // The reference computes (min(p) - o) * inv; rounding of a - o is
    // monotonic in a, so min(p) - o == min(p - o) exactly and the translated
    // coordinates above give the same bounds. Triangle vertices are finite,
    // so the bounds are NaN-free in both min / max forms.
    const float ix = sel3(r.kx, r.inv[0], r.inv[1], r.inv[2]);
    const float iy = sel3(r.ky, r.inv[0], r.inv[1], r.inv[2]);
    const float iz = sel3(r.code, r.inv[0], r.inv[1], r.inv[2]);
    float t1x = fminf(fminf(p0x, p1x), p2x) * ix, t2x = fmaxf(fmaxf(p0x, p1x), p2x) * ix;
    float t1y = fminf(fminf(p0y, p1y), p2y) * iy, t2y = fmaxf(fmaxf(p0y, p1y), p2y) * iy;
    float t1z = fminf(fminf(p0z, p1z), p2z) * iz, t2z = fmaxf(fmaxf(p0z, p1z), p2z) * iz;
    float tmin = tmax2<MM>(tmax2<MM>(tmin2<MM>(t1x, t2x), tmin2<MM>(t1y, t2y)), tmin2<MM>(t1z, t2z));
    float tmx = tmin2<MM>(tmin2<MM>(tmax2<MM>(t1x, t2x), tmax2<MM>(t1y, t2y)), tmax2<MM>(t1z, t2z));
    if (tmx < 0) return false;
    if (tmin > tmx) return false;
    if (tmax < tmin) return false;
  }
  p0x += r.sx * p0z; p0y += r.sy * p0z;
  p1x += r.sx * p1z; p1y += r.sy * p1z;
  p2x += r.sx * p2z; p2y += r.sy * p2z;
  float e0 = p1x * p2y - p1y * p2x;
  float e1 = p2x * p0y - p2y * p0x;
  float e2 = p0x * p1y - p0y * p1x;
  if (e0 == 0.0f || e1 == 0.0f || e2 == 0.0f) {
    // Double-precision fallback at triangle edges (triangle.cpp:136-147).
    // The float products are exact in double; this branch is rare.
    double p2txp1ty = (double)p2x * (double)p1y;
    double p2typ1tx = (double)p2y * (double)p1x;
    e0 = (float)(p2typ1tx - p2txp1ty);
    double p0txp2ty = (double)p0x * (double)p2y;
    double p0typ2tx = (double)p0y * (double)p2x;
    e1 = (float)(p0typ2tx - p0txp2ty);
    double p1txp0ty = (double)p1x * (double)p0y;
    double p1typ0tx = (double)p1y * (double)p0x;
    e2 = (float)(p1typ0tx - p1txp0ty);
  }
  if ((e0 < 0 || e1 < 0 || e2 < 0) && (e0 > 0 || e1 > 0 || e2 > 0)) return false;
  float det = e0 + e1 + e2;
  if (det == 0) return false;
  p0z *= r.sz; p1z *= r.sz; p2z *= r.sz;
  float t_scaled = e0 * p0z + e1 * p1z + e2 * p2z;
  if (det < 0 && (t_scaled >= 0 || t_scaled < tmax * det)) return false;
  else if (det > 0 && (t_scaled <= 0 || t_scaled > tmax * det)) return false;
  float inv_det = 1 / det;
  float b1 = e1 * inv_det;
  float b2 = e2 * inv_det;
  float t = t_scaled * inv_det;
  // Conservative t > 0 check (triangle.cpp:172-196).
  float max_zt = tmax2<MM>(tmax2<MM>(fabsf(p0z), fabsf(p1z)), fabsf(p2z));
  float delta_z = kGamma3 * max_zt;
  float max_xt = tmax2<MM>(tmax2<MM>(fabsf(p0x), fabsf(p1x)), fabsf(p2x));
  float max_yt = tmax2<MM>(tmax2<MM>(fabsf(p0y), fabsf(p1y)), fabsf(p2y));
  float delta_x = kGamma5 * (max_xt + max_zt);
  float delta_y = kGamma5 * (max_yt + max_zt);
  float delta_e = 2 * (kGamma2 * max_xt * max_yt + delta_y * max_xt + delta_x * max_yt);
  float max_e = tmax2<MM>(tmax2<MM>(fabsf(e0), fabsf(e1)), fabsf(e2));
  float delta_t =
      3 * (kGamma3 * max_e * max_zt + delta_e * max_zt + delta_z * max_e) * fabsf(inv_det);
  if (t <= delta_t) return false;
  t_out = t;
  b1_out = b1;
  b2_out = b2;
  return true;
}

// Moller-Trumbore test of triIntersect{L} / triAnyHit{L}
// (rayTracerTemplate.ispc:26-168), on points in the original axes.
BVHGPU_DEV bool moller_trumbore(const float (&p)[3][3], const Ray& r, float tmax, float& t_out,
                                float& b1_out, float& b2_out) {
  float e1x = p[1][0] - p[0][0], e1y = p[1][1] - p[0][1], e1z = p[1][2] - p[0][2];
  float e2x = p[2][0] - p[0][0], e2y = p[2][1] - p[0][1], e2z = p[2][2] - p[0][2];
  // s1 = cross(dir, e2)
  float s1x = r.d[1] * e2z - r.d[2] * e2y;
  float s1y = r.d[2] * e2x - r.d[0] * e2z;
  float s1z = r.d[0] * e2y - r.d[1] * e2x;
  float divisor = s1x * e1x + s1y * e1y + s1z * e1z;
  bool hit = true;
  if (divisor == 0.0f) hit = false;
  float inv_div = 1.f / divisor;
  float dx = r.o[0] - p[0][0], dy = r.o[1] - p[0][1], dz = r.o[2] - p[0][2];
  float b1 = (dx * s1x + dy * s1y + dz * s1z) * inv_div;
  if (b1 < 0.0f || b1 > 1.0f) hit = false;
  // s2 = cross(d, e1)
  float s2x = dy * e1z - dz * e1y;
  float s2y = dz * e1x - dx * e1z;
  float s2z = dx * e1y - dy * e1x;
  float b2 = (r.d[0] * s2x + r.d[1] * s2y + r.d[2] * s2z) * inv_div;
  if (b2 < 0.0f || b1 + b2 > 1.0f) hit = false;
  float t = (e2x * s2x + e2y * s2y + e2z * s2z) * inv_div;
  if (t < 0.0f || t > tmax) hit = false;
  t_out = t;
  b1_out = b1;
  b2_out = b2;
  return hit;
}

// ---- mbarrier + bulk copy (TMA) helpers, inline PTX (sm_90 and later) ----
BVHGPU_DEV uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
BVHGPU_DEV void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
BVHGPU_DEV void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// Global -> shared bulk copy completing on `bar`; 16-byte aligned addresses,
// size a multiple of 16.
BVHGPU_DEV void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Nanoseconds of the global timer.
BVHGPU_DEV uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the phase with the given parity to complete; gives up after
// `limit_ns` nanoseconds and returns false.
BVHGPU_DEV bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const uint32_t a = smem_addr(bar);
  const uint64_t t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Read-only global loads.
BVHGPU_DEV float4 ldg4(const void* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
BVHGPU_DEV uint4 ldgu4(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
BVHGPU_DEV uint32_t ldgu(const void* p) { return __ldg(reinterpret_cast<const uint32_t*>(p)); }

BVHGPU_DEV float f4get(const float4& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// Packed pairs of floats in one 64-bit register, and the sm_100-family
// instructions that apply one IEEE single-precision operation to both halves
// (sub / mul .rn.f32x2: round to nearest per half, subnormals kept, no
// contraction), so each half equals the scalar `a - b` / `a * b` of this
// build (-fmad=false -ftz=false) bit for bit.
BVHGPU_DEV uint64_t f2pack(float lo, float hi) {
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
BVHGPU_DEV float2 f2unpack(uint64_t v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
BVHGPU_DEV uint64_t f2sub(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
BVHGPU_DEV uint64_t f2mul(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// a + b rounded up / down per half (the pairs of __fadd_ru / __fadd_rd).
BVHGPU_DEV uint64_t f2add_ru(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rp.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
BVHGPU_DEV uint64_t f2add_rd(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rm.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
BVHGPU_DEV uint64_t f2splat(float v) { return f2pack(v, v); }
// (a - o) * s on a pair: two children's plane distances along one axis.
BVHGPU_DEV float2 f2plane(float a0, float a1, uint64_t o2, uint64_t s2) {
  return f2unpack(f2mul(f2sub(f2pack(a0, a1), o2), s2));
}

}  // namespace dev
}  // namespace bvhgpu
