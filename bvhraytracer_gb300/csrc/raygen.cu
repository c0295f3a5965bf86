// Ray generation on the GPU, so a frame never leaves the device between the
// primary and the secondary traces:
//   * camera rays: Camera::getRayTargetPosition (camera.h:82-98) and
//     FastRay(pos, target) (fastRay.cpp:3-20) for every pixel, emitted
//     workgroup by workgroup like CameraFast::renderImage
//     (cameraFast.h:465-490);
//   * secondary rays from closest hits: getSurfaceNormalPosition
//     (fastNodeManager.h:1700-1713) with computeNormal (glmUtil.h:36-39), the
//     origin offset along the normal (cameraFast.h:373, 521), one shadow ray
//     toward a point light and AO rays, either cosine-distributed from a
//     counter-based hash or the reference's hashed uniform hemisphere
//     (Camera::getAmbientDirection / sampleHemisphere, camera.cpp:21-52);
//   * the AO factor per pixel, 1 - occluded / samples (cameraData.h:403-406).
// Float expressions keep the reference's (GLM's) evaluation order; the
// library is compiled without FMA contraction.
#include <cuda_runtime.h>

#include "raygen.cuh"

namespace bvhgpu {
namespace dev {

namespace {

struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
// glm::dot: (x*x' + y*y') + z*z'
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
// glm::cross(x, y) = (x.y*y.z - y.y*x.z, x.z*y.x - y.z*x.x, x.x*y.y - y.x*x.y)
__device__ __forceinline__ V3 cross(V3 x, V3 y) {
  return v3(x.y * y.z - y.y * x.z, x.z * y.x - y.z * x.x, x.x * y.y - y.x * x.y);
}
// glm::normalize: v * inversesqrt(dot(v, v)), inversesqrt(x) = 1 / sqrt(x)
__device__ __forceinline__ V3 normalize(V3 v) { return mul(v, 1.0f / sqrtf(dot(v, v))); }

__device__ __forceinline__ void store_ray(bvhgpu_ray_t* out, uint64_t i, V3 o, float tmax, V3 d) {
  float4* q = reinterpret_cast<float4*>(out + i);
  q[0] = make_float4(o.x, o.y, o.z, tmax);
  q[1] = make_float4(d.x, d.y, d.z, 0.0f);
}

__device__ __forceinline__ void store_inactive(bvhgpu_ray_t* out, uint64_t i) {
  const float nan = __int_as_float(0x7FC00000);
  float4* q = reinterpret_cast<float4*>(out + i);
  q[0] = make_float4(nan, nan, nan, 0.0f);
  q[1] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
}

__global__ void camera_rays_kernel(CameraArgs c, bvhgpu_ray_t* out) {
  const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= c.n) return;
  // Tile-major pixel order: tiles of wg x wg pixels in row-major tile order,
  // row-major inside a tile; edge tiles keep only the pixels inside the image.
  const int wg = c.workgroup;
  const uint32_t tiles_x = (c.width + wg - 1) / wg;
  uint32_t col, row;
  {
    // Locate pixel p: full tile rows first, then the partial last tile row.
    const uint64_t full_rows = c.height / wg;
    const uint64_t per_tile_row = (uint64_t)c.width * wg;
    uint64_t tr = p / per_tile_row, rem = p % per_tile_row;
    const uint32_t tile_h = tr < full_rows ? wg : c.height - (uint32_t)tr * wg;
    // Inside a tile row: full tiles (wg wide) then the partial last tile.
    const uint64_t full_tiles = c.width / wg;
    const uint64_t per_tile = (uint64_t)wg * tile_h;
    uint64_t tc = rem / per_tile, in = rem % per_tile;
    uint32_t tile_w = wg;
    if (tc >= full_tiles) {
      tc = full_tiles;
      in = rem - full_tiles * per_tile;
      tile_w = c.width - (uint32_t)full_tiles * wg;
    }
    (void)tiles_x;
    row = (uint32_t)tr * wg + (uint32_t)(in / tile_w);
    col = (uint32_t)tc * wg + (uint32_t)(in % tile_w);
  }
  // cameraFast.h:484-489: h = -(row - height/2), w = col - width/2 (ints).
  const int h = -((int)row - (int)(c.height / 2));
  const int w = (int)col - (int)(c.width / 2);
  // centerOffset = ((0,1,0,0) h + (1,0,0,0) w) (1 / width) + (0,0,-focal,0)
  const float fh = (float)h, fw = (float)w, inv_w = 1.0f / (float)c.width;
  const float ox = (0.0f * fh + 1.0f * fw) * inv_w + 0.0f;
  const float oy = (1.0f * fh + 0.0f * fw) * inv_w + 0.0f;
  const float oz = (0.0f * fh + 0.0f * fw) * inv_w + -c.focal;
  const float ow = (0.0f * fh + 0.0f * fw) * inv_w + 0.0f;
  // mat4 * vec4 (GLM): (m0 x + m1 y) + (m2 z + m3 w), columns m0..m3.
  const float* m = c.transform;
  V3 t;
  t.x = (m[0] * ox + m[4] * oy) + (m[8] * oz + m[12] * ow);
  t.y = (m[1] * ox + m[5] * oy) + (m[9] * oz + m[13] * ow);
  t.z = (m[2] * ox + m[6] * oy) + (m[10] * oz + m[14] * ow);
  const V3 pos = v3(c.pos[0], c.pos[1], c.pos[2]);
  const V3 target = add(pos, t);
  store_ray(out, p, pos, c.tmax, sub(target, pos));
}

// FNV-1a, 64 bit, over the 8 little-endian bytes of x: std::hash<size_t> of
// the MSVC standard library the reference was built with.
__device__ __forceinline__ uint64_t fnv1a64(uint64_t x) {
  uint64_t h = 14695981039346656037ull;
  for (int b = 0; b < 8; ++b) {
    h ^= (x >> (8 * b)) & 0xFFu;
    h *= 1099511628211ull;
  }
  return h;
}

// SplitMix64 finaliser (Steele, Lea, Flood 2014): the counter-based hash of
// the cosine sampler.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float unit24(uint64_t h) {
  return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
}

__global__ void secondary_rays_kernel(SceneDev sc, SecondaryArgs a) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int S = a.ao_samples;
  const float4 hh = a.hits[i];
  const int prim = __float_as_int(hh.x);
  if (prim < 0 || (uint32_t)prim >= a.n_prims || a.prim_slot[prim] == 0xFFFFFFFFu) {
    // Missed primary ray: inactive secondaries (NaN origin), like
    // rays[j].pos = NaN in cameraFast.h:524-528.
    if (a.shadow) store_inactive(a.shadow, i);
    for (int k = 0; k < S; ++k) store_inactive(a.ao, i * S + k);
    return;
  }
  const uint32_t slot = a.prim_slot[prim];
  const uint32_t leaf = slot / (uint32_t)sc.leaf_memory, lane = slot % (uint32_t)sc.leaf_memory;
  const float* blk = sc.leaves + (size_t)leaf * 9 * sc.leaf_memory;
  int st = sc.leaf_memory;
  if (isnan(blk[sc.leaf_memory * 9 - 1])) st = (int)blk[sc.leaf_memory * 9 - 2];
  const V3 p0 = v3(blk[0 * st + lane], blk[1 * st + lane], blk[2 * st + lane]);
  const V3 p1 = v3(blk[3 * st + lane], blk[4 * st + lane], blk[5 * st + lane]);
  const V3 p2 = v3(blk[6 * st + lane], blk[7 * st + lane], blk[8 * st + lane]);
  const bvhgpu_ray_t in = load_ray(a.primary, i);
  const V3 o = v3(in.ox, in.oy, in.oz), d = v3(in.dx, in.dy, in.dz);
  // getSurfaceNormalPosition (fastNodeManager.h:1700-1713)
  const V3 nrm = normalize(cross(sub(p1, p0), sub(p2, p0)));
  const float denom = dot(nrm, d);
  const float t = dot(sub(p0, o), nrm) / denom;
  const V3 pos = add(o, mul(d, t));
  const V3 org = add(pos, mul(nrm, a.offset));
  if (a.shadow) {
    const V3 v = sub(v3(a.light[0], a.light[1], a.light[2]), org);
    const float dist = sqrtf(dot(v, v));
    store_ray(a.shadow, i, org, dist, mul(v, 1.0f / dist));
  }
  if (S == 0) return;
  if (a.sampling == BVHGPU_AO_REFERENCE) {
    // Camera::getAmbientDirection / sampleHemisphere (camera.cpp:21-52).
    const long long index = (long long)(a.seed + i);
    for (int k = 0; k < S; ++k) {
      const uint64_t hu = fnv1a64((uint64_t)(index * 599 + (long long)k * 223));
      const uint64_t hv = fnv1a64((uint64_t)(index * 181 + (long long)k * 691));
      // (float)SIZE_MAX rounds to 2^64
      const float u = __ull2float_rn(hu) / 18446744073709551616.0f;
      const float v = __ull2float_rn(hv) / 18446744073709551616.0f;
      const float phi = acosf(1.0f - 2.0f * u);
      const float theta = (float)(2.0 * 3.14159265358979323846 * (double)v);
      V3 r = v3(sinf(phi) * cosf(theta), sinf(phi) * sinf(theta), cosf(phi));
      if (dot(r, nrm) <= 0.0f) r = v3(-r.x, -r.y, -r.z);
      store_ray(a.ao, i * S + k, org, a.ao_length, r);
    }
    return;
  }
  // Cosine-distributed around the normal in the frame (t, b, n).
  const V3 ax = fabsf(nrm.x) > 0.9f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
  const V3 tg = normalize(cross(ax, nrm));
  const V3 bt = cross(nrm, tg);
  for (int k = 0; k < S; ++k) {
    const uint64_t h = mix64(a.seed ^ mix64(i * (uint64_t)S + (uint64_t)k));
    const float u1 = unit24(h), u2 = unit24(mix64(h));
    const float rr = sqrtf(u1);
    const float ph = 6.2831853071795864769f * u2;
    const float lx = rr * cosf(ph), ly = rr * sinf(ph), lz = sqrtf(fmaxf(0.0f, 1.0f - u1));
    const V3 dir = add(add(mul(tg, lx), mul(bt, ly)), mul(nrm, lz));
    store_ray(a.ao, i * S + k, org, a.ao_length, dir);
  }
}

__global__ void ao_factor_kernel(const uint8_t* occluded, uint64_t n, int samples, float* out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int count = 0;
  for (int k = 0; k < samples; ++k) count += occluded[i * samples + k] != 0;
  out[i] = 1.0f - (float)count / (float)samples;
}

}  // namespace

cudaError_t launch_camera_rays(const CameraArgs& c, bvhgpu_ray_t* out, cudaStream_t s) {
  if (c.n == 0) return cudaSuccess;
  camera_rays_kernel<<<(unsigned)((c.n + 255) / 256), 256, 0, s>>>(c, out);
  return cudaGetLastError();
}

cudaError_t launch_secondary_rays(const SceneDev& sc, const SecondaryArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  secondary_rays_kernel<<<(unsigned)((a.n + 127) / 128), 128, 0, s>>>(sc, a);
  return cudaGetLastError();
}

cudaError_t launch_ao_factor(const uint8_t* occluded, uint64_t n, int samples, float* out,
                             cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  ao_factor_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(occluded, n, samples, out);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
