// Ray reordering by direction: a counting sort of the rays over cube-map
// cells of their direction, so that the 32 lanes of a warp get rays that
// point the same way and walk similar paths through the tree (incoherent
// ambient-occlusion rays lose most of their SIMT efficiency otherwise).
//
// Bins: the major axis of |d| and its sign (6 faces) x k x k cells of the two
// minor components divided by the major one; rays with a NaN origin
// (inactive) go to one extra, last bin. Every block owns a contiguous chunk of
// kChunk input rays; the output of one bin holds the blocks' rays in block
// order, so rays of one bin that were close in the input (neighbouring
// pixels, one hit point's samples) stay close. Inside a block the positions
// come from shared-memory atomics, so their order there is not fixed; each
// ray is traced on its own, so the order changes no result.
//
// Passes: (1) bin of every ray and per-block bin counts; (2) per bin, an
// exclusive scan of the counts over blocks; (3) an exclusive scan of the bin
// totals; (4) scatter of the input indices into bin order. The rays are not
// copied: the trace kernels read ray perm[i] as their i-th ray and write its
// results to slot perm[i].
#include "reorder.cuh"

namespace bvhgpu {
namespace dev {

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 4096;  // input rays per block

inline uint64_t blocks_for(uint64_t n) { return (n + kChunk - 1) / kChunk; }
__host__ __device__ inline int bins_for(int k) { return 6 * k * k + 1; }

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

struct Scratch {
  uint16_t* bins;    // n
  uint32_t* counts;  // nb * blocks, bin-major
  uint32_t* totals;  // nb
  uint32_t* base;    // nb
};

Scratch carve(void* p, uint64_t n, int k) {
  const uint64_t nb = bins_for(k), blocks = blocks_for(n);
  uint8_t* b = static_cast<uint8_t*>(p);
  Scratch s;
  s.bins = reinterpret_cast<uint16_t*>(b);
  b += align256(n * 2);
  s.counts = reinterpret_cast<uint32_t*>(b);
  b += align256(nb * blocks * 4);
  s.totals = reinterpret_cast<uint32_t*>(b);
  b += align256(nb * 4);
  s.base = reinterpret_cast<uint32_t*>(b);
  return s;
}

__device__ __forceinline__ int cell(float u, float aw, int k) {
  // u / aw lies in [-1, 1]; NaN converts to 0.
  int c = (int)((u / aw + 1.0f) * 0.5f * (float)k);
  return c < 0 ? 0 : (c >= k ? k - 1 : c);
}

__device__ __forceinline__ uint32_t dir_bin(float ox, float dx, float dy, float dz, int k) {
  if (isnan(ox)) return (uint32_t)(6 * k * k);
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  int m;
  float w, u, v;
  if (ax >= ay && ax >= az) {
    m = 0; w = dx; u = dy; v = dz;
  } else if (ay >= az) {
    m = 1; w = dy; u = dz; v = dx;
  } else {
    m = 2; w = dz; u = dx; v = dy;
  }
  const float aw = fabsf(w);
  const int face = m * 2 + (w < 0.0f ? 1 : 0);
  if (!(aw > 0.0f)) return (uint32_t)(face * k * k);
  return (uint32_t)((face * k + cell(u, aw, k)) * k + cell(v, aw, k));
}

__global__ void __launch_bounds__(kThreads) bin_count_kernel(const bvhgpu_ray_t* rays, uint64_t n,
                                                             int k, Scratch s, uint64_t blocks) {
  extern __shared__ uint32_t hist[];
  const int nb = bins_for(k);
  for (int i = threadIdx.x; i < nb; i += kThreads) hist[i] = 0;
  __syncthreads();
  const uint64_t begin = (uint64_t)blockIdx.x * kChunk;
  const uint64_t end = begin + kChunk < n ? begin + kChunk : n;
  for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
    const float4* p = reinterpret_cast<const float4*>(rays + i);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    const uint32_t bin = dir_bin(a.x, b.x, b.y, b.z, k);
    s.bins[i] = (uint16_t)bin;
    atomicAdd(&hist[bin], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += kThreads)
    s.counts[(uint64_t)i * blocks + blockIdx.x] = hist[i];
}

// Exclusive scan of `len` values in place by one block; returns the total.
__device__ uint32_t block_scan_inplace(uint32_t* v, uint64_t len) {
  __shared__ uint32_t warp_sums[kThreads / 32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (uint64_t off = 0; off < len; off += kThreads) {
    const uint64_t i = off + threadIdx.x;
    const uint32_t x = i < len ? v[i] : 0u;
    uint32_t incl = x;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = lane < kThreads / 32 ? warp_sums[lane] : 0u;
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, w, d);
        if (lane >= d) w += y;
      }
      if (lane < kThreads / 32) warp_sums[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const uint32_t before = (warp > 0 ? warp_sums[warp - 1] : 0u) + carry;
    if (i < len) v[i] = before + incl - x;
    __syncthreads();
    if (threadIdx.x == kThreads - 1) carry = before + incl;
    __syncthreads();
  }
  return carry;
}

__global__ void __launch_bounds__(kThreads) scan_bins_kernel(Scratch s, uint64_t blocks) {
  const uint32_t total = block_scan_inplace(s.counts + (uint64_t)blockIdx.x * blocks, blocks);
  if (threadIdx.x == 0) s.totals[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) scan_totals_kernel(Scratch s, int nb) {
  for (int i = threadIdx.x; i < nb; i += kThreads) s.base[i] = s.totals[i];
  __syncthreads();
  block_scan_inplace(s.base, (uint64_t)nb);
}

__global__ void __launch_bounds__(kThreads) scatter_kernel(uint64_t n, int k, Scratch s,
                                                           uint64_t blocks, uint32_t* perm) {
  extern __shared__ uint32_t cursor[];
  const int nb = bins_for(k);
  for (int i = threadIdx.x; i < nb; i += kThreads)
    cursor[i] = s.base[i] + s.counts[(uint64_t)i * blocks + blockIdx.x];
  __syncthreads();
  const uint64_t begin = (uint64_t)blockIdx.x * kChunk;
  const uint64_t end = begin + kChunk < n ? begin + kChunk : n;
  for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
    const uint32_t pos = atomicAdd(&cursor[s.bins[i]], 1u);
    perm[pos] = (uint32_t)i;
  }
}

// Job of grid chunk c: the last job whose first chunk is <= c.
__device__ __forceinline__ int seg_job_of(const SegTable& t, uint32_t c) {
  int lo = 0, hi = t.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.jobs[mid].first_chunk <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kThreads) seg_bin_count_kernel(const __grid_constant__ SegTable t) {
  extern __shared__ uint32_t hist[];
  const int nb = bins_for(t.k);
  const SegJob& J = t.jobs[seg_job_of(t, blockIdx.x)];
  const uint32_t chunk = blockIdx.x - J.first_chunk;
  for (int i = threadIdx.x; i < nb; i += kThreads) hist[i] = 0;
  __syncthreads();
  const uint64_t begin = (uint64_t)chunk * kChunk;
  const uint64_t end = begin + kChunk < J.n ? begin + kChunk : J.n;
  for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
    const float4* p = reinterpret_cast<const float4*>(J.rays + i);
    const float4 a = __ldg(p), b = __ldg(p + 1);
    const uint32_t bin = dir_bin(a.x, b.x, b.y, b.z, t.k);
    J.bins[i] = (uint16_t)bin;
    atomicAdd(&hist[bin], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nb; i += kThreads)
    J.counts[(uint64_t)i * J.nchunks + chunk] = hist[i];
}

// blockIdx.x = bin, blockIdx.y = job: scan of the bin's counts over the
// job's chunks; the bin total goes to base[bin] (scanned next).
__global__ void __launch_bounds__(kThreads) seg_scan_bins_kernel(const __grid_constant__ SegTable t) {
  const SegJob& J = t.jobs[blockIdx.y];
  const uint32_t total = block_scan_inplace(J.counts + (uint64_t)blockIdx.x * J.nchunks, J.nchunks);
  if (threadIdx.x == 0) J.base[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) seg_scan_totals_kernel(const __grid_constant__ SegTable t) {
  const SegJob& J = t.jobs[blockIdx.x];
  block_scan_inplace(J.base, (uint64_t)bins_for(t.k));
}

__global__ void __launch_bounds__(kThreads) seg_scatter_kernel(const __grid_constant__ SegTable t) {
  extern __shared__ uint32_t cursor[];
  const int nb = bins_for(t.k);
  const SegJob& J = t.jobs[seg_job_of(t, blockIdx.x)];
  const uint32_t chunk = blockIdx.x - J.first_chunk;
  for (int i = threadIdx.x; i < nb; i += kThreads)
    cursor[i] = J.base[i] + J.counts[(uint64_t)i * J.nchunks + chunk];
  __syncthreads();
  const uint64_t begin = (uint64_t)chunk * kChunk;
  const uint64_t end = begin + kChunk < J.n ? begin + kChunk : J.n;
  for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
    const uint32_t pos = atomicAdd(&cursor[J.bins[i]], 1u);
    J.perm[pos] = (uint32_t)i;
  }
}

}  // namespace

uint32_t seg_chunks(uint64_t n) { return (uint32_t)((n + kChunk - 1) / kChunk); }

size_t seg_job_scratch_bytes(uint64_t n, int k) {
  const uint64_t nb = bins_for(k);
  return align256(n * 4) + align256(n * 2) + align256(nb * seg_chunks(n) * 4) + align256(nb * 4);
}

void seg_job_carve(SegJob& j, void* scratch, uint64_t n, int k) {
  const uint64_t nb = bins_for(k);
  uint8_t* b = static_cast<uint8_t*>(scratch);
  j.perm = reinterpret_cast<uint32_t*>(b);
  b += align256(n * 4);
  j.bins = reinterpret_cast<uint16_t*>(b);
  b += align256(n * 2);
  j.counts = reinterpret_cast<uint32_t*>(b);
  b += align256(nb * seg_chunks(n) * 4);
  j.base = reinterpret_cast<uint32_t*>(b);
  j.n = (uint32_t)n;
  j.nchunks = seg_chunks(n);
}

cudaError_t reorder_jobs(const SegTable& t, cudaStream_t st) {
  if (t.n_jobs == 0 || t.total_chunks == 0) return cudaSuccess;
  if (t.k < 1 || t.k > kReorderMaxK || t.n_jobs > kSegMaxJobs) return cudaErrorInvalidValue;
  const int nb = bins_for(t.k);
  const size_t smem = (size_t)nb * 4;
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(seg_bin_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(seg_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    if (e != cudaSuccess) return e;
  }
  seg_bin_count_kernel<<<t.total_chunks, kThreads, smem, st>>>(t);
  seg_scan_bins_kernel<<<dim3(nb, t.n_jobs), kThreads, 0, st>>>(t);
  seg_scan_totals_kernel<<<t.n_jobs, kThreads, 0, st>>>(t);
  seg_scatter_kernel<<<t.total_chunks, kThreads, smem, st>>>(t);
  return cudaGetLastError();
}

size_t reorder_scratch_bytes(uint64_t n, int k) {
  const uint64_t nb = bins_for(k), blocks = blocks_for(n);
  return align256(n * 2) + align256(nb * blocks * 4) + 2 * align256(nb * 4);
}

cudaError_t reorder_rays(const bvhgpu_ray_t* rays, uint64_t n, int k, uint32_t* perm,
                         void* scratch, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (k < 1 || k > kReorderMaxK || n > 0xFFFFFFFFull) return cudaErrorInvalidValue;
  const int nb = bins_for(k);
  const uint64_t blocks = blocks_for(n);
  const Scratch s = carve(scratch, n, k);
  const size_t smem = (size_t)nb * 4;
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(bin_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
    if (e != cudaSuccess) return e;
  }
  bin_count_kernel<<<(unsigned)blocks, kThreads, smem, st>>>(rays, n, k, s, blocks);
  scan_bins_kernel<<<nb, kThreads, 0, st>>>(s, blocks);
  scan_totals_kernel<<<1, kThreads, 0, st>>>(s, nb);
  scatter_kernel<<<(unsigned)blocks, kThreads, smem, st>>>(n, k, s, blocks, perm);
  return cudaGetLastError();
}

}  // namespace dev
}  // namespace bvhgpu
