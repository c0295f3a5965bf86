// Ray reordering by direction before a trace (see reorder.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bvhgpu.h"

namespace bvhgpu {
namespace dev {

constexpr int kReorderMaxK = 32;  // bins per face side: 6 * 32^2 + 1 bins at most

// Device scratch bytes for reordering n rays into 6 k^2 + 1 bins.
size_t reorder_scratch_bytes(uint64_t n, int k);

// Writes into perm[0..n) the input ray indices grouped by direction bin;
// `scratch` holds reorder_scratch_bytes(n, k) bytes (256-byte aligned).
// Asynchronous on s.
cudaError_t reorder_rays(const bvhgpu_ray_t* rays, uint64_t n, int k, uint32_t* perm,
                         void* scratch, cudaStream_t s);

// ---- per-job reordering for the batched (multi-scene) trace ---------------
// The same counting sort for many ray batches in four launches in all: each
// job's rays are cut into chunks of 4096, chunks of all jobs form one grid,
// and every job gets its own bins, so a job's permutation only moves its own
// rays. The tables travel in the kernel parameters (no host copies, so the
// launches can be recorded in a CUDA graph).
constexpr int kSegMaxJobs = 192;

struct SegJob {
  const bvhgpu_ray_t* rays;
  uint32_t* perm;        // n: the job's ray indices in bin order
  uint16_t* bins;        // n
  uint32_t* counts;      // bins * nchunks, bin-major
  uint32_t* base;        // bins: first position of each bin in perm
  uint32_t n;
  uint32_t first_chunk;  // index of the job's first chunk in the grid
  uint32_t nchunks;
  uint32_t pad;
};

struct SegTable {
  SegJob jobs[kSegMaxJobs];
  int n_jobs;
  int k;
  uint32_t total_chunks;
};

// Scratch bytes of one job (perm, bins, counts, base; 256-byte aligned parts)
// and the carving of a job's scratch into its SegJob pointers.
size_t seg_job_scratch_bytes(uint64_t n, int k);
void seg_job_carve(SegJob& j, void* scratch, uint64_t n, int k);
uint32_t seg_chunks(uint64_t n);

cudaError_t reorder_jobs(const SegTable& t, cudaStream_t s);

}  // namespace dev
}  // namespace bvhgpu
