// Launch interface of the batched path kernels (paths.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "trace_kernels.h"

namespace rdn {

struct PathParams {
  const float4* primary_rays;  // 2 per ray
  const uint32_t* tlas_idx;    // nullable
  uint32_t count, tlas_uniform, max_bounces, rr_start, seed;
  float albedo, rr_survive;
  float2* out;                 // (radiance, depth | flags bits)
  uint32_t* segment_counts;    // nullable, max_bounces + 1 entries
  // scratch (paths_bind_scratch)
  uint32_t* queue_count;       // max_bounces + 1 counters: entries appended by bounce b
  uint32_t* work_counter;      // max_bounces + 1 counters
  void* rays_a;
  void* rays_b;
  void* state_a;
  void* state_b;
  // ray regrouping between bounces (sort_key != 0)
  uint32_t sort_key, key_bits;
  uint32_t* keys;
  uint32_t* idx;
  void* sort_scratch;
  // 0: warps trace 32 queued rays at a time; k > 0: dynamic fetch whenever k
  // lanes of a warp are idle (ordered walks only)
  uint32_t refill;
};

// Ray-sort keys: 0 none; 1 (scene, direction octant); 2 (scene, octant, 12-bit
// Morton code of the origin inside the scene's root box).
size_t paths_scratch_bytes(uint32_t count, uint32_t max_bounces, uint32_t sort_key);

void paths_bind_scratch(PathParams& q, void* scratch);
// Sets the kernel attributes and returns the persistent grid (not stream-ordered:
// call before any capture).
cudaError_t prepare_paths(const TraceParams& p, const PathParams& q, int mode, uint32_t block, int sm_count,
                          uint32_t* grid);
// Records the counter reset and one launch per bounce on `stream`.
cudaError_t record_paths(const TraceParams& p, const PathParams& q, int mode, uint32_t block, uint32_t grid,
                         cudaStream_t stream);

}  // namespace rdn
