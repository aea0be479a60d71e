// Launch interface of the wavefront kernels (wavefront.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "trace_kernels.h"

namespace rdn {

// Per-pixel result, 32 B (rdn_pixel_result in include/rdn.h).
struct PixelResult {
  uint32_t primary_prim;
  float primary_t;
  uint32_t bounce_prim;
  float bounce_t;
  uint32_t primary_flags;
  uint32_t light;
  float direct;
  uint32_t primary_instance;
};
static_assert(sizeof(PixelResult) == 32, "32 B pixel");

struct WavefrontParams {
  float3 origin, forward, right, up, light;
  float tan_half, aspect;
  uint32_t width, height, sample_index, tlas;
  PixelResult* out;
  uint32_t* ray_counts;  // nullable: [primary, shadow, bounce]
  // scratch (wavefront_bind_scratch)
  uint32_t* queue_count;   // start of the 64 B the primary launch zeroes
  // bounce-queue bins (inside those 64 B): low word the grazing rays at the
  // queue's front, high word the steep rays at its back; their sum is the
  // count of shadow rays and of bounce rays
  unsigned long long* bins;
  uint32_t* tile_counter;  // primary tiles claimed (inside the 64 B the launch zeroes at queue_count)
  uint32_t* work_counter;
  void* shadow_rays;
  void* bounce_rays;
  uint32_t* shadow_pixel;
  uint32_t* bounce_pixel;
  // secondary schedule: 0 = batches of 32 per warp; k = 1..32: a warp refills
  // its idle lanes whenever at least k are idle (ordered walks only)
  uint32_t refill;
  // 1: traversal stacks in local memory (ordered walks, trees up to the
  // local stack's depth); 0: in shared memory
  uint32_t local_stack;
  // register budget of the local-stack kernels: 0 default (64), 1 = 72, 2 = 56
  uint32_t register_tier;
  // the launch covers rows [row0, row0 + height) of a frame of frame_height rows
  uint32_t row0, frame_height;
};

size_t wavefront_scratch_bytes(uint32_t width, uint32_t height);
void wavefront_bind_scratch(WavefrontParams& w, void* scratch);
// phases: bit 0 primary kernel, bit 1 secondary kernel (0 = both).
cudaError_t launch_wavefront(const TraceParams& p, const WavefrontParams& w, int mode, uint32_t block,
                             int sm_count, uint32_t phases, cudaStream_t stream);

// Looks up the device address of the library's static queue array on
// `device` (which must be current) and caches it; called when a context is
// created for the device.
cudaError_t wavefront_static_prepare(int device);
// Same launch as launch_wavefront with the queues in that static array;
// `device` must be current.
cudaError_t launch_wavefront_static(const TraceParams& p, WavefrontParams w, int mode, uint32_t block,
                                    int sm_count, uint32_t phases, int device, cudaStream_t stream);

}  // namespace rdn
