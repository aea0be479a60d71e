// Fused ambient-occlusion frame for sm_103a: the reference AO renderer's ray
// generation, primary closest hit, occlusion ray and miss shaders
// (feature/ao.rs:193-296) as one kernel, one thread per pixel, warps over 4x8
// pixel tiles. It computes what the task-graph form of the same pipeline
// computes, without the task pools. Built with -fmad=false: see ao.cuh.
#include <cuda_runtime.h>

#include <cstdint>

#include "ao.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) ao_kernel(TraceParams P, AoEnv A) {
  RDN_TRAVERSAL_STACK(LOCAL);
  uint32_t x, y;
  if (!ao_pixel(A, blockIdx.x * blockDim.x + threadIdx.x, x, y)) return;
  float3 o, d;
  ao_camera_ray(A, x, y, o, d);
  RayCtx R;
  R.o = o;
  R.d = d;
  R.tmin = F32_EPSILON;
  R.tmax = F32_MAX;
  R.ray_flags = RAY_FLAG_CULL_BACK;
  R.cull_mask = 0xFFFFFFFFu;
  bool bad;
  traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, A.tlas, stack_ptr, stack_stride, bad);
  float payload = 1.0f;  // miss shader
  if (R.best.have) {
    const float3 hit = o + d * R.best.t;
    const float3 n =
        ao_shading_normal(A, P.tlas_data + R.best.inst, __ldg(P.redirect + R.best.k), R.best.u, R.best.v, o, hit);
    RayCtx S;
    S.o = hit;
    S.d = ao_direction(n, ao_sample(A));
    S.tmin = AO_TEST_MIN;
    S.tmax = AO_TEST_MAX;
    S.ray_flags = RAY_FLAG_END_SEARCH;
    S.cull_mask = 0xFFFFFFFFu;
    bool bad2;
    traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, S, A.tlas, stack_ptr, stack_stride, bad2);
    bad |= bad2;
    payload = S.best.have ? 0.0f : 1.0f;  // secondary closest hit: occluded
  }
  if (bad) atomicOr(P.error_word, 2u);
  ao_count(A, 0, true);
  ao_count(A, 1, R.best.have);
  ao_accumulate(A, y * A.width + x, payload);
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_variant_wt(const TraceParams& p, const AoEnv& a, cudaStream_t st) {
  const uint32_t block = a.block ? a.block : 128;
  const uint32_t grid = (ao_dispatch_count(a.width, a.height) + block - 1) / block;
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t e = raise_smem_limit(attr_done, {(const void*)ao_kernel<MODE, LOCAL, WT>});
  if (e != cudaSuccess) return e;
  ao_kernel<MODE, LOCAL, WT><<<grid, block, smem, st>>>(p, a);
  return cudaGetLastError();
}

template <int MODE, bool LOCAL>
cudaError_t launch_variant(const TraceParams& p, const AoEnv& a, cudaStream_t st) {
  return p.watertight ? launch_variant_wt<MODE, LOCAL, true>(p, a, st) : launch_variant_wt<MODE, LOCAL, false>(p, a, st);
}

__global__ void ao_advance_kernel(uint32_t* counter) { *counter += 1u; }

}  // namespace

cudaError_t launch_ao_advance(uint32_t* counter, cudaStream_t st) {
  ao_advance_kernel<<<1, 1, 0, st>>>(counter);
  return cudaGetLastError();
}

cudaError_t launch_ao(const TraceParams& p, const AoEnv& a, int mode, cudaStream_t st) {
  if (a.width == 0 || a.height == 0) return cudaSuccess;
  if (mode == MODE_WIDE4)
    return p.local_stack ? launch_variant<MODE_WIDE4, true>(p, a, st) : launch_variant<MODE_WIDE4, false>(p, a, st);
  if (mode == MODE_BINARY)
    return p.local_stack ? launch_variant<MODE_BINARY, true>(p, a, st)
                         : launch_variant<MODE_BINARY, false>(p, a, st);
  return launch_variant<MODE_THREADED, false>(p, a, st);
}

}  // namespace rdn
