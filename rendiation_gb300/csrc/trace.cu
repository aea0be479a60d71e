// Batch ray-query kernel for sm_103a (rdn_trace): one thread per ray, the
// traversal of traverse.cuh, one 16 B hit (+ optional 16 B context) out.
// Built with -fmad=false: see traverse.cuh.
#include <cuda_runtime.h>

#include <cstdint>

#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

template <int MODE, bool COUNT, bool LOCAL, bool WT>
__global__ void __launch_bounds__(256) trace_kernel(TraceParams p) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  // Lanes past the ray count stay alive (with zero counts) until the counter
  // reduction, which reads every lane of the warp: block sizes are multiples of 32.
  unsigned long long nv = 0, tt = 0, th = 0, bt = 0;
  if (i < p.count) {
    const float4* rp = p.rays + 2 * (size_t)i;
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    RayCtx R;
    R.o = make_float3(r0.x, r0.y, r0.z);
    R.tmin = r0.w;
    R.d = make_float3(r1.x, r1.y, r1.z);
    R.tmax = r1.w;
    R.cull_mask = p.cull_mask;
    R.ray_flags = p.ray_flags;
    const uint32_t tidx = p.tlas_idx ? __ldg(p.tlas_idx + i) : p.tlas_uniform;
    bool bad;
    traverse_ray<MODE, COUNT, BuiltinAnyHit, WT>(p, R, tidx, stack_ptr, stack_stride, bad);

    float4 out;
    uint4 ext;
    if (R.best.have) {
      const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + R.best.geom_slot));
      const uint32_t prim = __ldg(p.redirect + R.best.k) - gm.z;
      out = make_float4(R.best.t, R.best.u, R.best.v, __uint_as_float(prim));
      ext = make_uint4(gm.y, R.best.inst, __ldg(&p.tlas_data[R.best.inst].instance_custom_index),
                       (R.best.s < 0.0f) ? 0xFFu : 0xFEu);
    } else {
      out = make_float4(R.tmax, 0.0f, 0.0f, __uint_as_float(INVALID_NEXT));
      ext = make_uint4(INVALID_NEXT, INVALID_NEXT, INVALID_NEXT, 0u);
    }
    reinterpret_cast<float4*>(p.hits)[i] = out;
    if (p.hits_ext) reinterpret_cast<uint4*>(p.hits_ext)[i] = ext;
    if (bad) atomicOr(p.error_word, 2u);
    if (COUNT) {
      nv = R.node_visits;
      tt = R.tri_tests;
      th = R.tri_hits;
      bt = bad ? 1ull : 0ull;
    }
  }
  if (COUNT) {
    __syncwarp();
    for (int off = 16; off > 0; off >>= 1) {
      nv += __shfl_down_sync(0xffffffffu, nv, off);
      tt += __shfl_down_sync(0xffffffffu, tt, off);
      th += __shfl_down_sync(0xffffffffu, th, off);
      bt += __shfl_down_sync(0xffffffffu, bt, off);
    }
    if ((threadIdx.x & 31) == 0 && (nv | tt | th | bt)) {
      atomicAdd(p.counters + 0, nv);
      atomicAdd(p.counters + 1, tt);
      atomicAdd(p.counters + 2, th);
      atomicAdd(p.counters + 3, bt);
    }
  }
}

}  // namespace

uint32_t stack_entries(int mode, uint32_t max_binary_depth, uint32_t max_wide4_depth) {
  uint32_t d = mode == MODE_WIDE4 ? 3 * max_wide4_depth + 1 : (mode == MODE_BINARY ? max_binary_depth + 1 : 0);
  d = (d + 3) & ~3u;
  return d < 8 ? 8 : d;
}

namespace {
template <int MODE, bool COUNT, bool LOCAL, bool WT>
cudaError_t launch_trace_wt(const TraceParams& p, uint32_t block, uint32_t grid, cudaStream_t stream) {
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t e = raise_smem_limit(attr_done, {(const void*)trace_kernel<MODE, COUNT, LOCAL, WT>});
  if (e != cudaSuccess) return e;
  trace_kernel<MODE, COUNT, LOCAL, WT><<<grid, block, smem, stream>>>(p);
  return cudaGetLastError();
}

template <int MODE, bool COUNT, bool LOCAL>
cudaError_t launch_trace_variant(const TraceParams& p, uint32_t block, uint32_t grid, cudaStream_t stream) {
  return p.watertight ? launch_trace_wt<MODE, COUNT, LOCAL, true>(p, block, grid, stream)
                      : launch_trace_wt<MODE, COUNT, LOCAL, false>(p, block, grid, stream);
}
}  // namespace

cudaError_t launch_trace(const TraceParams& p, int mode, bool counted, uint32_t block, cudaStream_t stream) {
  if (p.count == 0) return cudaSuccess;
  if (block == 0) block = 64;
  const uint32_t grid = (p.count + block - 1) / block;
  const bool local = p.local_stack != 0;
  if (mode == MODE_WIDE4) {
    if (counted) return launch_trace_variant<MODE_WIDE4, true, false>(p, block, grid, stream);
    return local ? launch_trace_variant<MODE_WIDE4, false, true>(p, block, grid, stream)
                 : launch_trace_variant<MODE_WIDE4, false, false>(p, block, grid, stream);
  }
  if (mode == MODE_BINARY) {
    if (counted) return launch_trace_variant<MODE_BINARY, true, false>(p, block, grid, stream);
    return local ? launch_trace_variant<MODE_BINARY, false, true>(p, block, grid, stream)
                 : launch_trace_variant<MODE_BINARY, false, false>(p, block, grid, stream);
  }
  return counted ? launch_trace_variant<MODE_THREADED, true, false>(p, block, grid, stream)
                 : launch_trace_variant<MODE_THREADED, false, false>(p, block, grid, stream);
}

}  // namespace rdn
