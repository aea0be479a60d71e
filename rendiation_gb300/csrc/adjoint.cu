// Differentiable closest hit: attribute-interpolation loss and its adjoint at
// frozen visibility, sm_103a.
//
// Forward (attr_forward_kernel): per ray, closest hit (the traversal of
// traverse.cuh), value = (1-u-v)*a[i0] + u*a[i1] + v*a[i2] with the hit
// triangle's vertex attributes, loss = (value - target)^2; a miss contributes
// nothing. The per-ray value and loss are written; the loss sum is accumulated
// per block and added once per block.
//
// Adjoint (attr_adjoint_kernel): the hit is recomputed by tracing the ray again
// instead of being stored by the forward pass. With r = 2 (value - target) * g
// (g = upstream gradient of the loss sum):
//   dL/da_k = r * w_k                       (w = (1-u-v, u, v))
//   gu = r (a1 - a0), gv = r (a2 - a0), gt = 0
// The hit solves o + t d = v0 + u e1 + v e2, i.e. M (t,u,v)^T = o - v0 with
// M = [-d | e1 | e2]. Differentiating at fixed visibility gives, with
// lambda = M^{-T} (gt, gu, gv):
//   dL/do = lambda, dL/dd = t lambda,
//   dL/dv0 = -(1-u-v) lambda, dL/dv1 = -u lambda, dL/dv2 = -v lambda,
// lambda = (gt (e1 x e2) + gu (e2 x -d) + gv (-d x e1)) / ((-d) . (e1 x e2)).
// Vertex gradients are accumulated as float4 (dx, dy, dz, dattr) per vertex
// with one vector atomicAdd per triangle corner. All quantities are in the
// instance's object space (world space for identity instances).
#include <cuda_runtime.h>

#include <cstdint>

#include "adjoint.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

struct HitGeom {
  uint32_t i0, i1, i2;
  float w0, u, v;
};

__device__ __forceinline__ HitGeom hit_vertices(const TraceParams& p, const AdjointParams& a, const RayCtx& R) {
  HitGeom h;
  const uint32_t tri = __ldg(p.redirect + R.best.k);
  h.i0 = __ldg(a.indices + 3 * (size_t)tri);
  h.i1 = __ldg(a.indices + 3 * (size_t)tri + 1);
  h.i2 = __ldg(a.indices + 3 * (size_t)tri + 2);
  h.u = R.best.u;
  h.v = R.best.v;
  h.w0 = 1.0f - h.u - h.v;
  return h;
}

template <int MODE>
__global__ void __launch_bounds__(128) attr_forward_kernel(TraceParams p, AdjointParams a) {
  extern __shared__ uint2 smem_stack[];
  __shared__ double block_sum[4];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float loss = 0.0f;
  if (i < a.count) {
    const float4* rp = a.rays + 2 * (size_t)i;
    const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
    RayCtx R;
    R.o = make_float3(r0.x, r0.y, r0.z);
    R.tmin = r0.w;
    R.d = make_float3(r1.x, r1.y, r1.z);
    R.tmax = r1.w;
    R.cull_mask = 0xFFu;
    R.ray_flags = 0u;
    bool bad;
    traverse_ray<MODE, false>(p, R, a.tlas_uniform, smem_stack + threadIdx.x, blockDim.x, bad);
    float value = 0.0f;
    if (R.best.have) {
      const HitGeom h = hit_vertices(p, a, R);
      value = h.w0 * __ldg(a.attributes + h.i0) + h.u * __ldg(a.attributes + h.i1) + h.v * __ldg(a.attributes + h.i2);
      const float diff = value - (a.targets ? __ldg(a.targets + i) : 0.0f);
      loss = diff * diff;
    }
    if (a.ray_value) a.ray_value[i] = value;
    if (a.ray_loss) a.ray_loss[i] = loss;
  }
  if (a.loss_sum) {
    double s = loss;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) block_sum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (uint32_t w = 0; w < (blockDim.x + 31) / 32; w++) t += block_sum[w];
      atomicAdd(a.loss_sum, t);
    }
  }
}

template <int MODE>
__global__ void __launch_bounds__(128) attr_adjoint_kernel(TraceParams p, AdjointParams a) {
  extern __shared__ uint2 smem_stack[];
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.count) return;
  const float4* rp = a.rays + 2 * (size_t)i;
  const float4 r0 = __ldg(rp), r1 = __ldg(rp + 1);
  RayCtx R;
  R.o = make_float3(r0.x, r0.y, r0.z);
  R.tmin = r0.w;
  R.d = make_float3(r1.x, r1.y, r1.z);
  R.tmax = r1.w;
  R.cull_mask = 0xFFu;
  R.ray_flags = 0u;
  bool bad;
  traverse_ray<MODE, false>(p, R, a.tlas_uniform, smem_stack + threadIdx.x, blockDim.x, bad);
  float3 go = make_float3(0.f, 0.f, 0.f), gd = go;
  if (R.best.have) {
    const HitGeom h = hit_vertices(p, a, R);
    const float a0 = __ldg(a.attributes + h.i0), a1 = __ldg(a.attributes + h.i1), a2 = __ldg(a.attributes + h.i2);
    const float value = h.w0 * a0 + h.u * a1 + h.v * a2;
    const float target = a.targets ? __ldg(a.targets + i) : 0.0f;
    const float r = 2.0f * (value - target) * a.grad_scale;
    const float gu = r * (a1 - a0), gv = r * (a2 - a0);
    // object-space ray of the hit instance and the triangle edges
    const InstanceRay ir = to_instance(p.tlas_data + R.best.inst, R.o, R.d, 0u);
    const float4* rec = p.tris + 4 * (size_t)R.best.k;
    const float4 q1 = __ldg(rec + 1), q2 = __ldg(rec + 2);
    const float3 e1 = make_float3(q1.x, q1.y, q1.z), e2 = make_float3(q2.x, q2.y, q2.z);
    const float3 nd = make_float3(-ir.d.x, -ir.d.y, -ir.d.z);
    const float3 c12 = cross3(e1, e2);
    const float det = dot3(nd, c12);
    const float3 b1 = cross3(e2, nd), b2 = cross3(nd, e1);
    const float inv = 1.0f / det;
    const float3 lam = make_float3((gu * b1.x + gv * b2.x) * inv, (gu * b1.y + gv * b2.y) * inv,
                                   (gu * b1.z + gv * b2.z) * inv);
    float4* g = reinterpret_cast<float4*>(a.grad_vertices);
    atomicAdd(g + h.i0, make_float4(-h.w0 * lam.x, -h.w0 * lam.y, -h.w0 * lam.z, r * h.w0));
    atomicAdd(g + h.i1, make_float4(-h.u * lam.x, -h.u * lam.y, -h.u * lam.z, r * h.u));
    atomicAdd(g + h.i2, make_float4(-h.v * lam.x, -h.v * lam.y, -h.v * lam.z, r * h.v));
    const float t_obj = R.best.t * ir.scaling;
    go = lam;
    gd = make_float3(t_obj * lam.x, t_obj * lam.y, t_obj * lam.z);
  }
  if (a.grad_ray_origin) {
    a.grad_ray_origin[3 * (size_t)i] = go.x;
    a.grad_ray_origin[3 * (size_t)i + 1] = go.y;
    a.grad_ray_origin[3 * (size_t)i + 2] = go.z;
  }
  if (a.grad_ray_direction) {
    a.grad_ray_direction[3 * (size_t)i] = gd.x;
    a.grad_ray_direction[3 * (size_t)i + 1] = gd.y;
    a.grad_ray_direction[3 * (size_t)i + 2] = gd.z;
  }
}

template <int MODE>
cudaError_t launch_attr_mode(const TraceParams& p, const AdjointParams& a, bool adjoint, uint32_t block,
                             cudaStream_t stream) {
  static bool done[2] = {false, false};
  if (!done[adjoint]) {
    cudaError_t e = adjoint ? cudaFuncSetAttribute(attr_adjoint_kernel<MODE>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024)
                            : cudaFuncSetAttribute(attr_forward_kernel<MODE>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    done[adjoint] = true;
  }
  const size_t smem = MODE != MODE_THREADED ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  const uint32_t grid = (a.count + block - 1) / block;
  if (adjoint) attr_adjoint_kernel<MODE><<<grid, block, smem, stream>>>(p, a);
  else attr_forward_kernel<MODE><<<grid, block, smem, stream>>>(p, a);
  return cudaGetLastError();
}

cudaError_t launch_attr(const TraceParams& p, const AdjointParams& a, int mode, bool adjoint, uint32_t block,
                        cudaStream_t stream) {
  if (a.count == 0) return cudaSuccess;
  if (block == 0) block = 128;
  if (mode == MODE_WIDE4) return launch_attr_mode<MODE_WIDE4>(p, a, adjoint, block, stream);
  if (mode == MODE_BINARY) return launch_attr_mode<MODE_BINARY>(p, a, adjoint, block, stream);
  return launch_attr_mode<MODE_THREADED>(p, a, adjoint, block, stream);
}

}  // namespace

cudaError_t launch_attr_forward(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream) {
  return launch_attr(p, a, mode, false, block, stream);
}

cudaError_t launch_attr_adjoint(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream) {
  return launch_attr(p, a, mode, true, block, stream);
}

}  // namespace rdn
