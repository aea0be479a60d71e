// Launch interface of the differentiable closest-hit kernels (adjoint.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "trace_kernels.h"

namespace rdn {

struct AdjointParams {
  const float4* rays;         // 2 per ray
  uint32_t count, tlas_uniform;
  const uint32_t* indices;    // built vertex indices, 3 per triangle
  const float* vertices;      // built vertex positions, 3 per vertex
  const float* attributes;    // per vertex of the built vertex array
  const float* targets;       // per ray, nullable (0)
  float* ray_value;           // per ray, nullable
  float* ray_loss;            // per ray, nullable
  double* loss_sum;           // nullable
  float* grad_vertices;       // 4 per vertex: d/dx, d/dy, d/dz, d/dattr (accumulated)
  float* grad_ray_origin;     // 3 per ray, nullable
  float* grad_ray_direction;  // 3 per ray, nullable
  float grad_scale;           // upstream gradient of the loss sum
};

cudaError_t launch_attr_forward(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream);
cudaError_t launch_attr_adjoint(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream);

}  // namespace rdn
