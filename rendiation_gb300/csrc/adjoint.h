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
  uint32_t* hit_tri;          // per ray, nullable: built triangle of the hit or ~0 (written by the forward)
  uint32_t* hit_inst;         // per ray, nullable: instance slot of the hit (written by the forward)
  bool from_record;           // adjoint: differentiate the recorded hits instead of tracing again
  float4* hit_out;            // hit query forward: (t, u, v, value) per ray, nullable
  const float4* grad_hit;     // hit query adjoint: (dL/dt, dL/du, dL/dv, dL/dvalue) per ray
};

// Multi-segment, multi-scene form: every path is a primary ray (its own TLAS
// index) followed by up to segments-1 cosine bounces; each segment's hit adds
// (value - target)^2. Bounce rays depend on the hit like the path executor's
// (facing normal, offset origin, sampler xxhash32(id, k, seed)); the adjoint
// treats each segment's ray as fixed (gradients do not flow through the bounce
// directions) and either recomputes every hit by tracing the path again or,
// with from_record, differentiates the hits the forward recorded in seg_tri,
// seg_inst and seg_rays.
struct PathAdjointParams {
  const float4* rays;         // 2 per path
  const uint32_t* tlas_idx;   // per path, nullable
  uint32_t count, tlas_uniform, segments, seed;
  const uint32_t* indices;
  const float* vertices;
  const float* attributes;
  const float* targets;       // segments per path, nullable (0)
  float* values;              // segments per path, nullable
  double* loss_sum;           // nullable
  float* grad_vertices;       // 4 per vertex (adjoint)
  uint32_t* seg_tri;          // segments per path, nullable: triangle index of each segment's hit (or ~0)
  float4* seg_rays;           // 2 float4 per segment per path, nullable
  uint32_t* seg_inst;         // segments per path, nullable: instance slot of each segment's hit
  bool from_record;           // adjoint: use seg_tri / seg_inst / seg_rays instead of tracing again
  float grad_scale;
  uint32_t* work_counter;     // persistent work distribution (reset by the launcher)
};

cudaError_t launch_attr_paths(const TraceParams& p, const PathAdjointParams& a, int mode, bool adjoint,
                              uint32_t block, int sm_count, cudaStream_t stream);

// Differentiable hit query: forward writes (t, u, v, value) per ray; adjoint
// scatters the caller's upstream gradients of those to the vertices and rays.
cudaError_t launch_hit_diff(const TraceParams& p, const AdjointParams& a, int mode, bool adjoint, uint32_t block,
                            int sm_count, cudaStream_t stream);

cudaError_t launch_attr_forward(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                cudaStream_t stream);
cudaError_t launch_attr_adjoint(const TraceParams& p, const AdjointParams& a, int mode, uint32_t block,
                                int sm_count, cudaStream_t stream);

}  // namespace rdn
