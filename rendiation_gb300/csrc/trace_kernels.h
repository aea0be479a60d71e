// Launch interface of the ray-query kernels (trace.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "rdn_core.h"

namespace rdn {

struct TraceParams {
  const float4* rays;  // 2 per ray (rdn_ray)
  rdn_hit* hits;
  rdn_hit_ext* hits_ext;
  const uint32_t* tlas_idx;
  uint32_t count, tlas_uniform, ray_flags, cull_mask, anyhit_mode, stack_depth;
  uint32_t n_binding, n_tlas_root;
  const uint32_t* tlas_binding;
  const uint32_t* tlas_bvh_root;
  const DeviceBVHNode* tlas_forest;
  const DeviceInstance* tlas_data;
  const TlasBounding* tlas_bounding;
  const BlasMetaInfo* blas_meta;
  const GeometryMetaInfo* tri_root;
  const DeviceBVHNode* tri_forest;
  const uint32_t* redirect;
  const float4* tris;   // 4 per triangle (TriRecord)
  const float4* wide;   // 4 per node (WideNode)
  const uint2* leaves;
  const uint32_t* geom_root_code;
  const float4* wide4;  // 8 per node (Wide4Node)
  const uint32_t* geom_root_code4;
  unsigned long long* counters;  // 4 x u64, used by counted launches
  uint32_t* error_word;          // bit 0 stack overflow, bit 1 bad tlas index, bit 2 iteration cap
  // 1: per-thread traversal stacks in local memory (ordered walks whose stack
  // fits kLocalStackEntries), 0: in shared memory
  uint32_t local_stack;
  // speculative ordered walk: lanes holding a leaf keep descending while more
  // than this many lanes of the warp are still looking for one (0 = until all
  // have one)
  uint32_t spec_threshold;
  const uint32_t* anyhit_mask;  // RDN_ANYHIT_PRIMITIVE_MASK: one bit per built triangle
  // iteration cap of the dynamic-fetch loops (0 = the built-in cap); on
  // reaching it a warp sets bit 2 of the error word and stops
  uint32_t iteration_limit;
  // 1: launch the kernels built for the watertight test (over `verts`, with
  // conservative box tests) instead of the reference's formula over `tris`
  // (which still gives the shading normal); kernels take the choice as a
  // template argument, so the reference-formula kernels carry no cost for it
  uint32_t watertight;
  const float4* verts;  // 3 per triangle (VertexRecord), sorted order
};

// 1 + 2 gamma_3 (gamma_n = n u / (1 - n u), u = 2^-24) rounded up to f32:
// 1 + 4 * 2^-23 (Ize, "Robust BVH Ray Traversal", JCGT 2013).
constexpr float kWatertightBoxFarScale = 1.000000476837158203125f;

// entries of a local-memory traversal stack
constexpr uint32_t kLocalStackEntries = 64;

// Traversal modes (template argument of every traversal kernel).
enum TraversalMode : int { MODE_THREADED = 0, MODE_BINARY = 1, MODE_WIDE4 = 2 };

// stack entries the mode needs per thread
uint32_t stack_entries(int mode, uint32_t max_binary_depth, uint32_t max_wide4_depth);

cudaError_t launch_trace(const TraceParams& p, int mode, bool counted, uint32_t block, cudaStream_t stream);

}  // namespace rdn
