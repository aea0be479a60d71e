// Device build of the triangle BVH forest (device_build.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "rdn_core.h"

namespace rdn {

// One triangle geometry of the build, in build order (host memory).
struct DeviceGeometry {
  const float* positions;   // 3 per vertex
  uint32_t vertex_count;
  const uint32_t* indices;  // nullptr = non-indexed (vertices taken three at a time)
  uint32_t triangle_count;
};

struct DeviceBlasOut {
  std::vector<Box> root_box;         // per geometry: box of its tree's root
  std::vector<uint32_t> tree_nodes;  // per geometry: nodes of its tree
  std::vector<uint32_t> root_code;   // per geometry: two-child code of the root
  std::vector<uint32_t> root_code4;  // per geometry: four-child code of the root
  uint64_t triangles = 0, nodes = 0, vertices = 0, sah_splits = 0, median_fallbacks = 0;
  uint32_t max_depth = 0, max_wide4_depth = 0;
  uint64_t bytes = 0;                // device bytes of the arrays written into DeviceBuilt
  double kernel_seconds = 0.0;       // span of the build on its stream (events), host round trips included
};

// Builds every geometry's tree with the reference's binned SAH (SAH::new(4),
// BalanceTree median fallback) on the current device and writes d.vertices,
// d.indices, d.indices_redirect, d.tri_records, d.tri_bvh_forest,
// d.wide_nodes, d.leaf_ranges and d.wide4_nodes. Trees are concatenated in
// geometry order exactly as the host build concatenates them. Returns "" or
// the error ("CUDA ..." for a failed CUDA call, "CUDA OOM ..." when device
// memory ran out); on error the arrays already written stay in `d` for the
// caller to free. Scratch memory comes from `pool` (stream-ordered; nullptr =
// the device's default pool) and goes back to it when the build returns.
std::string build_blas_device(const std::vector<DeviceGeometry>& geoms, uint32_t bin_size, uint32_t max_depth,
                              int sm_count, cudaMemPool_t pool, DeviceBuilt& d, DeviceBlasOut& out);

// Writes d.vertex_records[j] = the three vertices of sorted triangle j
// (d.indices_redirect, d.indices, d.vertices must be on the device), for j <
// d.indices_redirect.count, on `st`.
cudaError_t emit_vertex_records(const DeviceBuilt& d, cudaStream_t st);

}  // namespace rdn
