// Internal types of librdn: host-side acceleration-structure system and the
// device layouts it uploads. Host float code here must be compiled with
// -ffp-contract=off so that every f32 value it precomputes equals the value the
// reference computes at run time (Rust never fuses multiply-adds).
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <initializer_list>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rdn.h"

namespace rdn {

static const uint32_t INVALID_NEXT = 0xFFFFFFFFu;

// Raises the dynamic shared-memory limit of the given kernels to 200 KB on the
// current device, once per device. Function attributes belong to a device's
// context, so `done` holds one bit per device (devices past 63 set it on every
// call); concurrent first calls may both set the attribute, which is harmless.
inline cudaError_t raise_smem_limit(std::atomic<uint64_t>& done, std::initializer_list<const void*> fns) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  for (const void* f : fns) {
    e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
  }
  done.fetch_or(bit, std::memory_order_release);
  return cudaSuccess;
}

struct f3 {
  float x, y, z;
};
struct Box {
  f3 lo, hi;
};

// ---- reference flattened layout (naive/mod.rs:22-71), bit-compatible ----
struct DeviceBVHNode {
  float aabb_min[3];
  uint32_t hit_next;
  float aabb_max[3];
  uint32_t miss_next;
  uint32_t content_range[2];
  uint32_t tail[2];
};
static_assert(sizeof(DeviceBVHNode) == 48, "48 B node");
struct DeviceInstance {
  float transform[16];
  float transform_inv[16];
  uint32_t instance_custom_index;
  uint32_t sbt_offset;
  uint32_t flags;
  uint32_t acceleration_structure_handle;
};
static_assert(sizeof(DeviceInstance) == 144, "144 B instance");
struct TlasBounding {
  float world_min[3];
  uint32_t mask;
  float world_max[3];
  uint32_t flags;
};
struct BlasMetaInfo {
  uint32_t tri_root_range[2];
};
struct GeometryMetaInfo {
  uint32_t bvh_root_idx, geometry_idx, primitive_start, geometry_flags;
};

// ---- GB300 layout ----
// Precomputed triangle, 64 B, in BVH-sorted order (same index space as the
// reference's content_range / indices_redirect):
//   q0 = (v0.xyz, n.x)  q1 = (e1.xyz, n.y)  q2 = (e2.xyz, n.z)  q3 = (uu, uv, vv, inv_d)
// with e1 = v1-v0, e2 = v2-v0, n = normalize(cross(e1,e2)), uu = e1.e1,
// uv = e1.e2, vv = e2.e2, inv_d = 1/(uv*uv - uu*vv): exactly the f32 values the
// reference's intersect_ray_triangle_cpu computes per test (geometry/mod.rs:115-144).
struct TriRecord {
  float q[16];
};
static_assert(sizeof(TriRecord) == 64, "64 B triangle");
// The three vertices of a triangle, 48 B, in the same sorted order, for the
// watertight test (which must see the shared vertex values themselves, not
// edges rounded from them): q0 = (v0.xyz, v1.x) q1 = (v1.yz, v2.xy) q2 = (v2.z, 0, 0, 0).
struct VertexRecord {
  float q[12];
};
static_assert(sizeof(VertexRecord) == 48, "48 B vertex record");
// Two-child node, 64 B: children's boxes and child codes.
//   w0 = (c0.lo.x, c0.lo.y, c0.lo.z, c0.hi.x)  w1 = (c0.hi.y, c0.hi.z, c1.lo.x, c1.lo.y)
//   w2 = (c1.lo.z, c1.hi.x, c1.hi.y, c1.hi.z)  w3 = (code0, code1, 0, 0)
// code: bit 31 clear = index of a child WideNode, set = index of a leaf range.
struct WideNode {
  float w[12];
  uint32_t code[4];
};
static_assert(sizeof(WideNode) == 64, "64 B node");
static const uint32_t LEAF_BIT = 0x80000000u;
// Four-child node, 128 B, children's boxes as SoA rows:
//   lo_x[4] lo_y[4] lo_z[4] hi_x[4] hi_y[4] hi_z[4] code[4] pad[4]
// code: bit 31 clear = index of a child Wide4Node, set = index of a leaf range,
// EMPTY_SLOT = unused slot. Children are binary-tree nodes collapsed from the
// reference's SAH tree (the inner child with the largest surface area is opened
// until four slots are used); every child box is an exact reference node box.
struct Wide4Node {
  float lo_x[4], lo_y[4], lo_z[4], hi_x[4], hi_y[4], hi_z[4];
  uint32_t code[4];
  uint32_t pad[4];
};
static_assert(sizeof(Wide4Node) == 128, "128 B node");
static const uint32_t EMPTY_SLOT = 0xFFFFFFFFu;

struct GeometrySource {
  uint32_t type;
  uint32_t flags;
  std::vector<float> positions;
  bool indexed;
  std::vector<uint32_t> indices;
};
struct InstanceSource {
  float transform[16];
  uint32_t custom_index, mask, sbt_offset, flags, blas_handle;
};

// Host copy of everything a build produces.
struct HostBuilt {
  // reference layout
  std::vector<uint32_t> tlas_binding;
  std::vector<uint32_t> tlas_bvh_root;
  std::vector<DeviceBVHNode> tlas_bvh_forest;
  std::vector<DeviceInstance> tlas_data;
  std::vector<TlasBounding> tlas_bounding;
  std::vector<BlasMetaInfo> blas_meta_info;
  std::vector<GeometryMetaInfo> tri_bvh_root;
  std::vector<DeviceBVHNode> tri_bvh_forest;
  std::vector<uint32_t> indices_redirect;
  std::vector<uint32_t> indices;
  std::vector<float> vertices;
  // GB300 layout
  std::vector<TriRecord> tri_records;
  std::vector<WideNode> wide_nodes;
  std::vector<uint32_t> leaf_ranges;  // 2 per leaf: [start, end)
  std::vector<uint32_t> geom_root_code;  // per tri_bvh_root entry
  std::vector<Wide4Node> wide4_nodes;
  std::vector<uint32_t> geom_root_code4;  // per tri_bvh_root entry
  uint32_t max_blas_depth = 0;
  uint32_t max_wide4_depth = 0;
  uint64_t sah_splits = 0, median_fallbacks = 0;
  // sizes of the reference-layout arrays (kept when they live on the device only)
  uint64_t n_triangles = 0, n_nodes = 0, n_indices = 0, n_vertices = 0;
  // true: the triangle forest, geometry arrays and GB300 node layouts were
  // built on the device and exist only there
  bool device_blas = false;
  uint64_t device_bytes = 0;
};

template <class T>
struct DevBuf {
  T* ptr = nullptr;
  size_t count = 0;
};

struct DeviceBuilt {
  DevBuf<uint32_t> tlas_binding, tlas_bvh_root, indices_redirect, leaf_ranges, geom_root_code, indices;
  DevBuf<float> vertices;
  DevBuf<DeviceBVHNode> tlas_bvh_forest, tri_bvh_forest;
  DevBuf<DeviceInstance> tlas_data;
  DevBuf<TlasBounding> tlas_bounding;
  DevBuf<BlasMetaInfo> blas_meta_info;
  DevBuf<GeometryMetaInfo> tri_bvh_root;
  DevBuf<TriRecord> tri_records;
  DevBuf<VertexRecord> vertex_records;
  DevBuf<WideNode> wide_nodes;
  DevBuf<Wide4Node> wide4_nodes;
  DevBuf<uint32_t> geom_root_code4;
  uint32_t max_blas_depth = 0;
  uint32_t max_wide4_depth = 0;
  uint64_t vertex_count = 0;
  uint64_t bytes = 0;
};

struct BuildOptions {
  uint32_t blas_bin_size = 2, blas_max_depth = 50, tlas_bin_size = 10, tlas_max_depth = 50, host_threads = 0;
  uint32_t device_build = 0;
};

// Builds the whole structure from the sources (reference: NaiveSahBvhSource::build,
// naive/mod.rs:322-494). Returns an empty string on success, else the error.
std::string build_host(const std::vector<std::unique_ptr<std::vector<GeometrySource>>>& blas,
                       const std::vector<std::unique_ptr<std::vector<InstanceSource>>>& tlas,
                       const std::vector<uint32_t>& binding, const BuildOptions& opt, HostBuilt& out);

// Same structure with the triangle trees built on the current device
// (device_build.cu): the device arrays of the BLAS forest are written into
// `d`, the small per-tree and TLAS arrays into `out`.
std::string build_with_device_blas(const std::vector<std::unique_ptr<std::vector<GeometrySource>>>& blas,
                                   const std::vector<std::unique_ptr<std::vector<InstanceSource>>>& tlas,
                                   const std::vector<uint32_t>& binding, const BuildOptions& opt, int sm_count,
                                   cudaMemPool_t pool, HostBuilt& out, DeviceBuilt& d, double* device_seconds);

}  // namespace rdn

struct rdn_ctx {
  std::mutex lock;
  int device = -1;
  int sm_count = 0;
  std::vector<std::unique_ptr<std::vector<rdn::GeometrySource>>> blas;
  std::vector<std::unique_ptr<std::vector<rdn::InstanceSource>>> tlas;
  std::vector<uint32_t> binding;
  rdn::BuildOptions opts;
  bool dirty = true;
  std::unique_ptr<rdn::HostBuilt> host;
  rdn::DeviceBuilt dev;
  // 16 words: 0-7 four u64 trace counters, 8 error word, 12 work counter of
  // the differentiable paths, 13 path tracer's pixel fetch. Calls of one
  // context that use the same word must not overlap on the GPU.
  uint32_t* d_counters = nullptr;
  uint32_t iteration_limit = 0;     // cap of the dynamic-fetch loops (0 = built-in)
  cudaMemPool_t build_pool = nullptr;  // stream-ordered scratch of device builds, kept for the next build
  double build_seconds = 0.0, upload_seconds = 0.0, device_seconds = 0.0;
  std::string err;
};
