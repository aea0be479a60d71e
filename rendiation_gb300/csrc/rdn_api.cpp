// C ABI of librdn (include/rdn.h): the acceleration-structure system
// (GPUAccelerationStructureSystemProvider, shader/ray-tracing/src/api/backend.rs:120-142,
// implemented by NaiveSahBVHSystem, .../geometry/naive/mod.rs:496-609) and the
// batch trace entry points.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <exception>
#include <new>

#include <nvtx3/nvToolsExt.h>

#include "rdn_core.h"
#include "trace_kernels.h"
#include "adjoint.h"
#include "device_build.h"
#include "parallel.h"
#include "paths.h"
#include "pt.h"
#include "task_graph.h"
#include "wavefront.h"

using rdn::DevBuf;

namespace {

// NVTX range around an entry point (a no-op unless a profiler is attached):
// the timeline shows build / trace / frame / paths / differentiable phases.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
};

rdn_status fail(rdn_ctx* c, rdn_status code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

rdn_status cuda_fail(rdn_ctx* c, cudaError_t e, const char* what) {
  return fail(c, e == cudaErrorMemoryAllocation ? RDN_ERR_OOM : RDN_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
void free_buf(DevBuf<T>& b) {
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.count = 0;
}

void free_device(rdn::DeviceBuilt& d) {
  free_buf(d.tlas_binding);
  free_buf(d.tlas_bvh_root);
  free_buf(d.indices_redirect);
  free_buf(d.leaf_ranges);
  free_buf(d.geom_root_code);
  free_buf(d.indices);
  free_buf(d.vertices);
  free_buf(d.tlas_bvh_forest);
  free_buf(d.tri_bvh_forest);
  free_buf(d.tlas_data);
  free_buf(d.tlas_bounding);
  free_buf(d.blas_meta_info);
  free_buf(d.tri_bvh_root);
  free_buf(d.tri_records);
  free_buf(d.vertex_records);
  free_buf(d.wide_nodes);
  free_buf(d.wide4_nodes);
  free_buf(d.geom_root_code4);
  d.bytes = 0;
}

// Uploads one array; an empty array still gets one zeroed element, as the
// reference's create_gpu_buffer does (naive/mod.rs:401-416).
template <class T>
cudaError_t upload(DevBuf<T>& dst, const std::vector<T>& src, uint64_t& bytes) {
  const size_t n = src.empty() ? 1 : src.size();
  cudaError_t e = cudaMalloc(&dst.ptr, n * sizeof(T));
  if (e != cudaSuccess) return e;
  dst.count = src.size();
  bytes += n * sizeof(T);
  if (src.empty()) return cudaMemset(dst.ptr, 0, sizeof(T));
  return cudaMemcpy(dst.ptr, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

rdn_status do_build(rdn_ctx* c) {
  auto t0 = std::chrono::steady_clock::now();
  auto hb = std::make_unique<rdn::HostBuilt>();
  std::string err;
  const bool on_device = c->opts.device_build != 0;
  c->device_seconds = 0.0;
  if (on_device) {
    if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot build on a device");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    e = cudaDeviceSynchronize();  // no trace may still read the buffers being replaced
    if (e != cudaSuccess) return cuda_fail(c, e, "synchronize before build");
    free_device(c->dev);
    if (!c->build_pool) {
      // the build's scratch (about 200 B per triangle) stays in this pool
      // between builds, so that a rebuild allocates nothing from the driver
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = c->device;
      e = cudaMemPoolCreate(&c->build_pool, &props);
      if (e != cudaSuccess) {
        c->build_pool = nullptr;
        return cuda_fail(c, e, "cudaMemPoolCreate");
      }
      uint64_t keep = ~0ull;
      e = cudaMemPoolSetAttribute(c->build_pool, cudaMemPoolAttrReleaseThreshold, &keep);
      if (e != cudaSuccess) return cuda_fail(c, e, "cudaMemPoolSetAttribute");
    }
  }
  try {
    err = on_device ? rdn::build_with_device_blas(c->blas, c->tlas, c->binding, c->opts, c->sm_count, c->build_pool,
                                                  *hb, c->dev, &c->device_seconds)
                    : rdn::build_host(c->blas, c->tlas, c->binding, c->opts, *hb);
  } catch (const std::bad_alloc&) {
    if (on_device) free_device(c->dev);
    return fail(c, RDN_ERR_OOM, "host allocation failed during build");
  } catch (const std::exception& ex) {
    if (on_device) free_device(c->dev);
    return fail(c, RDN_ERR_INVALID_ARG, ex.what());
  }
  if (!err.empty()) {
    if (on_device) free_device(c->dev);
    const rdn_status code = err.rfind("CUDA OOM ", 0) == 0 ? RDN_ERR_OOM
                            : err.rfind("CUDA ", 0) == 0   ? RDN_ERR_CUDA
                                                           : RDN_ERR_INVALID_HANDLE;
    return fail(c, code, err);
  }
  auto t1 = std::chrono::steady_clock::now();
  c->build_seconds = std::chrono::duration<double>(t1 - t0).count();
  c->upload_seconds = 0.0;
  if (c->device >= 0) {
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
    if (!on_device) {
      e = cudaDeviceSynchronize();  // no trace may still read the buffers being replaced
      if (e != cudaSuccess) return cuda_fail(c, e, "synchronize before upload");
      free_device(c->dev);
    }
    rdn::DeviceBuilt& d = c->dev;
    uint64_t bytes = hb->device_bytes;
#define UP(field, src)                                      \
  e = upload(d.field, hb->src, bytes);                      \
  if (e != cudaSuccess) {                                   \
    free_device(d);                                         \
    return cuda_fail(c, e, "upload " #src);                 \
  }
    UP(tlas_binding, tlas_binding)
    UP(tlas_bvh_root, tlas_bvh_root)
    UP(tlas_bvh_forest, tlas_bvh_forest)
    UP(tlas_data, tlas_data)
    UP(tlas_bounding, tlas_bounding)
    UP(blas_meta_info, blas_meta_info)
    UP(tri_bvh_root, tri_bvh_root)
    UP(geom_root_code, geom_root_code)
    UP(geom_root_code4, geom_root_code4)
    if (!hb->device_blas) {
      UP(tri_bvh_forest, tri_bvh_forest)
      UP(indices_redirect, indices_redirect)
      UP(tri_records, tri_records)
      UP(wide_nodes, wide_nodes)
      UP(leaf_ranges, leaf_ranges)
      UP(indices, indices)
      UP(vertices, vertices)
      UP(wide4_nodes, wide4_nodes)
    }
#undef UP
    {
      // vertices of every sorted triangle, for the watertight test, gathered on the device
      const size_t n = d.indices_redirect.count;
      e = cudaMalloc(&d.vertex_records.ptr, (n ? n : 1) * sizeof(rdn::VertexRecord));
      if (e == cudaSuccess) {
        d.vertex_records.count = n;
        bytes += (n ? n : 1) * sizeof(rdn::VertexRecord);
        e = n ? rdn::emit_vertex_records(d, 0) : cudaMemset(d.vertex_records.ptr, 0, sizeof(rdn::VertexRecord));
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(0);
      if (e != cudaSuccess) {
        free_device(d);
        return cuda_fail(c, e, "vertex records");
      }
    }
    d.max_blas_depth = hb->max_blas_depth;
    d.max_wide4_depth = hb->max_wide4_depth;
    d.vertex_count = hb->n_vertices;
    d.bytes = bytes;
    c->upload_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
  }
  c->host = std::move(hb);
  c->dirty = false;
  return RDN_OK;
}

// The walk order of a traversal value (RDN_INTERSECT_WATERTIGHT may be OR-ed in).
uint32_t order_of(uint32_t traversal) { return traversal & ~RDN_INTERSECT_WATERTIGHT; }
bool traversal_ok(uint32_t traversal) { return order_of(traversal) <= RDN_TRAVERSAL_ORDERED_WIDE; }

int mode_of(uint32_t traversal) {
  if (order_of(traversal) == RDN_TRAVERSAL_REFERENCE) return rdn::MODE_THREADED;
  if (order_of(traversal) == RDN_TRAVERSAL_ORDERED_WIDE) return rdn::MODE_WIDE4;
  return rdn::MODE_BINARY;
}

rdn_status fill_params(rdn_ctx* c, const rdn_trace_desc* desc, rdn::TraceParams& p) {
  const rdn::DeviceBuilt& d = c->dev;
  std::memset(&p, 0, sizeof(p));
  p.rays = reinterpret_cast<const float4*>(desc->rays);
  p.hits = desc->hits;
  p.hits_ext = desc->hits_ext;
  p.tlas_idx = desc->tlas_idx;
  p.count = desc->count;
  p.tlas_uniform = desc->tlas_uniform;
  p.ray_flags = desc->ray_flags;
  p.cull_mask = desc->cull_mask;
  p.anyhit_mode = desc->anyhit_mode;
  p.anyhit_mask = desc->anyhit_mask;
  p.stack_depth = rdn::stack_entries(mode_of(desc->traversal), d.max_blas_depth, d.max_wide4_depth);
  p.n_binding = (uint32_t)d.tlas_binding.count;
  p.n_tlas_root = (uint32_t)d.tlas_bvh_root.count;
  p.tlas_binding = d.tlas_binding.ptr;
  p.tlas_bvh_root = d.tlas_bvh_root.ptr;
  p.tlas_forest = d.tlas_bvh_forest.ptr;
  p.tlas_data = d.tlas_data.ptr;
  p.tlas_bounding = d.tlas_bounding.ptr;
  p.blas_meta = d.blas_meta_info.ptr;
  p.tri_root = d.tri_bvh_root.ptr;
  p.tri_forest = d.tri_bvh_forest.ptr;
  p.redirect = d.indices_redirect.ptr;
  p.tris = reinterpret_cast<const float4*>(d.tri_records.ptr);
  p.wide = reinterpret_cast<const float4*>(d.wide_nodes.ptr);
  p.leaves = reinterpret_cast<const uint2*>(d.leaf_ranges.ptr);
  p.geom_root_code = d.geom_root_code.ptr;
  p.wide4 = reinterpret_cast<const float4*>(d.wide4_nodes.ptr);
  p.geom_root_code4 = d.geom_root_code4.ptr;
  p.counters = reinterpret_cast<unsigned long long*>(c->d_counters);
  p.error_word = c->d_counters + 8;
  p.local_stack = desc->local_stack && order_of(desc->traversal) != RDN_TRAVERSAL_REFERENCE &&
                  p.stack_depth <= rdn::kLocalStackEntries;
  p.iteration_limit = c->iteration_limit;
  p.watertight = (desc->traversal & RDN_INTERSECT_WATERTIGHT) ? 1u : 0u;
  p.verts = reinterpret_cast<const float4*>(d.vertex_records.ptr);
  return RDN_OK;
}

rdn_status validate_trace(rdn_ctx* c, const rdn_trace_desc* desc) {
  if (!c || !desc) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (desc->count && (!desc->rays || !desc->hits)) return fail(c, RDN_ERR_INVALID_ARG, "null ray or hit buffer");
  if ((reinterpret_cast<uintptr_t>(desc->rays) & 15) || (reinterpret_cast<uintptr_t>(desc->hits) & 15) ||
      (reinterpret_cast<uintptr_t>(desc->hits_ext) & 15))
    return fail(c, RDN_ERR_INVALID_ARG, "ray and hit buffers must be 16-byte aligned");
  if (!traversal_ok(desc->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (desc->anyhit_mode > RDN_ANYHIT_PRIMITIVE_MASK) return fail(c, RDN_ERR_INVALID_ARG, "unknown any-hit mode");
  if (desc->anyhit_mode == RDN_ANYHIT_PRIMITIVE_MASK && !desc->anyhit_mask)
    return fail(c, RDN_ERR_INVALID_ARG, "RDN_ANYHIT_PRIMITIVE_MASK needs anyhit_mask");
  if (desc->block_size && (desc->block_size % 32 || desc->block_size > 256))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 256");
  if (desc->local_stack > 1) return fail(c, RDN_ERR_INVALID_ARG, "local_stack must be 0 or 1");
  return RDN_OK;
}

rdn_status ensure_built(rdn_ctx* c) {
  if (!c->dirty && c->host) return RDN_OK;
  return do_build(c);
}

// Checks of the knobs that rdn_wavefront_shadow_bounce and its allocation-free
// variant share (their scratch checks differ).
rdn_status wavefront_check_knobs(rdn_ctx* c, const rdn_wavefront_desc* d) {
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->phases > 3) return fail(c, RDN_ERR_INVALID_ARG, "unknown phase mask");
  if (d->refill > 32) return fail(c, RDN_ERR_INVALID_ARG, "refill must be 0..32");
  if (d->local_stack > 1) return fail(c, RDN_ERR_INVALID_ARG, "local_stack must be 0 or 1");
  if (d->register_tier > 2) return fail(c, RDN_ERR_INVALID_ARG, "register_tier must be 0, 1 or 2");
  if (d->speculation > 31) return fail(c, RDN_ERR_INVALID_ARG, "speculation must be 0..31");
  if (d->block_size && (d->block_size % 32 || d->block_size > 128))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 128");
  const uint64_t fh = d->frame_height ? d->frame_height : d->camera.height;
  if ((uint64_t)d->row_offset + d->camera.height > fh)
    return fail(c, RDN_ERR_INVALID_ARG, "row_offset + camera.height exceeds frame_height");
  return RDN_OK;
}

// Launch parameters of both wavefront entry points (the queues are bound by
// the caller); the structure must be built.
void wavefront_fill(rdn_ctx* c, const rdn_wavefront_desc* d, rdn::TraceParams& p, rdn::WavefrontParams& w) {
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFF;
  td.traversal = d->traversal;
  fill_params(c, &td, p);
  std::memset(&w, 0, sizeof(w));
  const rdn_camera& cam = d->camera;
  w.origin = make_float3(cam.origin[0], cam.origin[1], cam.origin[2]);
  w.forward = make_float3(cam.forward[0], cam.forward[1], cam.forward[2]);
  w.right = make_float3(cam.right[0], cam.right[1], cam.right[2]);
  w.up = make_float3(cam.up[0], cam.up[1], cam.up[2]);
  w.light = make_float3(d->light[0], d->light[1], d->light[2]);
  w.tan_half = cam.tan_half;
  w.aspect = cam.aspect;
  w.width = d->camera.width;
  w.height = d->camera.height;
  w.sample_index = d->sample_index;
  w.tlas = d->tlas_uniform;
  w.out = reinterpret_cast<rdn::PixelResult*>(d->out);
  w.ray_counts = d->ray_counts;
  w.refill = d->refill;
  w.local_stack = d->local_stack;
  w.register_tier = d->register_tier;
  w.row0 = d->row_offset;
  w.frame_height = d->frame_height ? d->frame_height : d->camera.height;
  p.spec_threshold = d->speculation;
}

}  // namespace

extern "C" {

uint32_t rdn_api_version(void) { return RDN_API_VERSION; }

rdn_status rdn_create(rdn_ctx** out, int device) {
  if (!out) return RDN_ERR_INVALID_ARG;
  *out = nullptr;
  rdn_ctx* c = new (std::nothrow) rdn_ctx();
  if (!c) return RDN_ERR_OOM;
  c->device = device;
  if (device >= 0) {
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_counters, 64);
    if (e == cudaSuccess) e = cudaMemset(c->d_counters, 0, 64);
    // device address of the allocation-free entry point's static queue array
    if (e == cudaSuccess) e = rdn::wavefront_static_prepare(device);
    if (e != cudaSuccess) {
      delete c;
      return e == cudaErrorMemoryAllocation ? RDN_ERR_OOM : RDN_ERR_CUDA;
    }
  } else if (device != -1) {
    delete c;
    return RDN_ERR_INVALID_ARG;
  }
  *out = c;
  return RDN_OK;
}

rdn_status rdn_destroy(rdn_ctx* c) {
  if (!c) return RDN_ERR_INVALID_ARG;
  if (c->device >= 0) {
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    free_device(c->dev);
    if (c->d_counters) cudaFree(c->d_counters);
    if (c->build_pool) cudaMemPoolDestroy(c->build_pool);
  }
  delete c;
  return RDN_OK;
}

const char* rdn_last_error(const rdn_ctx* c) { return c ? c->err.c_str() : "null context"; }

rdn_status rdn_set_iteration_limit(rdn_ctx* c, uint32_t limit) {
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  c->iteration_limit = limit;
  return RDN_OK;
}

rdn_status rdn_check_errors(rdn_ctx* c, void* stream, uint32_t* flags) {
  if (!c) return RDN_ERR_INVALID_ARG;
  if (flags) *flags = 0;
  if (c->device < 0) return RDN_OK;
  std::lock_guard<std::mutex> lk(c->lock);
  uint32_t word = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&word, c->d_counters + 8, 4, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_counters + 8, 0, 4, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "read the error word");
  if (flags) *flags = word;
  if (word & RDN_ERROR_ITERATION_LIMIT)
    return fail(c, RDN_ERR_TIMEOUT, "a dynamic-fetch warp reached its iteration limit; its rays are incomplete");
  if (word & RDN_ERROR_STACK_OVERFLOW) return fail(c, RDN_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
  return RDN_OK;
}

rdn_status rdn_blas_create(rdn_ctx* c, const rdn_geometry* g, uint32_t count, uint32_t* out_handle) {
  if (!c || !out_handle || (count && !g)) return fail(c, RDN_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(c->lock);
  auto v = std::make_unique<std::vector<rdn::GeometrySource>>();
  try {
    for (uint32_t i = 0; i < count; i++) {
      rdn::GeometrySource s;
      s.type = g[i].type;
      s.flags = g[i].flags;
      if (s.type > 1) return fail(c, RDN_ERR_INVALID_ARG, "unknown geometry type");
      if (s.type == 0) {
        if (g[i].vertex_count && !g[i].positions) return fail(c, RDN_ERR_INVALID_ARG, "null positions");
        s.positions.assign(g[i].positions, g[i].positions + (size_t)g[i].vertex_count * 3);
        s.indexed = g[i].indices != nullptr;
        if (s.indexed) {
          s.indices.assign(g[i].indices, g[i].indices + g[i].index_count);
          for (uint32_t k = 0; k < (s.indices.size() / 3) * 3; k++)
            if (s.indices[k] >= g[i].vertex_count) return fail(c, RDN_ERR_INVALID_ARG, "index out of range");
        }
      } else {
        s.indexed = false;
      }
      v->push_back(std::move(s));
    }
  } catch (const std::bad_alloc&) {
    return fail(c, RDN_ERR_OOM, "host allocation failed");
  }
  c->blas.push_back(std::move(v));
  c->dirty = true;
  *out_handle = (uint32_t)(c->blas.size() - 1);
  return RDN_OK;
}

rdn_status rdn_blas_delete(rdn_ctx* c, uint32_t h) {
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  if (h >= c->blas.size() || !c->blas[h]) return fail(c, RDN_ERR_INVALID_HANDLE, "no such BLAS");
  c->blas[h].reset();
  c->dirty = true;
  return RDN_OK;
}

rdn_status rdn_tlas_create(rdn_ctx* c, const rdn_instance* inst, uint32_t count, uint32_t* out_handle) {
  if (!c || !out_handle || (count && !inst)) return fail(c, RDN_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(c->lock);
  auto v = std::make_unique<std::vector<rdn::InstanceSource>>();
  for (uint32_t i = 0; i < count; i++) {
    rdn::InstanceSource s;
    std::memcpy(s.transform, inst[i].transform, 64);
    s.custom_index = inst[i].custom_index;
    s.mask = inst[i].mask;
    s.sbt_offset = inst[i].sbt_offset;
    s.flags = inst[i].flags;
    s.blas_handle = inst[i].blas_handle;
    v->push_back(s);
  }
  c->tlas.push_back(std::move(v));
  c->dirty = true;
  *out_handle = (uint32_t)(c->tlas.size() - 1);
  return RDN_OK;
}

rdn_status rdn_tlas_delete(rdn_ctx* c, uint32_t h) {
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  if (h >= c->tlas.size() || !c->tlas[h]) return fail(c, RDN_ERR_INVALID_HANDLE, "no such TLAS");
  c->tlas[h].reset();
  c->dirty = true;
  return RDN_OK;
}

rdn_status rdn_bind_tlas(rdn_ctx* c, const uint32_t* handles, uint32_t count) {
  if (!c || (count && !handles)) return fail(c, RDN_ERR_INVALID_ARG, "null argument");
  std::lock_guard<std::mutex> lk(c->lock);
  std::vector<uint32_t> nb(handles, handles + count);
  if (nb != c->binding) {
    c->binding = std::move(nb);
    c->dirty = true;
  }
  return RDN_OK;
}

rdn_status rdn_build(rdn_ctx* c, const rdn_build_opts* o) {
  Range range_("rdn_build");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::BuildOptions opts;
  if (o) {
    if (o->blas_bin_size) opts.blas_bin_size = o->blas_bin_size;
    if (o->blas_max_depth) opts.blas_max_depth = o->blas_max_depth;
    if (o->tlas_bin_size) opts.tlas_bin_size = o->tlas_bin_size;
    if (o->tlas_max_depth) opts.tlas_max_depth = o->tlas_max_depth;
    opts.host_threads = o->host_threads;
    opts.device_build = o->device_build;
    if (opts.device_build > 1) return fail(c, RDN_ERR_INVALID_ARG, "device_build must be 0 or 1");
    if (opts.blas_max_depth > 64 || opts.tlas_max_depth > 64)
      return fail(c, RDN_ERR_INVALID_ARG, "max tree depth above 64 is not supported");
  }
  c->opts = opts;
  return do_build(c);
}

rdn_status rdn_get_build_stats(const rdn_ctx* cc, rdn_build_stats* out) {
  rdn_ctx* c = const_cast<rdn_ctx*>(cc);
  if (!c || !out) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  if (!c->host || c->dirty) return fail(c, RDN_ERR_NOT_BUILT, "structure not built");
  std::memset(out, 0, sizeof(*out));
  out->device_bytes = c->dev.bytes;
  out->triangles = c->host->n_triangles;
  out->nodes = c->host->n_nodes;
  out->device_built = c->host->device_blas ? 1u : 0u;
  out->device_seconds = c->device_seconds;
  out->sah_splits = c->host->sah_splits;
  out->median_fallbacks = c->host->median_fallbacks;
  out->max_blas_depth = c->host->max_blas_depth;
  out->build_seconds = c->build_seconds;
  out->upload_seconds = c->upload_seconds;
  return RDN_OK;
}

rdn_status rdn_get_built_array(const rdn_ctx* cc, uint32_t which, void* dst, size_t capacity, size_t* size) {
  rdn_ctx* c = const_cast<rdn_ctx*>(cc);
  if (!c || !size) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  if (!c->host || c->dirty) return fail(c, RDN_ERR_NOT_BUILT, "structure not built");
  const rdn::HostBuilt& B = *c->host;
  const void* src = nullptr;
  size_t bytes = 0;
#define CASE(i, v)                       \
  case i:                                \
    src = B.v.data();                    \
    bytes = B.v.size() * sizeof(B.v[0]); \
    break;
  switch (which) {
    CASE(0, tlas_binding)
    CASE(1, tlas_bvh_root)
    CASE(2, tlas_bvh_forest)
    CASE(3, tlas_data)
    CASE(4, tlas_bounding)
    CASE(5, blas_meta_info)
    CASE(6, tri_bvh_root)
    CASE(7, tri_bvh_forest)
    CASE(8, indices_redirect)
    CASE(9, indices)
    CASE(10, vertices)
    default:
      return fail(c, RDN_ERR_INVALID_ARG, "unknown array");
  }
#undef CASE
  const void* dev_src = nullptr;
  if (B.device_blas) {  // these arrays were built on the device and live only there
    switch (which) {
      case 7:
        dev_src = c->dev.tri_bvh_forest.ptr;
        bytes = B.n_nodes * sizeof(rdn::DeviceBVHNode);
        break;
      case 8:
        dev_src = c->dev.indices_redirect.ptr;
        bytes = B.n_triangles * sizeof(uint32_t);
        break;
      case 9:
        dev_src = c->dev.indices.ptr;
        bytes = B.n_indices * sizeof(uint32_t);
        break;
      case 10:
        dev_src = c->dev.vertices.ptr;
        bytes = B.n_vertices * 3 * sizeof(float);
        break;
      default:
        break;
    }
  }
  *size = bytes;
  if (dst) {
    if (capacity < bytes) return fail(c, RDN_ERR_INVALID_ARG, "destination too small");
    if (bytes && dev_src) {
      cudaError_t e = cudaSetDevice(c->device);
      if (e == cudaSuccess) e = cudaMemcpy(dst, dev_src, bytes, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return cuda_fail(c, e, "read back built array");
    } else if (bytes) {
      std::memcpy(dst, src, bytes);
    }
  }
  return RDN_OK;
}

rdn_status rdn_trace(rdn_ctx* c, const rdn_trace_desc* desc, void* stream) {
  Range range_("rdn_trace");
  rdn_status st = validate_trace(c, desc);
  if (st != RDN_OK) return st;
  std::lock_guard<std::mutex> lk(c->lock);
  st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn::TraceParams p;
  fill_params(c, desc, p);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_trace(p, mode_of(desc->traversal), false, desc->block_size, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "trace launch");
  return RDN_OK;
}

rdn_status rdn_trace_params(rdn_ctx* c, uint32_t traversal, void* out, size_t* size) {
  if (!c || !size) return fail(c, RDN_ERR_INVALID_ARG, "null context or size");
  if (!out) {
    *size = sizeof(rdn::TraceParams);
    return RDN_OK;
  }
  if (*size < sizeof(rdn::TraceParams)) return fail(c, RDN_ERR_INVALID_ARG, "output smaller than the parameter block");
  if (!traversal_ok(traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context has no device structure");
  std::lock_guard<std::mutex> lk(c->lock);
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.cull_mask = 0xFF;
  td.traversal = traversal;
  td.local_stack = 1;
  rdn::TraceParams p;
  fill_params(c, &td, p);
  if (order_of(traversal) != RDN_TRAVERSAL_REFERENCE && !p.local_stack)
    return fail(c, RDN_ERR_UNSUPPORTED, "the tree is too deep for a 64-entry local traversal stack");
  std::memcpy(out, &p, sizeof(p));
  *size = sizeof(p);
  return RDN_OK;
}

rdn_status rdn_trace_counted(rdn_ctx* c, const rdn_trace_desc* desc, void* stream, rdn_counters* out) {
  Range range_("rdn_trace_counted");
  rdn_status st = validate_trace(c, desc);
  if (st != RDN_OK) return st;
  if (!out) return fail(c, RDN_ERR_INVALID_ARG, "null counters");
  std::lock_guard<std::mutex> lk(c->lock);
  st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn::TraceParams p;
  fill_params(c, desc, p);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_counters, 0, 64, s);
  if (e == cudaSuccess) e = rdn::launch_trace(p, mode_of(desc->traversal), true, desc->block_size, s);
  uint64_t h[8];
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, c->d_counters, 64, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(c, e, "counted trace");
  out->node_visits = h[0];
  out->tri_tests = h[1];
  out->tri_hits = h[2];
  out->bad_tlas_rays = h[3];
  return RDN_OK;
}

rdn_status rdn_wavefront_scratch_size(uint32_t width, uint32_t height, size_t* bytes) {
  if (!bytes) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::wavefront_scratch_bytes(width, height);
  return RDN_OK;
}

rdn_status rdn_wavefront_shadow_bounce(rdn_ctx* c, const rdn_wavefront_desc* d, void* stream) {
  Range range_("rdn_wavefront_shadow_bounce");
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  const uint32_t W = d->camera.width, H = d->camera.height;
  if ((uint64_t)W * H > 0xFFFFFFFFull / 2) return fail(c, RDN_ERR_INVALID_ARG, "launch too large");
  if (W && H && (!d->out || !d->scratch)) return fail(c, RDN_ERR_INVALID_ARG, "null output or scratch");
  if (d->scratch_bytes < rdn::wavefront_scratch_bytes(W, H)) return fail(c, RDN_ERR_INVALID_ARG, "scratch too small");
  if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) || (reinterpret_cast<uintptr_t>(d->out) & 15))
    return fail(c, RDN_ERR_INVALID_ARG, "scratch must be 256-byte and output 16-byte aligned");
  rdn_status st = wavefront_check_knobs(c, d);
  if (st != RDN_OK) return st;
  std::lock_guard<std::mutex> lk(c->lock);
  st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn::TraceParams p;
  rdn::WavefrontParams w;
  wavefront_fill(c, d, p, w);
  rdn::wavefront_bind_scratch(w, d->scratch);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_wavefront(p, w, mode_of(d->traversal), d->block_size, c->sm_count, d->phases,
                              static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "wavefront launch");
  return RDN_OK;
}

}  // extern "C"

struct rdn_graph {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int device = -1;
};

namespace {

rdn_status prepare_path_launch(rdn_ctx* c, const rdn_path_desc* d, rdn::TraceParams& p, rdn::PathParams& q,
                               uint32_t* grid) {
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->max_bounces > 16) return fail(c, RDN_ERR_INVALID_ARG, "max_bounces above 16");
  if (d->count && (!d->rays || !d->out || !d->scratch)) return fail(c, RDN_ERR_INVALID_ARG, "null buffer");
  if (d->sort_key > 2) return fail(c, RDN_ERR_INVALID_ARG, "unknown sort key");
  if (d->refill > 32) return fail(c, RDN_ERR_INVALID_ARG, "refill must be 0..32");
  if (d->speculation > 31) return fail(c, RDN_ERR_INVALID_ARG, "speculation must be 0..31");
  if (d->scratch_bytes < rdn::paths_scratch_bytes(d->count, d->max_bounces, d->sort_key))
    return fail(c, RDN_ERR_INVALID_ARG, "scratch too small");
  if ((reinterpret_cast<uintptr_t>(d->scratch) & 255) || (reinterpret_cast<uintptr_t>(d->rays) & 15) ||
      (reinterpret_cast<uintptr_t>(d->out) & 7))
    return fail(c, RDN_ERR_INVALID_ARG, "misaligned buffer");
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->block_size && (d->block_size % 32 || d->block_size > 128))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 128");
  if (!(d->rr_survive > 0.0f && d->rr_survive <= 1.0f)) return fail(c, RDN_ERR_INVALID_ARG, "rr_survive not in (0, 1]");
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFF;
  td.traversal = d->traversal;
  td.local_stack = d->local_stack;
  fill_params(c, &td, p);
  std::memset(&q, 0, sizeof(q));
  q.primary_rays = reinterpret_cast<const float4*>(d->rays);
  q.tlas_idx = d->tlas_idx;
  q.count = d->count;
  q.tlas_uniform = d->tlas_uniform;
  q.max_bounces = d->max_bounces;
  q.rr_start = d->rr_start;
  q.seed = d->seed;
  q.albedo = d->albedo;
  q.rr_survive = d->rr_survive;
  q.out = reinterpret_cast<float2*>(d->out);
  q.segment_counts = d->segment_counts;
  q.sort_key = d->sort_key;
  q.refill = d->refill;
  p.spec_threshold = d->speculation;
  if (d->sort_key) {
    uint32_t bits = 0;
    while (bits < 32 && (1ull << bits) < (uint64_t)std::max<size_t>(1, c->dev.tlas_binding.count)) bits++;
    bits += 3 + (d->sort_key == 2 ? 12 : 0);
    if (bits > 32) return fail(c, RDN_ERR_INVALID_ARG, "too many bound TLASes for this sort key");
    q.key_bits = bits;
  }
  if (d->count) rdn::paths_bind_scratch(q, d->scratch);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess && d->count)
    e = rdn::prepare_paths(p, q, mode_of(d->traversal), d->block_size, c->sm_count, grid);
  if (e != cudaSuccess) return cuda_fail(c, e, "path launch preparation");
  return RDN_OK;
}

}  // namespace

extern "C" {

rdn_status rdn_paths_scratch_size(uint32_t count, uint32_t max_bounces, uint32_t sort_key, size_t* bytes) {
  if (!bytes || max_bounces > 16 || sort_key > 2) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::paths_scratch_bytes(count, max_bounces, sort_key);
  return RDN_OK;
}

rdn_status rdn_trace_paths(rdn_ctx* c, const rdn_path_desc* d, void* stream) {
  Range range_("rdn_trace_paths");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::PathParams q;
  uint32_t grid = 0;
  rdn_status st = prepare_path_launch(c, d, p, q, &grid);
  if (st != RDN_OK || d->count == 0) return st;
  cudaError_t e = rdn::record_paths(p, q, mode_of(d->traversal), d->block_size, grid,
                                    static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "path launch");
  return RDN_OK;
}

rdn_status rdn_trace_paths_graph(rdn_ctx* c, const rdn_path_desc* d, rdn_graph** out) {
  Range range_("rdn_trace_paths_graph");
  if (!c || !out) return RDN_ERR_INVALID_ARG;
  *out = nullptr;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::PathParams q;
  uint32_t grid = 0;
  rdn_status st = prepare_path_launch(c, d, p, q, &grid);
  if (st != RDN_OK) return st;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(c, e, "capture stream");
  auto* g = new (std::nothrow) rdn_graph();
  if (!g) {
    cudaStreamDestroy(s);
    return fail(c, RDN_ERR_OOM, "host allocation failed");
  }
  g->device = c->device;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t rec = d->count ? rdn::record_paths(p, q, mode_of(d->traversal), d->block_size, grid, s) : cudaSuccess;
    e = cudaStreamEndCapture(s, &g->graph);
    if (rec != cudaSuccess) e = rec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(c, e, "path graph capture");
  }
  *out = g;
  return RDN_OK;
}

rdn_status rdn_graph_launch(rdn_graph* g, void* stream) {
  Range range_("rdn_graph_launch");
  if (!g || !g->exec) return RDN_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(g->device);
  if (e == cudaSuccess) e = cudaGraphLaunch(g->exec, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RDN_OK : RDN_ERR_CUDA;
}

rdn_status rdn_graph_destroy(rdn_graph* g) {
  if (!g) return RDN_ERR_INVALID_ARG;
  cudaSetDevice(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
  return RDN_OK;
}

}  // extern "C"

namespace {

rdn_status prepare_attr(rdn_ctx* c, const rdn_attr_loss_desc* d, bool adjoint, rdn::TraceParams& p,
                        rdn::AdjointParams& a) {
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->count && (!d->rays || !d->attributes)) return fail(c, RDN_ERR_INVALID_ARG, "null rays or attributes");
  if (adjoint && d->count && !d->grad_vertices) return fail(c, RDN_ERR_INVALID_ARG, "null gradient buffer");
  if ((reinterpret_cast<uintptr_t>(d->rays) & 15) || (reinterpret_cast<uintptr_t>(d->grad_vertices) & 15))
    return fail(c, RDN_ERR_INVALID_ARG, "rays and gradients must be 16-byte aligned");
  if (d->from_record > 1) return fail(c, RDN_ERR_INVALID_ARG, "from_record must be 0 or 1");
  if (adjoint && d->from_record && d->count && (!d->hit_tri || !d->hit_inst))
    return fail(c, RDN_ERR_INVALID_ARG, "from_record needs the hit_tri and hit_inst records of the forward");
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->block_size && (d->block_size % 32 || d->block_size > 128))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 128");
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFF;
  td.traversal = d->traversal;
  td.local_stack = d->local_stack;
  fill_params(c, &td, p);
  if (d->speculation > 31) return fail(c, RDN_ERR_INVALID_ARG, "speculation must be 0..31");
  p.spec_threshold = d->speculation;
  std::memset(&a, 0, sizeof(a));
  a.rays = reinterpret_cast<const float4*>(d->rays);
  a.count = d->count;
  a.tlas_uniform = d->tlas_uniform;
  a.indices = c->dev.indices.ptr;
  a.vertices = c->dev.vertices.ptr;
  a.attributes = d->attributes;
  a.targets = d->targets;
  a.ray_value = d->ray_value;
  a.ray_loss = d->ray_loss;
  a.loss_sum = d->loss_sum;
  a.grad_vertices = d->grad_vertices;
  a.grad_ray_origin = d->grad_ray_origin;
  a.grad_ray_direction = d->grad_ray_direction;
  a.grad_scale = d->grad_scale;
  a.hit_tri = d->hit_tri;
  a.hit_inst = d->hit_inst;
  a.from_record = d->from_record != 0;
  return RDN_OK;
}

rdn_status prepare_hit_diff(rdn_ctx* c, const rdn_hit_diff_desc* d, bool adjoint, rdn::TraceParams& p,
                            rdn::AdjointParams& a) {
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->count && !d->rays) return fail(c, RDN_ERR_INVALID_ARG, "null rays");
  if (adjoint && d->count && (!d->grad_hit || !d->grad_vertices))
    return fail(c, RDN_ERR_INVALID_ARG, "the adjoint needs grad_hit and grad_vertices");
  if ((reinterpret_cast<uintptr_t>(d->rays) & 15) || (reinterpret_cast<uintptr_t>(d->hit) & 15) ||
      (reinterpret_cast<uintptr_t>(d->grad_hit) & 15) || (reinterpret_cast<uintptr_t>(d->grad_vertices) & 15))
    return fail(c, RDN_ERR_INVALID_ARG, "rays, hits and gradients must be 16-byte aligned");
  if (d->from_record > 1) return fail(c, RDN_ERR_INVALID_ARG, "from_record must be 0 or 1");
  if (adjoint && d->from_record && d->count && (!d->hit_tri || !d->hit_inst))
    return fail(c, RDN_ERR_INVALID_ARG, "from_record needs the hit_tri and hit_inst records of the forward");
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->block_size && (d->block_size % 32 || d->block_size > 128))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 128");
  if (d->local_stack > 1) return fail(c, RDN_ERR_INVALID_ARG, "local_stack must be 0 or 1");
  if (d->speculation > 31) return fail(c, RDN_ERR_INVALID_ARG, "speculation must be 0..31");
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFF;
  td.traversal = d->traversal;
  td.local_stack = d->local_stack;
  fill_params(c, &td, p);
  p.spec_threshold = d->speculation;
  std::memset(&a, 0, sizeof(a));
  a.rays = reinterpret_cast<const float4*>(d->rays);
  a.count = d->count;
  a.tlas_uniform = d->tlas_uniform;
  a.indices = c->dev.indices.ptr;
  a.vertices = c->dev.vertices.ptr;
  a.attributes = d->attributes;
  a.hit_out = reinterpret_cast<float4*>(d->hit);
  a.hit_tri = d->hit_tri;
  a.hit_inst = d->hit_inst;
  a.grad_hit = reinterpret_cast<const float4*>(d->grad_hit);
  a.grad_vertices = d->grad_vertices;
  a.grad_ray_origin = d->grad_ray_origin;
  a.grad_ray_direction = d->grad_ray_direction;
  a.from_record = d->from_record != 0;
  return RDN_OK;
}

}  // namespace

extern "C" {

rdn_status rdn_hit_diff_forward(rdn_ctx* c, const rdn_hit_diff_desc* d, void* stream) {
  Range range_("rdn_hit_diff_forward");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::AdjointParams a;
  rdn_status st = prepare_hit_diff(c, d, false, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_hit_diff(p, a, mode_of(d->traversal), false, d->block_size, c->sm_count,
                             static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "hit query forward");
  return RDN_OK;
}

rdn_status rdn_hit_diff_adjoint(rdn_ctx* c, const rdn_hit_diff_desc* d, void* stream) {
  Range range_("rdn_hit_diff_adjoint");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::AdjointParams a;
  rdn_status st = prepare_hit_diff(c, d, true, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_hit_diff(p, a, mode_of(d->traversal), true, d->block_size, c->sm_count,
                             static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "hit query adjoint");
  return RDN_OK;
}

rdn_status rdn_attr_loss_forward(rdn_ctx* c, const rdn_attr_loss_desc* d, void* stream) {
  Range range_("rdn_attr_loss_forward");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::AdjointParams a;
  rdn_status st = prepare_attr(c, d, false, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_attr_forward(p, a, mode_of(d->traversal), d->block_size, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "attribute loss forward");
  return RDN_OK;
}

rdn_status rdn_attr_loss_adjoint(rdn_ctx* c, const rdn_attr_loss_desc* d, void* stream) {
  Range range_("rdn_attr_loss_adjoint");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::AdjointParams a;
  rdn_status st = prepare_attr(c, d, true, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_attr_adjoint(p, a, mode_of(d->traversal), d->block_size, c->sm_count,
                                 static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "attribute loss adjoint");
  return RDN_OK;
}

}  // extern "C"

namespace {

rdn_status prepare_attr_paths(rdn_ctx* c, const rdn_attr_path_desc* d, bool adjoint, rdn::TraceParams& p,
                              rdn::PathAdjointParams& a) {
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->segments < 1 || d->segments > 8) return fail(c, RDN_ERR_INVALID_ARG, "segments must be 1..8");
  if (d->count && (!d->rays || !d->attributes)) return fail(c, RDN_ERR_INVALID_ARG, "null rays or attributes");
  if (adjoint && d->count && !d->grad_vertices) return fail(c, RDN_ERR_INVALID_ARG, "null gradient buffer");
  if ((reinterpret_cast<uintptr_t>(d->rays) & 15) || (reinterpret_cast<uintptr_t>(d->grad_vertices) & 15) ||
      (reinterpret_cast<uintptr_t>(d->seg_rays) & 15))
    return fail(c, RDN_ERR_INVALID_ARG, "rays, segment rays and gradients must be 16-byte aligned");
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->block_size && (d->block_size % 32 || d->block_size > 128))
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be a multiple of 32 up to 128");
  if (d->from_record > 1) return fail(c, RDN_ERR_INVALID_ARG, "from_record must be 0 or 1");
  if (adjoint && d->from_record && d->count && (!d->seg_tri || !d->seg_inst || !d->seg_rays))
    return fail(c, RDN_ERR_INVALID_ARG, "from_record needs the seg_tri, seg_inst and seg_rays records of the forward");
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFF;
  td.traversal = d->traversal;
  td.local_stack = d->local_stack;
  fill_params(c, &td, p);
  if (d->speculation > 31) return fail(c, RDN_ERR_INVALID_ARG, "speculation must be 0..31");
  p.spec_threshold = d->speculation;
  std::memset(&a, 0, sizeof(a));
  a.rays = reinterpret_cast<const float4*>(d->rays);
  a.tlas_idx = d->tlas_idx;
  a.count = d->count;
  a.tlas_uniform = d->tlas_uniform;
  a.segments = d->segments;
  a.seed = d->seed;
  a.indices = c->dev.indices.ptr;
  a.vertices = c->dev.vertices.ptr;
  a.attributes = d->attributes;
  a.targets = d->targets;
  a.values = d->values;
  a.loss_sum = d->loss_sum;
  a.grad_vertices = d->grad_vertices;
  a.seg_tri = d->seg_tri;
  a.seg_rays = reinterpret_cast<float4*>(d->seg_rays);
  a.seg_inst = d->seg_inst;
  a.from_record = d->from_record != 0;
  a.grad_scale = d->grad_scale;
  a.work_counter = c->d_counters + 12;
  return RDN_OK;
}

}  // namespace

extern "C" {

rdn_status rdn_attr_paths_forward(rdn_ctx* c, const rdn_attr_path_desc* d, void* stream) {
  Range range_("rdn_attr_paths_forward");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::PathAdjointParams a;
  rdn_status st = prepare_attr_paths(c, d, false, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_attr_paths(p, a, mode_of(d->traversal), false, d->block_size, c->sm_count,
                               static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "attribute paths forward");
  return RDN_OK;
}

rdn_status rdn_attr_paths_adjoint(rdn_ctx* c, const rdn_attr_path_desc* d, void* stream) {
  Range range_("rdn_attr_paths_adjoint");
  if (!c) return RDN_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::PathAdjointParams a;
  rdn_status st = prepare_attr_paths(c, d, true, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_attr_paths(p, a, mode_of(d->traversal), true, d->block_size, c->sm_count,
                               static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "attribute paths adjoint");
  return RDN_OK;
}

rdn_status rdn_attr_paths_graph(rdn_ctx* c, const rdn_attr_path_desc* d, uint64_t num_vertices, rdn_graph** out) {
  Range range_("rdn_attr_paths_graph");
  if (!c || !out) return RDN_ERR_INVALID_ARG;
  *out = nullptr;
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::PathAdjointParams a;
  rdn_status st = prepare_attr_paths(c, d, d->grad_vertices != nullptr, p, a);
  if (st != RDN_OK) return st;
  if (num_vertices > c->dev.vertex_count) return fail(c, RDN_ERR_INVALID_ARG, "more vertices than the structure has");
  // warm launch outside the capture sets the kernel attributes
  cudaStream_t s = nullptr;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(c, e, "capture stream");
  const int mode = mode_of(d->traversal);
  rdn::PathAdjointParams fwd = a;
  fwd.grad_vertices = nullptr;
  auto record = [&]() -> cudaError_t {
    cudaError_t r = cudaSuccess;
    if (d->loss_sum) r = cudaMemsetAsync(d->loss_sum, 0, sizeof(double), s);
    if (r == cudaSuccess && d->grad_vertices) r = cudaMemsetAsync(d->grad_vertices, 0, num_vertices * 16, s);
    if (r == cudaSuccess) r = rdn::launch_attr_paths(p, fwd, mode, false, d->block_size, c->sm_count, s);
    if (r == cudaSuccess && d->grad_vertices)
      r = rdn::launch_attr_paths(p, a, mode, true, d->block_size, c->sm_count, s);
    return r;
  };
  e = record();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  auto* g = new (std::nothrow) rdn_graph();
  if (!g) {
    cudaStreamDestroy(s);
    return fail(c, RDN_ERR_OOM, "host allocation failed");
  }
  g->device = c->device;
  if (e == cudaSuccess) e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t rec = record();
    e = cudaStreamEndCapture(s, &g->graph);
    if (rec != cudaSuccess) e = rec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(c, e, "attribute paths graph capture");
  }
  *out = g;
  return RDN_OK;
}

rdn_status rdn_scan_scratch_size(uint32_t count, size_t* bytes) {
  if (!bytes) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::scan_scratch_bytes(count);
  return RDN_OK;
}

rdn_status rdn_scan_u32(const uint32_t* in, uint32_t* out, uint32_t count, int inclusive, uint32_t segment,
                        void* scratch, size_t scratch_bytes, void* stream) {
  Range range_("rdn_scan_u32");
  if (count && (!in || !out || !scratch)) return RDN_ERR_INVALID_ARG;
  if (segment & (segment - 1)) return RDN_ERR_INVALID_ARG;
  if (scratch_bytes < rdn::scan_scratch_bytes(count) || (reinterpret_cast<uintptr_t>(scratch) & 255))
    return RDN_ERR_INVALID_ARG;
  cudaError_t e = rdn::scan_u32(in, out, count, inclusive != 0, segment, scratch, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RDN_OK : RDN_ERR_CUDA;
}

rdn_status rdn_compact_scratch_size(uint32_t count, size_t* bytes) {
  if (!bytes) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::compact_scratch_bytes(count);
  return RDN_OK;
}

rdn_status rdn_compact_u32(const uint32_t* values, const uint32_t* flags, uint32_t* out, uint32_t* out_count,
                           uint32_t count, void* scratch, size_t scratch_bytes, void* stream) {
  Range range_("rdn_compact_u32");
  if (!out_count || (count && (!values || !flags || !out || !scratch))) return RDN_ERR_INVALID_ARG;
  if (scratch_bytes < rdn::compact_scratch_bytes(count) || (reinterpret_cast<uintptr_t>(scratch) & 255))
    return RDN_ERR_INVALID_ARG;
  cudaError_t e = rdn::compact_u32(values, flags, out, out_count, count, scratch, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RDN_OK : RDN_ERR_CUDA;
}

rdn_status rdn_radix_sort_scratch_size(uint32_t count, size_t* bytes) {
  if (!bytes) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::sort_scratch_bytes(count);
  return RDN_OK;
}

rdn_status rdn_radix_sort_u32(uint32_t* keys, uint32_t* values, uint32_t count, uint32_t key_bits, void* scratch,
                              size_t scratch_bytes, void* stream) {
  Range range_("rdn_radix_sort_u32");
  if (count > 1 && (!keys || !scratch)) return RDN_ERR_INVALID_ARG;
  if (key_bits < 1 || key_bits > 32) return RDN_ERR_INVALID_ARG;
  if (scratch_bytes < rdn::sort_scratch_bytes(count) || (reinterpret_cast<uintptr_t>(scratch) & 255))
    return RDN_ERR_INVALID_ARG;
  cudaError_t e = rdn::radix_sort_u32(keys, values, count, key_bits, scratch, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? RDN_OK : RDN_ERR_CUDA;
}

// Allocation-free wavefront: identical work to rdn_wavefront_shadow_bounce with
// the queues in the library's static device array (see wavefront_static.cu).
// A build allocates, so this entry point never builds: a structure changed
// since its last build is RDN_ERR_NOT_BUILT.
rdn_status rdn_wavefront_shadow_bounce_static(rdn_ctx* c, const rdn_wavefront_desc* d, void* stream) {
  Range range_("rdn_wavefront_shadow_bounce_static");
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->scratch || d->scratch_bytes)
    return fail(c, RDN_ERR_INVALID_ARG, "the static variant uses the library's own scratch: pass scratch = NULL, 0");
  const uint32_t W = d->camera.width, H = d->camera.height;
  if ((uint64_t)W * H > 0xFFFFFFFFull / 2) return fail(c, RDN_ERR_INVALID_ARG, "launch too large");
  const size_t need = rdn::wavefront_scratch_bytes(W, H);
  if (need > RDN_WAVEFRONT_STATIC_SCRATCH_BYTES)
    return fail(c, RDN_ERR_INVALID_ARG,
                "launch of " + std::to_string(W) + "x" + std::to_string(H) + " needs " + std::to_string(need) +
                    " bytes of queue scratch; the static array holds " +
                    std::to_string(RDN_WAVEFRONT_STATIC_SCRATCH_BYTES) + " (about 466,000 pixels)");
  if (W && H && !d->out) return fail(c, RDN_ERR_INVALID_ARG, "null output");
  if (reinterpret_cast<uintptr_t>(d->out) & 15) return fail(c, RDN_ERR_INVALID_ARG, "output must be 16-byte aligned");
  rdn_status st = wavefront_check_knobs(c, d);
  if (st != RDN_OK) return st;
  std::lock_guard<std::mutex> lk(c->lock);
  if (c->dirty || !c->host)
    return fail(c, RDN_ERR_NOT_BUILT, "structure changed since its last build: call rdn_build first (a build allocates)");
  rdn::TraceParams p;
  rdn::WavefrontParams w;
  wavefront_fill(c, d, p, w);
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = rdn::launch_wavefront_static(p, w, mode_of(d->traversal), d->block_size, c->sm_count, d->phases,
                                     c->device, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "static wavefront launch");
  return RDN_OK;
}

}  // extern "C"

// ---- device task graph and AO -------------------------------------------

struct rdn_task_graph {
  rdn_ctx* ctx = nullptr;
  rdn::TaskGraph graph;
  bool needs_env = false;    // a TRACE program or an AO operation
  bool uses_ao = false;      // an AO operation (reads the camera and writes the image)
  bool ao_pipeline = false;  // made by rdn_ao_pipeline_create
  uint32_t width = 0, height = 0;
};

namespace {

// need_image: the launch runs AO operations (a trace-only task graph reads the
// traversal fields alone).
rdn_status ao_env(rdn_ctx* c, const rdn_ao_desc* d, rdn::TraceParams& p, rdn::AoEnv& a, bool need_image = true) {
  if (need_image) {
    if (!d->image) return fail(c, RDN_ERR_INVALID_ARG, "null AO image");
    if (reinterpret_cast<uintptr_t>(d->image) & 3)
      return fail(c, RDN_ERR_INVALID_ARG, "AO image must be 4-byte aligned");
    if (d->width == 0 || d->height == 0 || (uint64_t)d->width * d->height > 0x7FFFFFFFull)
      return fail(c, RDN_ERR_INVALID_ARG, "AO frame size must be 1..2^31 pixels");
  }
  if (!traversal_ok(d->traversal)) return fail(c, RDN_ERR_INVALID_ARG, "unknown traversal order");
  if (d->block_size && d->block_size != 32 && d->block_size != 64 && d->block_size != 128)
    return fail(c, RDN_ERR_INVALID_ARG, "block_size must be 32, 64 or 128");
  rdn_status st = ensure_built(c);
  if (st != RDN_OK) return st;
  rdn_trace_desc td;
  std::memset(&td, 0, sizeof(td));
  td.tlas_uniform = d->tlas_uniform;
  td.cull_mask = 0xFFFFFFFFu;
  td.traversal = d->traversal;
  td.local_stack = 1;
  fill_params(c, &td, p);
  std::memset(&a, 0, sizeof(a));
  std::memcpy(a.vp_inv, d->view_projection_inv, sizeof(a.vp_inv));
  std::memcpy(a.cam, d->camera_position, sizeof(a.cam));
  a.width = d->width;
  a.height = d->height;
  a.sample_count = d->sample_count;
  a.tlas = d->tlas_uniform;
  a.sbt_closest[0] = d->sbt_closest[0];
  a.sbt_closest[1] = d->sbt_closest[1];
  a.sbt_miss = d->sbt_miss;
  a.image = d->image;
  a.normals = d->normals;
  a.indices = c->dev.indices.ptr;
  a.vertices = c->dev.vertices.ptr;
  a.n_instances = (uint32_t)c->dev.tlas_data.count;
  a.n_triangles = (uint32_t)(c->dev.indices.count / 3);
  a.ray_counts = d->ray_counts;
  a.sample_dev = d->sample_counter;
  a.block = d->block_size;
  p.spec_threshold = d->speculation;
  return RDN_OK;
}

}  // namespace

extern "C" {

rdn_status rdn_task_graph_create(rdn_ctx* c, const rdn_task_group_desc* groups, uint32_t count, uint32_t capacity,
                                 void* stream, rdn_task_graph** out) {
  if (!c || !groups || !out) return fail(c, RDN_ERR_INVALID_ARG, "null context, groups or output");
  *out = nullptr;
  if (count > RDN_TASK_MAX_GROUPS) return fail(c, RDN_ERR_INVALID_ARG, "a task graph holds 1 to 16 task groups");
  std::vector<rdn::TaskGroupDesc> desc(count);
  bool needs_env = false, uses_ao = false;
  for (uint32_t g = 0; g < count; g++) {
    rdn::TaskGroupDesc& d = desc[g];
    d.program = groups[g].program;
    d.max_in_flight = groups[g].max_in_flight;
    d.payload_words = groups[g].payload_words;
    d.n_spawn = groups[g].n_spawn;
    d.map_op = groups[g].map_op;
    for (uint32_t k = 0; k < 4; k++) {
      d.spawn_type[k] = groups[g].spawn_type[k];
      d.spawn_op[k] = k < d.n_spawn ? groups[g].spawn_op[k] : 0u;
      if (k < d.n_spawn && d.spawn_op[k] != RDN_TASK_SPAWN_ZERO) needs_env = uses_ao = true;
    }
    if (d.program == RDN_TASK_PROGRAM_TRACE) needs_env = true;
    if (d.map_op == RDN_TASK_MAP_AO_ACCUMULATE) needs_env = uses_ao = true;
  }
  const std::string bad = rdn::TaskGraph::validate(desc, capacity);
  if (!bad.empty()) return fail(c, RDN_ERR_INVALID_ARG, bad);
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context has no device");
  std::unique_ptr<rdn_task_graph> tg(new (std::nothrow) rdn_task_graph());
  if (!tg) return fail(c, RDN_ERR_OOM, "out of host memory");
  tg->ctx = c;
  tg->needs_env = needs_env;
  tg->uses_ao = uses_ao;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  const std::string err = tg->graph.create(desc, capacity, c->sm_count, static_cast<cudaStream_t>(stream));
  if (!err.empty()) {
    const bool oom = err.find("cudaMalloc") != std::string::npos;
    return fail(c, oom ? RDN_ERR_OOM : RDN_ERR_INVALID_ARG, err);
  }
  *out = tg.release();
  return RDN_OK;
}

rdn_status rdn_task_graph_destroy(rdn_task_graph* g) {
  if (!g) return RDN_OK;
  if (g->ctx && g->ctx->device >= 0) cudaSetDevice(g->ctx->device);
  delete g;
  return RDN_OK;
}

rdn_status rdn_task_graph_dispatch_init(rdn_task_graph* g, uint32_t group, uint32_t count, uint32_t init_op,
                                        void* stream) {
  if (!g) return RDN_ERR_INVALID_ARG;
  rdn_ctx* c = g->ctx;
  if (group >= g->graph.group_count()) return fail(c, RDN_ERR_INVALID_ARG, "no such task group");
  if (init_op > RDN_TASK_INIT_INDEX) return fail(c, RDN_ERR_INVALID_ARG, "unknown init payload");
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = g->graph.dispatch_init(group, count, init_op, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "task graph dispatch");
  return RDN_OK;
}

}  // extern "C"

namespace {

// `rounds` rounds of every group; with until_empty (inside a stream capture
// only) a device-ended loop of at most `rounds` rounds instead.
rdn_status run_rounds(rdn_task_graph* g, uint32_t rounds, const rdn_ao_desc* env, cudaStream_t s, bool until_empty) {
  rdn_ctx* c = g->ctx;
  const std::string missing = g->graph.check_external();
  if (!missing.empty()) return fail(c, RDN_ERR_INVALID_ARG, missing);
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  rdn::TraceParams p;
  rdn::AoEnv a;
  const rdn::TraceParams* pp = nullptr;
  const rdn::AoEnv* ap = nullptr;
  int mode = rdn::MODE_THREADED;
  std::unique_lock<std::mutex> lk(c->lock, std::defer_lock);
  if (g->needs_env) {
    if (!env) return fail(c, RDN_ERR_INVALID_ARG, "this graph traces or shades: pass an rdn_ao_desc environment");
    lk.lock();
    rdn_status st = ao_env(c, env, p, a, g->uses_ao);
    if (st != RDN_OK) return st;
    pp = &p;
    ap = &a;
    mode = mode_of(env->traversal);
  }
  e = until_empty ? g->graph.record_until_empty(rounds, pp, mode, ap, s) : g->graph.execute(rounds, pp, mode, ap, s);
  if (e != cudaSuccess) return cuda_fail(c, e, until_empty ? "task graph drain loop" : "task graph execute");
  return RDN_OK;
}

// Captures record(stream) into an executable graph.
template <class F>
rdn_status capture_graph(rdn_ctx* c, const char* what, F record, rdn_graph** out) {
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaSetDevice");
  cudaStream_t s = nullptr;
  e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(c, e, "capture stream");
  auto* g = new (std::nothrow) rdn_graph();
  if (!g) {
    cudaStreamDestroy(s);
    return fail(c, RDN_ERR_OOM, "host allocation failed");
  }
  g->device = c->device;
  rdn_status st = RDN_OK;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    st = record(s);
    e = cudaStreamEndCapture(s, &g->graph);
  }
  if (e == cudaSuccess && st == RDN_OK) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  cudaStreamDestroy(s);
  if (e != cudaSuccess || st != RDN_OK) {
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return st != RDN_OK ? st : cuda_fail(c, e, what);
  }
  *out = g;
  return RDN_OK;
}

rdn_status require_built(rdn_ctx* c) {
  std::lock_guard<std::mutex> lk(c->lock);
  // a build allocates and synchronises, which a capture cannot hold
  if (c->dirty || !c->host) return fail(c, RDN_ERR_NOT_BUILT, "build the structure before capturing");
  return RDN_OK;
}

}  // namespace

extern "C" {

rdn_status rdn_task_graph_execute(rdn_task_graph* g, uint32_t rounds, const rdn_ao_desc* env, void* stream) {
  if (!g) return RDN_ERR_INVALID_ARG;
  return run_rounds(g, rounds, env, static_cast<cudaStream_t>(stream), false);
}

rdn_status rdn_task_graph_set_poll(rdn_task_graph* g, uint32_t group, rdn_task_poll_fn fn, void* user) {
  if (!g) return RDN_ERR_INVALID_ARG;
  rdn_ctx* c = g->ctx;
  if (group >= g->graph.group_count()) return fail(c, RDN_ERR_INVALID_ARG, "no such task group");
  if (g->graph.groups()[group].program != RDN_TASK_PROGRAM_EXTERNAL)
    return fail(c, RDN_ERR_INVALID_ARG, "the group runs a built-in program");
  g->graph.set_external(group, reinterpret_cast<rdn::ExternalPoll>(fn), user);
  return RDN_OK;
}

rdn_status rdn_task_graph_capture(rdn_task_graph* g, uint32_t group, uint32_t count, uint32_t init_op,
                                  uint32_t max_rounds, const rdn_ao_desc* env, rdn_graph** out) {
  if (!g || !out) return RDN_ERR_INVALID_ARG;
  *out = nullptr;
  rdn_ctx* c = g->ctx;
  if (group >= g->graph.group_count()) return fail(c, RDN_ERR_INVALID_ARG, "no such task group");
  if (init_op > RDN_TASK_INIT_INDEX) return fail(c, RDN_ERR_INVALID_ARG, "unknown init payload");
  if (max_rounds == 0) return fail(c, RDN_ERR_INVALID_ARG, "max_rounds must be at least 1");
  if (g->needs_env) {
    rdn_status st = require_built(c);
    if (st != RDN_OK) return st;
  }
  return capture_graph(
      c, "task graph capture",
      [&](cudaStream_t s) {
        cudaError_t e = g->graph.dispatch_init(group, count, init_op, s);
        if (e != cudaSuccess) return cuda_fail(c, e, "task graph dispatch");
        return run_rounds(g, max_rounds, env, s, true);
      },
      out);
}

rdn_status rdn_task_graph_states(rdn_task_graph* g, uint32_t* wake, uint32_t* sleep_or_finished, uint32_t* empty,
                                 void* stream) {
  if (!g) return RDN_ERR_INVALID_ARG;
  rdn_ctx* c = g->ctx;
  if (!wake || !sleep_or_finished || !empty) return fail(c, RDN_ERR_INVALID_ARG, "null output array");
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = g->graph.states(wake, empty, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "task graph states");
  for (uint32_t i = 0; i < g->graph.group_count(); i++)
    sleep_or_finished[i] = g->graph.group_cap(i) - empty[i] - wake[i];
  return RDN_OK;
}

rdn_status rdn_task_graph_debug(rdn_task_graph* g, uint32_t group, uint32_t* active, uint32_t* n_active,
                                uint32_t* empty, uint32_t* n_empty, uint32_t* task_states, void* stream) {
  if (!g) return RDN_ERR_INVALID_ARG;
  rdn_ctx* c = g->ctx;
  if (group >= g->graph.group_count()) return fail(c, RDN_ERR_INVALID_ARG, "no such task group");
  if (!active || !n_active || !empty || !n_empty || !task_states)
    return fail(c, RDN_ERR_INVALID_ARG, "null output array");
  std::vector<uint32_t> a, em, s;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = g->graph.debug(group, a, em, s, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "task graph debug");
  std::copy(a.begin(), a.end(), active);
  std::copy(em.begin(), em.end(), empty);
  std::copy(s.begin(), s.end(), task_states);
  *n_active = (uint32_t)a.size();
  *n_empty = (uint32_t)em.size();
  return RDN_OK;
}

rdn_status rdn_task_graph_check_errors(rdn_task_graph* g, void* stream, uint32_t* flags) {
  if (!g || !flags) return RDN_ERR_INVALID_ARG;
  cudaError_t e = cudaSetDevice(g->ctx->device);
  if (e == cudaSuccess) e = g->graph.read_error(flags, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "task graph error word");
  return RDN_OK;
}

rdn_status rdn_ao_pipeline_create(rdn_ctx* c, uint32_t width, uint32_t height, void* stream, rdn_task_graph** out) {
  if (!c || !out) return fail(c, RDN_ERR_INVALID_ARG, "null context or output");
  if (width == 0 || height == 0 || (uint64_t)width * height * 2 >= (1ull << 28))
    return fail(c, RDN_ERR_INVALID_ARG, "AO pipeline frame must have 1..2^27 pixels");
  rdn_task_group_desc g[5];
  std::memset(g, 0, sizeof(g));
  // 0: ray-trace task (max_in_flight_trace_ray(2))
  g[0].program = RDN_TASK_PROGRAM_TRACE;
  g[0].max_in_flight = 2;
  g[0].payload_words = 16;
  // 1: ray generation: then_trace(camera ray).map(accumulate)
  g[1].max_in_flight = 1;
  g[1].payload_words = 1;
  g[1].n_spawn = 1;
  g[1].spawn_type[0] = 0;
  g[1].spawn_op[0] = RDN_TASK_SPAWN_AO_PRIMARY;
  g[1].map_op = RDN_TASK_MAP_AO_ACCUMULATE;
  // 2: primary closest hit: then_trace(occlusion ray).map(store the result)
  g[2].max_in_flight = 1;
  g[2].payload_words = 24;
  g[2].n_spawn = 1;
  g[2].spawn_type[0] = 0;
  g[2].spawn_op[0] = RDN_TASK_SPAWN_AO_OCCLUSION;
  g[2].map_op = RDN_TASK_MAP_STORE_CHILD;
  // 3: occlusion closest hit: payload 0
  g[3].max_in_flight = 1;
  g[3].payload_words = 24;
  g[3].map_op = RDN_TASK_MAP_STORE_ZERO;
  // 4: miss: payload 1
  g[4].max_in_flight = 1;
  g[4].payload_words = 16;
  g[4].map_op = RDN_TASK_MAP_STORE_ONE;
  // one ray-generation task per dispatch index, 4x8 pixel tiles (ao_pixel)
  rdn_status st = rdn_task_graph_create(c, g, 5, rdn::ao_dispatch_count(width, height), stream, out);
  if (st != RDN_OK) return st;
  (*out)->ao_pipeline = true;
  (*out)->width = width;
  (*out)->height = height;
  return RDN_OK;
}

}  // extern "C"

namespace {

// One AO frame on the pipeline graph: dispatch, then the reference's 8 rounds,
// or (inside a capture) a device-ended loop of at most 8 rounds.
rdn_status ao_graph_frame(rdn_task_graph* g, const rdn_ao_desc* d, cudaStream_t s, bool until_empty) {
  rdn_ctx* c = g->ctx;
  if (!g->ao_pipeline) return fail(c, RDN_ERR_INVALID_ARG, "not an AO pipeline graph");
  if (d->width != g->width || d->height != g->height)
    return fail(c, RDN_ERR_INVALID_ARG, "frame size differs from the pipeline's");
  rdn_ao_desc env = *d;
  env.sbt_closest[0] = 2;
  env.sbt_closest[1] = 3;
  env.sbt_miss = 4;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess)
    e = g->graph.dispatch_init(1, rdn::ao_dispatch_count(d->width, d->height), RDN_TASK_INIT_INDEX, s);
  if (e != cudaSuccess) return cuda_fail(c, e, "task graph dispatch");
  rdn_status st = run_rounds(g, 8, &env, s, until_empty);
  if (st != RDN_OK || !d->sample_counter) return st;
  e = rdn::launch_ao_advance(d->sample_counter, s);
  return e == cudaSuccess ? RDN_OK : cuda_fail(c, e, "AO sample counter");
}

}  // namespace

extern "C" {

rdn_status rdn_ao_render_graph(rdn_task_graph* g, const rdn_ao_desc* d, void* stream) {
  if (!g || !d) return RDN_ERR_INVALID_ARG;
  return ao_graph_frame(g, d, static_cast<cudaStream_t>(stream), false);
}

rdn_status rdn_ao_render(rdn_ctx* c, const rdn_ao_desc* d, void* stream) {
  Range range_("rdn_ao_render");
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  std::lock_guard<std::mutex> lk(c->lock);
  rdn::TraceParams p;
  rdn::AoEnv a;
  rdn_status st = ao_env(c, d, p, a);
  if (st != RDN_OK) return st;
  cudaError_t e = cudaSetDevice(c->device);
  if (e == cudaSuccess) e = rdn::launch_ao(p, a, mode_of(d->traversal), static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess && d->sample_counter) e = rdn::launch_ao_advance(d->sample_counter, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(c, e, "AO launch");
  return RDN_OK;
}

rdn_status rdn_ao_capture(rdn_ctx* c, rdn_task_graph* pipeline, const rdn_ao_desc* d, rdn_graph** out) {
  Range range_("rdn_ao_capture");
  if (!c || !d || !out) return fail(c, RDN_ERR_INVALID_ARG, "null context, descriptor or output");
  *out = nullptr;
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (pipeline && pipeline->ctx != c) return fail(c, RDN_ERR_INVALID_ARG, "the pipeline belongs to another context");
  rdn_status st = require_built(c);
  if (st != RDN_OK) return st;
  return capture_graph(
      c, "AO frame capture",
      [&](cudaStream_t s) { return pipeline ? ao_graph_frame(pipeline, d, s, true) : rdn_ao_render(c, d, s); },
      out);
}

rdn_status rdn_pt_scratch_size(uint32_t width, uint32_t height, size_t* bytes) {
  if (!bytes || (uint64_t)width * height > 0x7FFFFFFFull) return RDN_ERR_INVALID_ARG;
  *bytes = rdn::pt_scratch_bytes(width, height);
  return RDN_OK;
}

static_assert(sizeof(rdn_pt_material) == sizeof(rdn::PtMaterial), "rdn_pt_material layout");
static_assert(sizeof(rdn_pt_directional_light) == sizeof(rdn::PtLight), "rdn_pt_directional_light layout");

rdn_status rdn_path_tracing_render(rdn_ctx* c, const rdn_pt_desc* d, void* stream) {
  Range range_("rdn_path_tracing_render");
  if (!c || !d) return fail(c, RDN_ERR_INVALID_ARG, "null context or descriptor");
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  if (d->tone_map > RDN_TONE_MAP_ACES_FILMIC) return fail(c, RDN_ERR_INVALID_ARG, "unknown tone map");
  if (d->background > RDN_PT_BACKGROUND_ENV_CUBE) return fail(c, RDN_ERR_INVALID_ARG, "unknown background");
  if (d->background == RDN_PT_BACKGROUND_ENV_CUBE &&
      (!d->env_cube || d->env_size == 0 || d->env_size > 16384 || (reinterpret_cast<uintptr_t>(d->env_cube) & 15)))
    return fail(c, RDN_ERR_INVALID_ARG, "the environment cube needs 16-byte aligned faces of 1..16384 texels");
  if (d->max_path_depth > 64) return fail(c, RDN_ERR_INVALID_ARG, "max_path_depth must be at most 64");
  if (d->light_count && !d->lights) return fail(c, RDN_ERR_INVALID_ARG, "null lights with light_count > 0");
  if (d->material_count && !d->materials)
    return fail(c, RDN_ERR_INVALID_ARG, "null materials with material_count > 0");
  if (d->sm_count && !d->sm_to_material)
    return fail(c, RDN_ERR_INVALID_ARG, "null sm_to_material with sm_count > 0");
  if ((reinterpret_cast<uintptr_t>(d->lights) & 3) || (reinterpret_cast<uintptr_t>(d->materials) & 3) ||
      (reinterpret_cast<uintptr_t>(d->sm_to_material) & 3) || (reinterpret_cast<uintptr_t>(d->normals) & 3))
    return fail(c, RDN_ERR_INVALID_ARG, "lights, materials, sm_to_material and normals must be 4-byte aligned");
  if (reinterpret_cast<uintptr_t>(d->radiance) & 15)
    return fail(c, RDN_ERR_INVALID_ARG, "radiance must be 16-byte aligned");
  if (reinterpret_cast<uintptr_t>(d->sample_counter) & 3)
    return fail(c, RDN_ERR_INVALID_ARG, "sample_counter must be 4-byte aligned");
  if (d->schedule > RDN_PT_SCHEDULE_WAVEFRONT) return fail(c, RDN_ERR_INVALID_ARG, "unknown schedule");
  if (d->schedule == RDN_PT_SCHEDULE_WAVEFRONT) {
    if (!d->scratch || (reinterpret_cast<uintptr_t>(d->scratch) & 255))
      return fail(c, RDN_ERR_INVALID_ARG, "the wavefront schedule needs 256-byte aligned scratch");
    if (d->scratch_bytes < rdn::pt_scratch_bytes(d->width, d->height))
      return fail(c, RDN_ERR_INVALID_ARG, "scratch smaller than rdn_pt_scratch_size()");
  }
  if (d->register_tier > 2) return fail(c, RDN_ERR_INVALID_ARG, "register_tier must be 0, 1 or 2");
  std::lock_guard<std::mutex> lk(c->lock);
  rdn_ao_desc ad;
  std::memset(&ad, 0, sizeof(ad));
  std::memcpy(ad.view_projection_inv, d->view_projection_inv, sizeof(ad.view_projection_inv));
  std::memcpy(ad.camera_position, d->camera_position, sizeof(ad.camera_position));
  ad.width = d->width;
  ad.height = d->height;
  ad.sample_count = d->sample_count;
  ad.tlas_uniform = d->tlas_uniform;
  ad.traversal = d->traversal;
  ad.normals = d->normals;
  ad.image = d->image;
  ad.block_size = d->block_size;
  ad.ray_counts = d->ray_counts;
  ad.sample_counter = d->sample_counter;
  ad.speculation = d->speculation;
  rdn::TraceParams p;
  rdn::PtEnv e;
  std::memset(&e, 0, sizeof(e));
  rdn_status st = ao_env(c, &ad, p, e.view);
  if (st != RDN_OK) return st;
  e.max_depth = d->max_path_depth;
  e.tone_map = d->tone_map;
  e.exposure = d->exposure;
  e.background = d->background;
  std::memcpy(e.bg, d->background_color, sizeof(e.bg));
  e.lights = reinterpret_cast<const rdn::PtLight*>(d->lights);
  e.light_count = d->light_count;
  e.materials = reinterpret_cast<const rdn::PtMaterial*>(d->materials);
  e.material_count = d->material_count;
  e.sm_to_material = d->sm_to_material;
  e.sm_count = d->sm_count;
  e.radiance = reinterpret_cast<float4*>(d->radiance);
  e.schedule = d->schedule;
  e.register_tier = d->register_tier;
  e.env = reinterpret_cast<const float4*>(d->env_cube);
  e.env_size = d->env_size;
  std::memcpy(e.env_transform, d->env_transform, sizeof(e.env_transform));
  e.env_intensity = d->env_intensity;
  e.fetch = c->d_counters + 13;
  rdn::PtWave w;
  std::memset(&w, 0, sizeof(w));
  if (d->schedule == RDN_PT_SCHEDULE_WAVEFRONT) w = rdn::pt_wave_layout(d->scratch, d->width, d->height);
  cudaError_t err = cudaSetDevice(c->device);
  if (err == cudaSuccess)
    err = rdn::launch_pt(p, e, &w, mode_of(d->traversal), c->sm_count, static_cast<cudaStream_t>(stream));
  if (err == cudaSuccess && d->sample_counter)
    err = rdn::launch_ao_advance(d->sample_counter, static_cast<cudaStream_t>(stream));
  if (err != cudaSuccess) return cuda_fail(c, err, "path tracing launch");
  return RDN_OK;
}

rdn_status rdn_pt_capture(rdn_ctx* c, const rdn_pt_desc* d, rdn_graph** out) {
  Range range_("rdn_pt_capture");
  if (!c || !d || !out) return fail(c, RDN_ERR_INVALID_ARG, "null context, descriptor or output");
  *out = nullptr;
  if (c->device < 0) return fail(c, RDN_ERR_UNSUPPORTED, "host-only context cannot trace");
  rdn_status st = require_built(c);
  if (st != RDN_OK) return st;
  return capture_graph(
      c, "path-traced frame capture", [&](cudaStream_t s) { return rdn_path_tracing_render(c, d, s); }, out);
}

}  // extern "C"
