// Wavefront executor for the first bounce of the path tracer, sm_103a.
//
// The reference runs raygen -> trace -> closest-hit -> (shadow trace, bounce)
// as device tasks whose queues are compacted every round by a two-level
// Kogge-Stone prefix scan plus a shuffle move
// (shader/ray-tracing/src/backend/wavefront_compute/mod.rs:111-196,
// shader/task-graph/src/runtime/task_group.rs:176-278,
// shader/parallel-compute/src/stream_compaction.rs:3-45). Here the fixed
// pipeline of DeviceReferencePathTracingRenderer's first bounce
// (scene/rendering/gpu-ray-tracing/src/feature/path_tracing/{ray_gen.rs,ray_hit.rs})
// is two kernels:
//
//   primary_kernel: one thread per pixel, warps mapped to 8x4 pixel tiles.
//     Pinhole ray -> closest hit -> geometric normal facing the ray ->
//     offset_ray_hit origin -> one shadow ray to the point light and one
//     cosine-weighted bounce ray, appended to two queues that share one
//     counter: a warp ballot and one atomicAdd per warp reserve the slots, so
//     the queues come out compacted without a separate scan pass.
//   secondary_kernel: persistent warps that fetch 32 queue entries at a time
//     from a global work counter; shadow rays (first-hit search) occupy the
//     first half of the index space and bounce rays (closest hit) the second,
//     so warps stay homogeneous. Results scatter to the pixel records.
//
// Built with -fmad=false: all shading arithmetic is IEEE f32 in the same
// order as the oracle, so secondary rays are bit-identical.
#include <cuda_runtime.h>

#include <cstdint>

#include "traverse.cuh"
#include "wavefront.h"

namespace rdn {
namespace {

using namespace dev;

constexpr float F32_EPSILON = 1.1920929e-7f;
constexpr float F32_MAX = 3.40282347e+38f;

__device__ __forceinline__ uint32_t pcg_next(uint32_t& state) {
  const uint32_t prev = state * 747796405u + 2891336453u;
  const uint32_t word = ((prev >> ((prev >> 28u) + 4u)) ^ prev) * 277803737u;
  state = prev;
  return (word >> 22u) ^ word;
}
__device__ __forceinline__ float sample_next(uint32_t& state) {
  return __uint_as_float(0x3f800000u | (pcg_next(state) >> 9u)) - 1.0f;
}
__device__ __forceinline__ uint32_t rotl17(uint32_t h) { return (h << 17) | (h >> 15); }
__device__ __forceinline__ uint32_t xxhash32(uint32_t x, uint32_t y, uint32_t z) {
  uint32_t h = z + 374761393u + x * 3266489917u;
  h = 668265263u * rotl17(h);
  h = h + y * 3266489917u;
  h = 668265263u * rotl17(h);
  h = 2246822519u * (h ^ (h >> 15));
  h = 3266489917u * (h ^ (h >> 13));
  return h ^ (h >> 16);
}
// Taylor polynomials on [-pi/4, pi/4], evaluated identically on host and device.
__device__ __forceinline__ float poly_sin(float x) {
  const float x2 = x * x;
  float p = 2.7557319e-6f;
  p = -1.9841270e-4f + x2 * p;
  p = 8.3333333e-3f + x2 * p;
  p = -1.6666667e-1f + x2 * p;
  return x + x * (x2 * p);
}
__device__ __forceinline__ float poly_cos(float x) {
  const float x2 = x * x;
  float p = -2.7557319e-7f;
  p = 2.4801587e-5f + x2 * p;
  p = -1.3888889e-3f + x2 * p;
  p = 4.1666667e-2f + x2 * p;
  p = -0.5f + x2 * p;
  return 1.0f + x2 * p;
}

__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float3 normalize3(float3 v) {
  const float mag_sq = dot3(v, v);
  if (mag_sq > 0.0f) return v * (1.0f / sqrtf(mag_sq));
  return v;
}

// cosine_sample_hemisphere_in_dir (math/statistics/src/distribution_map.rs:29-58)
__device__ __forceinline__ float3 cosine_sample_in_dir(float3 dir, float sx, float sy) {
  const float ux = sx * 2.0f - 1.0f, uy = sy * 2.0f - 1.0f;
  float dx = 0.0f, dy = 0.0f;
  if (!(ux == 0.0f && uy == 0.0f)) {
    float r, c, s;
    if (fabsf(ux) > fabsf(uy)) {
      r = ux;
      const float phi = 0.78539819f * (uy / ux);
      c = poly_cos(phi);
      s = poly_sin(phi);
    } else {
      r = uy;
      const float phi = 0.78539819f * (ux / uy);
      c = poly_sin(phi);
      s = poly_cos(phi);
    }
    dx = c * r;
    dy = s * r;
  }
  const float oz = sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy));
  const float3 left = normalize3(cross3(make_float3(0.0f, 1.0f, 0.0f), dir));
  const float3 up = cross3(left, dir);
  const float xy_r = sqrtf(dx * dx + dy * dy);
  if (xy_r == 0.0f) return dir;
  const float cos_phi = dx / xy_r, sin_phi = dy / xy_r;
  const float3 v = left * xy_r * cos_phi + up * xy_r * sin_phi + dir * oz;
  return normalize3(v);
}

// offset_ray_hit (scene/rendering/gpu-ray-tracing/src/ray_util.rs:5-40)
__device__ __forceinline__ float offset_axis(float p, float n) {
  const int32_t of_i = (int32_t)(n * 256.0f);
  const float p_i = __uint_as_float(__float_as_uint(p) + (uint32_t)((p < 0.0f) ? -of_i : of_i));
  return (fabsf(p) < 0.03125f) ? (p + 1.52587891e-5f * n) : p_i;
}
__device__ __forceinline__ float3 offset_ray_hit(float3 p, float3 n) {
  return make_float3(offset_axis(p.x, n.x), offset_axis(p.y, n.y), offset_axis(p.z, n.z));
}

// Warp-aggregated append: every lane with `want` gets a unique slot.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
  const uint32_t active = __activemask();
  const uint32_t mask = __ballot_sync(active, want);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t leader = __ffs(active) - 1;
  uint32_t base = 0;
  if (lane == leader && mask) base = atomicAdd(counter, __popc(mask));
  base = __shfl_sync(active, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

template <bool ORDERED>
__global__ void __launch_bounds__(128) primary_kernel(TraceParams p, WavefrontParams w) {
  extern __shared__ uint2 smem_stack[];
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t warp = gtid >> 5, lane = gtid & 31u;
  const uint32_t tiles_x = (w.width + 7u) / 8u;
  const uint32_t px = (warp % tiles_x) * 8u + (lane & 7u);
  const uint32_t py = (warp / tiles_x) * 4u + (lane >> 3);
  const bool valid = px < w.width && py < w.height;

  bool want = false;
  float3 org = make_float3(0.f, 0.f, 0.f), ldir = org, bdir = org;
  float dist = 0.0f;
  if (valid) {
    // camera ray (pixel centre), the same f32 steps as the host generator
    const float sx = (((float)px + 0.5f) / (float)w.width * 2.0f - 1.0f) * w.tan_half * w.aspect;
    const float sy = (1.0f - ((float)py + 0.5f) / (float)w.height * 2.0f) * w.tan_half;
    const float3 d = normalize3(make_float3((w.forward.x + sx * w.right.x) + sy * w.up.x,
                                            (w.forward.y + sx * w.right.y) + sy * w.up.y,
                                            (w.forward.z + sx * w.right.z) + sy * w.up.z));
    RayCtx R;
    R.o = w.origin;
    R.d = d;
    R.tmin = 0.0f;
    R.tmax = __int_as_float(0x7f800000);
    R.cull_mask = 0xFFu;
    R.ray_flags = 0u;
    bool bad;
    traverse_ray<ORDERED, false>(p, R, w.tlas, smem_stack + threadIdx.x, blockDim.x, bad);
    PixelResult out;
    out.primary_prim = INVALID_NEXT;
    out.primary_t = R.tmax;
    out.bounce_prim = INVALID_NEXT;
    out.bounce_t = F32_MAX;
    out.primary_flags = 0u;
    out.light = 0u;
    out.direct = 0.0f;
    out.primary_instance = INVALID_NEXT;
    if (R.best.have) {
      const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + R.best.geom_slot));
      out.primary_prim = __ldg(p.redirect + R.best.k) - gm.z;
      out.primary_t = R.best.t;
      out.primary_flags = 1u;
      out.primary_instance = R.best.inst;
      // hit point and world geometric normal facing the incoming ray
      const float3 hp = R.o + d * R.best.t;
      const float4* rec = p.tris + 4 * (size_t)R.best.k;
      const float3 n = make_float3(__ldg(&rec[0].w), __ldg(&rec[1].w), __ldg(&rec[2].w));
      const float* m = p.tlas_data[R.best.inst].transform_inv;
      const float3 nw = normalize3(make_float3(n.x * __ldg(m + 0) + n.y * __ldg(m + 1) + n.z * __ldg(m + 2),
                                               n.x * __ldg(m + 4) + n.y * __ldg(m + 5) + n.z * __ldg(m + 6),
                                               n.x * __ldg(m + 8) + n.y * __ldg(m + 9) + n.z * __ldg(m + 10)));
      const float3 nf = dot3(nw, d) < 0.0f ? nw : make_float3(-nw.x, -nw.y, -nw.z);
      org = offset_ray_hit(hp, nf);
      const float3 L = w.light - org;
      const float dist2 = dot3(L, L);
      dist = sqrtf(dist2);
      ldir = normalize3(L);
      out.direct = fmaxf(0.0f, dot3(nf, ldir)) / dist2;  // kept only if the light is visible
      uint32_t state = xxhash32(px, py, w.sample_index * 3u);
      const float s0 = sample_next(state);
      const float s1 = sample_next(state);
      bdir = cosine_sample_in_dir(nf, s0, s1);
      want = true;
    }
    w.out[(size_t)py * w.width + px] = out;
  }
  // compacted append of both secondary rays (one counter for the pair)
  const uint32_t slot = warp_append(w.queue_count, want);
  if (want) {
    const uint32_t pix = py * w.width + px;
    float4* sq = reinterpret_cast<float4*>(w.shadow_rays) + 2 * (size_t)slot;
    sq[0] = make_float4(org.x, org.y, org.z, F32_EPSILON);
    sq[1] = make_float4(ldir.x, ldir.y, ldir.z, dist);
    float4* bq = reinterpret_cast<float4*>(w.bounce_rays) + 2 * (size_t)slot;
    bq[0] = make_float4(org.x, org.y, org.z, F32_EPSILON);
    bq[1] = make_float4(bdir.x, bdir.y, bdir.z, F32_MAX);
    w.shadow_pixel[slot] = pix;
    w.bounce_pixel[slot] = pix;
  }
}

template <bool ORDERED>
__global__ void __launch_bounds__(128) secondary_kernel(TraceParams p, WavefrontParams w) {
  extern __shared__ uint2 smem_stack[];
  const uint32_t n = *(volatile uint32_t*)w.queue_count;
  const uint32_t total = 2u * n;
  const uint32_t lane = threadIdx.x & 31u;
  if (blockIdx.x == 0 && threadIdx.x == 0 && w.ray_counts) {
    w.ray_counts[0] = w.width * w.height;
    w.ray_counts[1] = n;
    w.ray_counts[2] = n;
  }
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(w.work_counter, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const uint32_t j = base + lane;
    if (j < total) {
      const bool shadow = j < n;
      const uint32_t q = shadow ? j : j - n;
      const float4* rq = reinterpret_cast<const float4*>(shadow ? w.shadow_rays : w.bounce_rays) + 2 * (size_t)q;
      const float4 r0 = rq[0], r1 = rq[1];
      RayCtx R;
      R.o = make_float3(r0.x, r0.y, r0.z);
      R.tmin = r0.w;
      R.d = make_float3(r1.x, r1.y, r1.z);
      R.tmax = r1.w;
      R.cull_mask = 0xFFu;
      R.ray_flags = shadow ? TF_END_SEARCH : 0u;
      bool bad;
      traverse_ray<ORDERED, false>(p, R, w.tlas, smem_stack + threadIdx.x, blockDim.x, bad);
      if (shadow) {
        PixelResult* o = w.out + w.shadow_pixel[q];
        o->light = R.best.have ? 2u : 1u;
        if (R.best.have) o->direct = 0.0f;
      } else {
        PixelResult* o = w.out + w.bounce_pixel[q];
        if (R.best.have) {
          const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + R.best.geom_slot));
          o->bounce_prim = __ldg(p.redirect + R.best.k) - gm.z;
          o->bounce_t = R.best.t;
        }
      }
    }
  }
}

}  // namespace

size_t wavefront_scratch_bytes(uint32_t width, uint32_t height) {
  const size_t n = (size_t)width * height;
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  return 256 + 2 * up(n * 32) + 2 * up(n * 4);
}

void wavefront_bind_scratch(WavefrontParams& w, void* scratch) {
  const size_t n = (size_t)w.width * w.height;
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  char* s = static_cast<char*>(scratch);
  w.queue_count = reinterpret_cast<uint32_t*>(s);
  w.work_counter = reinterpret_cast<uint32_t*>(s + 64);
  size_t off = 256;
  w.shadow_rays = s + off;
  off += up(n * 32);
  w.bounce_rays = s + off;
  off += up(n * 32);
  w.shadow_pixel = reinterpret_cast<uint32_t*>(s + off);
  off += up(n * 4);
  w.bounce_pixel = reinterpret_cast<uint32_t*>(s + off);
}

cudaError_t launch_wavefront(const TraceParams& p, const WavefrontParams& w, bool ordered, uint32_t block,
                             int sm_count, uint32_t phases, cudaStream_t stream) {
  if (phases == 0) phases = 3;
  if (block == 0) block = 128;
  const size_t n = (size_t)w.width * w.height;
  if (n == 0) return cudaSuccess;
  const size_t smem = ordered ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static bool attr_done[2] = {false, false};
  const void* fns[4] = {(const void*)primary_kernel<false>, (const void*)secondary_kernel<false>,
                        (const void*)primary_kernel<true>, (const void*)secondary_kernel<true>};
  if (!attr_done[ordered ? 1 : 0]) {
    for (int k = 0; k < 2; k++) {
      cudaError_t e = cudaFuncSetAttribute(fns[(ordered ? 2 : 0) + k], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           200 * 1024);
      if (e != cudaSuccess) return e;
    }
    attr_done[ordered ? 1 : 0] = true;
  }
  cudaError_t e;
  if (phases & 1u) {
    e = cudaMemsetAsync(w.queue_count, 0, 64, stream);
    if (e != cudaSuccess) return e;
    // primary grid: whole 8x4 tiles, one warp each
    const uint32_t tiles = ((w.width + 7) / 8) * ((w.height + 3) / 4);
    const uint32_t threads = tiles * 32;
    const uint32_t grid1 = (threads + block - 1) / block;
    if (ordered) primary_kernel<true><<<grid1, block, smem, stream>>>(p, w);
    else primary_kernel<false><<<grid1, block, smem, stream>>>(p, w);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (!(phases & 2u)) return cudaSuccess;
  e = cudaMemsetAsync(w.work_counter, 0, 64, stream);
  if (e != cudaSuccess) return e;
  // persistent secondary grid: enough resident blocks to fill every SM
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fns[(ordered ? 2 : 0) + 1], (int)block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const uint32_t grid2 = (uint32_t)(sm_count * per_sm);
  if (ordered) secondary_kernel<true><<<grid2, block, smem, stream>>>(p, w);
  else secondary_kernel<false><<<grid2, block, smem, stream>>>(p, w);
  return cudaGetLastError();
}

}  // namespace rdn
