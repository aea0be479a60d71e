// Path-tracing frame for sm_103a: the reference path tracer's ray generation
// (path_tracing/ray_gen.rs:89-211), closest hit with its shadow trace
// (ray_hit.rs:12-103), shadow closest hit / miss (mod.rs:197-209) and miss
// (ray_miss.rs:10-28) fused into one kernel. A path is a small state machine
// (PtPath) advanced one ray at a time: the core ray and the shadow ray of a hit
// take turns through one traversal call site, so the kernel holds one inlined
// traversal instead of two. Two schedules:
//   fused   one thread per pixel, warps over 4x8 pixel tiles; a warp runs until
//           its longest path ends;
//   refill  persistent warps: a lane whose path ends takes the next pixel
//           (warp-aggregated atomic on a frame counter), so warps stay full
//           until the frame runs out (Aila and Laine 2009, "persistent
//           while-while" with dynamic fetch, at path granularity);
//   wavefront  one pass per ray kind and depth over queues of pixel indices,
//           the path state in HBM between passes: every warp traces rays of
//           one kind (camera, bounce or shadow).
// All compute each pixel with the same operations. Built with -fmad=false:
// see pt.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "pt.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

struct PtPath {
  uint32_t x, y;
  float3 o, d, throughput, radiance;
  float3 sn, origin, ldir, lrad;  // the hit carried across its shadow trace
  uint32_t sm_id, depth, core, shadow;
  bool shadow_phase;
};

__device__ __forceinline__ void pt_begin(const PtEnv& E, PtPath& q, uint32_t x, uint32_t y) {
  q.x = x;
  q.y = y;
  ao_camera_ray(E.view, x, y, q.o, q.d);
  q.throughput = splat3(1.0f);
  q.radiance = splat3(0.0f);
  q.sn = q.origin = q.ldir = q.lrad = splat3(0.0f);
  q.sm_id = 0;
  q.depth = 0;
  q.core = 0;
  q.shadow = 0;
  q.shadow_phase = false;
}

// The ray the path traces next.
__device__ __forceinline__ void pt_ray(const PtPath& q, RayCtx& R) {
  R.o = q.shadow_phase ? q.origin : q.o;
  R.d = q.shadow_phase ? q.ldir : q.d;
  R.tmin = F32_EPSILON;
  R.tmax = F32_MAX;  // core: RayRange::default; shadow: the directional light's distance
  R.ray_flags = q.shadow_phase ? RAY_FLAG_END_SEARCH : RAY_FLAG_CULL_BACK;
  R.cull_mask = 0xFFFFFFFFu;
}

// Consumes the traced ray's result; returns true when the path has ended.
__device__ __forceinline__ bool pt_advance(const TraceParams& P, const PtEnv& E, uint32_t sample, PtPath& q,
                                           const RayCtx& R) {
  if (!q.shadow_phase) {
    q.core++;
    if (!R.best.have) {  // miss shader, then the ray generation's miss branch
      const float3 s = pt_miss(E, q.d);
      q.radiance = make_float3((q.throughput.x * s.x + 0.0f) + q.radiance.x,
                               (q.throughput.y * s.y + 0.0f) + q.radiance.y,
                               (q.throughput.z * s.z + 0.0f) + q.radiance.z);
      return true;
    }
    // closest hit, first part: light sample and shadow ray
    const float3 hit = q.o + q.d * R.best.t;
    const DeviceInstance* inst = P.tlas_data + R.best.inst;
    float3 gn;
    q.sn = hit_normals(E.view, inst, __ldg(P.redirect + R.best.k), R.best.u, R.best.v, q.o, hit, gn);
    q.sm_id = __ldg(&inst->instance_custom_index);
    uint32_t ls = xxhash32(q.x, q.y, sample * 2u);
    const float r = sample_next(ls);
    const uint32_t n_lights = E.light_count;
    uint32_t li = (uint32_t)floorf(r * (float)n_lights);
    const bool light_ok = n_lights != 0u;
    if (li == n_lights && light_ok) li = li - 1u;
    const float pmf = n_lights == 0u ? 0.0f : 1.0f / (float)n_lights;
    float3 illum = splat3(0.0f), dir = splat3(0.0f);
    if (light_ok) {
      const float* lp = reinterpret_cast<const float*>(E.lights + li);
      illum = make_float3(__ldg(lp + 0), __ldg(lp + 1), __ldg(lp + 2));
      dir = make_float3(__ldg(lp + 3), __ldg(lp + 4), __ldg(lp + 5));
    }
    q.ldir = neg3(dir);
    const float pdf_l = 1.0f * pmf;
    q.lrad = light_ok ? illum / pdf_l : splat3(0.0f);
    q.origin = offset_ray_hit(hit, gn);
    if (light_ok) {
      q.shadow_phase = true;
      return false;
    }
  } else {
    q.shadow++;
    if (R.best.have) q.lrad = splat3(0.0f);  // shadow closest hit
    q.shadow_phase = false;
  }
  // closest hit, map: BRDF sample, direct light through the BRDF
  const float3 view = neg3(q.d);
  const PtSurface s = pt_surface(E, q.sm_id);
  uint32_t bs = xxhash32(q.x, q.y, sample * 3u);
  float3 brdf;
  float pdf;
  const float3 sdir = pt_sample(s, view, q.sn, bs, brdf, pdf);
  const float3 brdf_l = pt_bsdf(s, view, q.ldir, q.sn);
  const float light_dot = fabsf(dot3(q.sn, q.ldir));
  const float3 sampled = make_float3((light_dot * brdf_l.x) * q.lrad.x, (light_dot * brdf_l.y) * q.lrad.y,
                                     (light_dot * brdf_l.z) * q.lrad.z);
  // ray generation's hit branch
  if (pdf == 0.0f) q.depth = E.max_depth;
  q.depth = q.depth + 1u;
  const float cosv = dot3(sdir, q.sn);
  const float pdf_c = fmaxf(pdf, PT_MIN_PDF);
  q.throughput = make_float3(((q.throughput.x * cosv) * brdf.x) / pdf_c, ((q.throughput.y * cosv) * brdf.y) / pdf_c,
                             ((q.throughput.z * cosv) * brdf.z) / pdf_c);
  q.radiance = make_float3(q.throughput.x * sampled.x + q.radiance.x, q.throughput.y * sampled.y + q.radiance.y,
                           q.throughput.z * sampled.z + q.radiance.z);
  q.o = q.origin;
  q.d = sdir;
  return q.depth >= E.max_depth;
}

// Ray generation's resolve: tone map and running average; the HDR record.
__device__ __forceinline__ void pt_finish(const PtEnv& E, const PtPath& q) {
  const uint32_t pixel = q.y * E.view.width + q.x;
  pt_accumulate(E, pixel, pt_tone_map(E, q.radiance));
  if (E.radiance) E.radiance[pixel] = make_float4(q.radiance.x, q.radiance.y, q.radiance.z, (float)q.core);
}

// A path's state parked in shared memory while its ray is traced, so that
// the traversal's registers are not held alongside it (word k of thread t at
// [k][t], conflict-free; blocks of at most 128 threads). A static array: with
// the park area in dynamic shared memory, indexed by blockDim.x, the compiler
// kept more registers and the 1080p sample took 3.38 ms instead of 3.05 ms.
constexpr uint32_t kPtStash = 26;
__device__ __forceinline__ void pt_park(float (*stash)[128], const PtPath& q) {
  const uint32_t t = threadIdx.x;
  const float v[kPtStash] = {q.o.x, q.o.y, q.o.z, q.d.x, q.d.y, q.d.z, q.throughput.x, q.throughput.y,
                             q.throughput.z, q.radiance.x, q.radiance.y, q.radiance.z, q.sn.x, q.sn.y, q.sn.z,
                             q.origin.x, q.origin.y, q.origin.z, q.ldir.x, q.ldir.y, q.ldir.z, q.lrad.x, q.lrad.y,
                             q.lrad.z, __uint_as_float(q.sm_id), __uint_as_float(q.depth)};
#pragma unroll
  for (uint32_t k = 0; k < kPtStash; k++) stash[k][t] = v[k];
}
__device__ __forceinline__ void pt_unpark(float (*stash)[128], PtPath& q) {
  const uint32_t t = threadIdx.x;
  q.o = make_float3(stash[0][t], stash[1][t], stash[2][t]);
  q.d = make_float3(stash[3][t], stash[4][t], stash[5][t]);
  q.throughput = make_float3(stash[6][t], stash[7][t], stash[8][t]);
  q.radiance = make_float3(stash[9][t], stash[10][t], stash[11][t]);
  q.sn = make_float3(stash[12][t], stash[13][t], stash[14][t]);
  q.origin = make_float3(stash[15][t], stash[16][t], stash[17][t]);
  q.ldir = make_float3(stash[18][t], stash[19][t], stash[20][t]);
  q.lrad = make_float3(stash[21][t], stash[22][t], stash[23][t]);
  q.sm_id = __float_as_uint(stash[24][t]);
  q.depth = __float_as_uint(stash[25][t]);
}

__device__ __forceinline__ void pt_count(const PtEnv& E, uint32_t core, uint32_t shadow) {
  if (!E.view.ray_counts) return;
  const uint32_t c = __reduce_add_sync(0xffffffffu, core), s = __reduce_add_sync(0xffffffffu, shadow);
  if ((threadIdx.x & 31u) == 0u) {
    if (c) atomicAdd(E.view.ray_counts + 0, c);
    if (s) atomicAdd(E.view.ray_counts + 1, s);
  }
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) pt_kernel(TraceParams P, PtEnv E) {
  RDN_TRAVERSAL_STACK(LOCAL);
  __shared__ float stash[kPtStash][128];
  uint32_t x, y;
  const bool valid = ao_pixel(E.view, blockIdx.x * blockDim.x + threadIdx.x, x, y);
  uint32_t core = 0, shadow = 0;
  if (valid) {
    const uint32_t sample = ao_sample(E.view);
    PtPath q;
    pt_begin(E, q, x, y);
    bool bad = false, done = E.max_depth == 0u;
    while (!done) {
      RayCtx R;
      pt_ray(q, R);
      pt_park(stash, q);
      bool b;
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, E.view.tlas, stack_ptr, stack_stride, b);
      bad |= b;
      pt_unpark(stash, q);
      done = pt_advance(P, E, sample, q, R);
    }
    if (bad) atomicOr(P.error_word, 2u);
    pt_finish(E, q);
    core = q.core;
    shadow = q.shadow;
  }
  pt_count(E, core, shadow);
}

// Register budget of the refill kernel (local-stack walks): 0 = the
// compiler's choice for 128-thread blocks, 1 = at least 5 such blocks per SM
// (at most 96 registers), 2 = at least 8 (at most 64).
constexpr int pt_min_blocks(int tier) { return tier == 1 ? 5 : (tier == 2 ? 8 : 0); }

template <int MODE, bool LOCAL, bool WT, int TIER>
__global__ void __launch_bounds__(128, pt_min_blocks(TIER)) pt_refill_kernel(TraceParams P, PtEnv E, uint32_t total) {
  RDN_TRAVERSAL_STACK(LOCAL);
  __shared__ float stash[kPtStash][128];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t sample = ao_sample(E.view);
  PtPath q;
  bool active = false, exhausted = false, bad = false;
  uint32_t core = 0, shadow = 0;
  for (;;) {
    // lanes without a path take the next dispatch indices, one atomic per warp
    const bool need = !active && !exhausted;
    const uint32_t m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const uint32_t leader = __ffs(m) - 1u;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(E.fetch, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const uint32_t idx = base + __popc(m & ((1u << lane) - 1u));
        uint32_t x, y;
        if (idx >= total) {
          exhausted = true;
        } else if (ao_pixel(E.view, idx, x, y)) {
          pt_begin(E, q, x, y);
          if (E.max_depth == 0u) pt_finish(E, q);  // a path of no rays resolves at once
          else active = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (active) {
      RayCtx R;
      pt_ray(q, R);
      pt_park(stash, q);
      bool b;
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, E.view.tlas, stack_ptr, stack_stride, b);
      bad |= b;
      pt_unpark(stash, q);
      if (pt_advance(P, E, sample, q, R)) {
        pt_finish(E, q);
        core += q.core;
        shadow += q.shadow;
        active = false;
      }
    }
  }
  if (bad) atomicOr(P.error_word, 2u);
  pt_count(E, core, shadow);
}

// ---- wavefront schedule ----
// Path state word-major (word k of pixel i at state[k * n_pix + i]):
// o 0-2, d 3-5, throughput 6-8, radiance 9-11, shading normal 12-14,
// shadow origin 15-17, light direction 18-20, light radiance 21-23, sm_id 24,
// depth 25, core rays 26, shadow rays 27.
__device__ __forceinline__ void pt_st3(uint32_t* s, uint32_t n, uint32_t k, uint32_t i, float3 v) {
  s[(size_t)k * n + i] = __float_as_uint(v.x);
  s[(size_t)(k + 1) * n + i] = __float_as_uint(v.y);
  s[(size_t)(k + 2) * n + i] = __float_as_uint(v.z);
}
__device__ __forceinline__ float3 pt_ld3(const uint32_t* s, uint32_t n, uint32_t k, uint32_t i) {
  return make_float3(__uint_as_float(s[(size_t)k * n + i]), __uint_as_float(s[(size_t)(k + 1) * n + i]),
                     __uint_as_float(s[(size_t)(k + 2) * n + i]));
}
__device__ __forceinline__ void pt_save(const PtWave& W, uint32_t i, const PtPath& q) {
  uint32_t* s = W.state;
  const uint32_t n = W.n_pix;
  pt_st3(s, n, 0, i, q.o);
  pt_st3(s, n, 3, i, q.d);
  pt_st3(s, n, 6, i, q.throughput);
  pt_st3(s, n, 9, i, q.radiance);
  pt_st3(s, n, 12, i, q.sn);
  pt_st3(s, n, 15, i, q.origin);
  pt_st3(s, n, 18, i, q.ldir);
  pt_st3(s, n, 21, i, q.lrad);
  s[(size_t)24 * n + i] = q.sm_id;
  s[(size_t)25 * n + i] = q.depth;
  s[(size_t)26 * n + i] = q.core;
  s[(size_t)27 * n + i] = q.shadow;
}
__device__ __forceinline__ void pt_load(const PtWave& W, uint32_t i, uint32_t width, PtPath& q) {
  const uint32_t* s = W.state;
  const uint32_t n = W.n_pix;
  q.x = i % width;
  q.y = i / width;
  q.o = pt_ld3(s, n, 0, i);
  q.d = pt_ld3(s, n, 3, i);
  q.throughput = pt_ld3(s, n, 6, i);
  q.radiance = pt_ld3(s, n, 9, i);
  q.sn = pt_ld3(s, n, 12, i);
  q.origin = pt_ld3(s, n, 15, i);
  q.ldir = pt_ld3(s, n, 18, i);
  q.lrad = pt_ld3(s, n, 21, i);
  q.sm_id = s[(size_t)24 * n + i];
  q.depth = s[(size_t)25 * n + i];
  q.core = s[(size_t)26 * n + i];
  q.shadow = s[(size_t)27 * n + i];
}

// One pass of the wavefront schedule: persistent warps take 32 queue entries
// at a time; each lane traces its path's next ray (all core rays or all
// shadow rays: with lights the passes alternate core, shadow, core, ...,
// since every core hit casts a shadow ray and every shadow ray is followed by
// a core ray), advances the path and queues it for the next pass or resolves
// its pixel. Pass 0 starts the paths from the camera, 4x8 pixel tiles per warp.
template <int MODE, bool LOCAL, bool WT, int TIER>
__global__ void __launch_bounds__(128, pt_min_blocks(TIER))
    pt_pass_kernel(TraceParams P, PtEnv E, PtWave W, uint32_t pass, uint32_t shadow_pass) {
  RDN_TRAVERSAL_STACK(LOCAL);
  __shared__ float stash[kPtStash][128];
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t sample = ao_sample(E.view);
  const uint32_t width = E.view.width;
  const uint32_t total = pass == 0 ? ao_dispatch_count(E.view.width, E.view.height) : W.counters[pass - 1];
  const uint32_t* qin = W.queue[(pass + 1) & 1];
  uint32_t* qout = W.queue[pass & 1];
  uint32_t* fetch = W.counters + kPtMaxPasses + pass;
  uint32_t core = 0, shadow = 0;
  bool bad = false;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(fetch, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    const uint32_t i = base + lane;
    PtPath q;
    uint32_t pix = 0;
    bool live = false;
    if (i < total) {
      if (pass == 0) {
        uint32_t x, y;
        if (ao_pixel(E.view, i, x, y)) {
          pt_begin(E, q, x, y);
          pix = y * width + x;
          live = E.max_depth != 0u;
          if (!live) pt_finish(E, q);  // a path of no rays resolves at once
        }
      } else {
        pix = qin[i];
        pt_load(W, pix, width, q);
        q.shadow_phase = shadow_pass != 0u;
        live = true;
      }
    }
    bool cont = false;
    if (live) {
      RayCtx R;
      pt_ray(q, R);
      pt_park(stash, q);
      bool b;
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, E.view.tlas, stack_ptr, stack_stride, b);
      bad |= b;
      pt_unpark(stash, q);
      if (pt_advance(P, E, sample, q, R)) {
        pt_finish(E, q);
        core += q.core;
        shadow += q.shadow;
      } else {
        pt_save(W, pix, q);
        cont = true;
      }
    }
    const uint32_t slot = warp_append(W.counters + pass, cont);
    if (cont) qout[slot] = pix;
  }
  if (bad) atomicOr(P.error_word, 2u);
  pt_count(E, core, shadow);
}

template <int MODE, bool LOCAL, bool WT, int TIER>
cudaError_t launch_passes(const TraceParams& p, const PtEnv& e, const PtWave& w, int sm_count, uint32_t block,
                          size_t smem, cudaStream_t st) {
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t err = raise_smem_limit(attr_done, {(const void*)pt_pass_kernel<MODE, LOCAL, WT, TIER>});
  if (err != cudaSuccess) return err;
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pt_pass_kernel<MODE, LOCAL, WT, TIER>, (int)block,
                                                      smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  const uint32_t total = ao_dispatch_count(e.view.width, e.view.height);
  uint32_t grid = (uint32_t)((sm_count > 0 ? sm_count : 1) * per_sm);
  const uint32_t need = (total + block - 1) / block;
  if (grid > need) grid = need;
  err = cudaMemsetAsync(w.counters, 0, 2 * kPtMaxPasses * sizeof(uint32_t), st);
  if (err != cudaSuccess) return err;
  const bool lights = e.light_count != 0u;
  const uint32_t passes = std::max<uint32_t>(1u, lights ? 2u * e.max_depth : e.max_depth);
  for (uint32_t pass = 0; pass < passes; pass++) {
    pt_pass_kernel<MODE, LOCAL, WT, TIER><<<grid, block, smem, st>>>(p, e, w, pass, lights ? (pass & 1u) : 0u);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
  }
  return cudaSuccess;
}

template <int MODE, bool LOCAL, bool WT, int TIER>
cudaError_t launch_refill(const TraceParams& p, const PtEnv& e, int sm_count, uint32_t block, size_t smem,
                          cudaStream_t st) {
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t err = raise_smem_limit(attr_done, {(const void*)pt_refill_kernel<MODE, LOCAL, WT, TIER>});
  if (err != cudaSuccess) return err;
  const uint32_t total = ao_dispatch_count(e.view.width, e.view.height);
  int per_sm = 0;
  err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pt_refill_kernel<MODE, LOCAL, WT, TIER>, (int)block,
                                                      smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  uint32_t grid = (uint32_t)((sm_count > 0 ? sm_count : 1) * per_sm);
  const uint32_t need = (total + block - 1) / block;
  if (grid > need) grid = need;
  err = cudaMemsetAsync(e.fetch, 0, 4, st);
  if (err != cudaSuccess) return err;
  pt_refill_kernel<MODE, LOCAL, WT, TIER><<<grid, block, smem, st>>>(p, e, total);
  return cudaGetLastError();
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_variant_wt(const TraceParams& p, const PtEnv& e, const PtWave* w, int sm_count, cudaStream_t st) {
  const uint32_t block = e.view.block ? e.view.block : 128;
  const uint32_t total = ao_dispatch_count(e.view.width, e.view.height);
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  if (e.schedule == 2u) {
    if constexpr (LOCAL) {
      if (e.register_tier == 1) return launch_passes<MODE, LOCAL, WT, 1>(p, e, *w, sm_count, block, smem, st);
      if (e.register_tier == 2) return launch_passes<MODE, LOCAL, WT, 2>(p, e, *w, sm_count, block, smem, st);
    }
    return launch_passes<MODE, LOCAL, WT, 0>(p, e, *w, sm_count, block, smem, st);
  }
  if (!e.schedule) {
    static std::atomic<uint64_t> attr_done{0};
    const cudaError_t err = raise_smem_limit(attr_done, {(const void*)pt_kernel<MODE, LOCAL, WT>});
    if (err != cudaSuccess) return err;
    pt_kernel<MODE, LOCAL, WT><<<(total + block - 1) / block, block, smem, st>>>(p, e);
    return cudaGetLastError();
  }
  // register tiers apply to the local-stack walks
  if constexpr (LOCAL) {
    if (e.register_tier == 1) return launch_refill<MODE, LOCAL, WT, 1>(p, e, sm_count, block, smem, st);
    if (e.register_tier == 2) return launch_refill<MODE, LOCAL, WT, 2>(p, e, sm_count, block, smem, st);
  }
  return launch_refill<MODE, LOCAL, WT, 0>(p, e, sm_count, block, smem, st);
}

template <int MODE, bool LOCAL>
cudaError_t launch_variant(const TraceParams& p, const PtEnv& e, const PtWave* w, int sm_count, cudaStream_t st) {
  return p.watertight ? launch_variant_wt<MODE, LOCAL, true>(p, e, w, sm_count, st)
                      : launch_variant_wt<MODE, LOCAL, false>(p, e, w, sm_count, st);
}

constexpr size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

size_t pt_scratch_bytes(uint32_t width, uint32_t height) {
  const size_t n = (size_t)width * height;
  return align256(n * kPtStateWords * 4) + 2 * align256(n * 4) + align256(2 * kPtMaxPasses * 4);
}

PtWave pt_wave_layout(void* scratch, uint32_t width, uint32_t height) {
  const size_t n = (size_t)width * height;
  char* b = static_cast<char*>(scratch);
  PtWave w;
  w.n_pix = (uint32_t)n;
  w.state = reinterpret_cast<uint32_t*>(b);
  b += align256(n * kPtStateWords * 4);
  w.queue[0] = reinterpret_cast<uint32_t*>(b);
  b += align256(n * 4);
  w.queue[1] = reinterpret_cast<uint32_t*>(b);
  b += align256(n * 4);
  w.counters = reinterpret_cast<uint32_t*>(b);
  return w;
}

cudaError_t launch_pt(const TraceParams& p, const PtEnv& e, const PtWave* w, int mode, int sm_count, cudaStream_t st) {
  if (e.view.width == 0 || e.view.height == 0) return cudaSuccess;
  if (mode == MODE_WIDE4)
    return p.local_stack ? launch_variant<MODE_WIDE4, true>(p, e, w, sm_count, st)
                         : launch_variant<MODE_WIDE4, false>(p, e, w, sm_count, st);
  if (mode == MODE_BINARY)
    return p.local_stack ? launch_variant<MODE_BINARY, true>(p, e, w, sm_count, st)
                         : launch_variant<MODE_BINARY, false>(p, e, w, sm_count, st);
  return launch_variant<MODE_THREADED, false>(p, e, w, sm_count, st);
}

}  // namespace rdn
