// Batched multi-scene path tracing, sm_103a.
//
// The reference's path tracer (scene/rendering/gpu-ray-tracing/src/feature/path_tracing/
// ray_gen.rs:89-211, ray_hit.rs:12-103) loops up to max_path_depth bounces per
// pixel through the task graph, one wavefront round per bounce. Here every ray
// of every scene goes through one persistent launch per bounce:
//
//   path_kernel: warps fetch 32 queue entries at a time from a global work
//   counter (load balance across scenes of very different size and across
//   paths of different length); each entry is a 32 B ray plus a 16 B path
//   state {output id, TLAS index, throughput, flags}. Closest hit in the
//   entry's own scene (the reference's per-ray tlas_idx, traverse_cpu.rs:63),
//   then one cosine-weighted diffuse bounce from an offset_ray_hit origin,
//   Russian roulette from the configured bounce on, and a warp-ballot /
//   one-atomic-per-warp append of the surviving path to the next queue.
//
// Path semantics (shared with the oracle): albedo a; a miss at bounce k
// writes radiance = throughput (sky = 1) and depth k; a hit at k == max_bounces
// or a path killed by roulette writes radiance 0. The sampler for bounce k of
// path i is xxhash32(i, k, seed) -> next() x3 (direction, roulette).
// Built with -fmad=false, like every traversal unit.
#include <cuda_runtime.h>

#include <cstdint>

#include "parallel.h"
#include "paths.h"
#include "shade.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

// Queue of bounce b: rays (2 float4) and states {id, tlas, throughput, 0}.
// from_user: bounce 0 reads the caller's primary rays instead of a queue.
template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) path_kernel(TraceParams p, PathParams q, uint32_t bounce, bool from_user,
                                                   const float4* __restrict__ in_rays,
                                                   const uint4* __restrict__ in_state, float4* __restrict__ out_rays,
                                                   uint4* __restrict__ out_state) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const uint32_t n = bounce == 0 ? q.count : *(volatile uint32_t*)(q.queue_count + bounce - 1);
  const uint32_t lane = threadIdx.x & 31u;
  uint32_t* work = q.work_counter + bounce;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(work, 32u);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= n) break;
    const uint32_t j = base + lane;
    bool keep = false;
    float4 nr0 = make_float4(0.f, 0.f, 0.f, 0.f), nr1 = nr0;
    uint4 ns = make_uint4(0u, 0u, 0u, 0u);
    if (j < n) {
      float4 r0, r1;
      uint32_t id, tlas;
      float throughput;
      if (from_user) {
        const float4* rp = q.primary_rays + 2 * (size_t)j;
        r0 = __ldg(rp);
        r1 = __ldg(rp + 1);
        id = j;
        tlas = q.tlas_idx ? __ldg(q.tlas_idx + j) : q.tlas_uniform;
        throughput = 1.0f;
      } else {
        r0 = in_rays[2 * (size_t)j];
        r1 = in_rays[2 * (size_t)j + 1];
        const uint4 s = in_state[j];
        id = s.x;
        tlas = s.y;
        throughput = __uint_as_float(s.z);
      }
      RayCtx R;
      R.o = make_float3(r0.x, r0.y, r0.z);
      R.tmin = r0.w;
      R.d = make_float3(r1.x, r1.y, r1.z);
      R.tmax = r1.w;
      R.cull_mask = 0xFFu;
      R.ray_flags = 0u;
      bool bad;
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, tlas, stack_ptr, stack_stride, bad);
      if (!R.best.have) {
        q.out[id] = make_float2(throughput, __uint_as_float(bounce | RDN_PATH_ESCAPED));
      } else if (bounce == q.max_bounces) {
        q.out[id] = make_float2(0.0f, __uint_as_float(bounce));
      } else {
        uint32_t st = xxhash32(id, bounce, q.seed);
        const float s0 = sample_next(st);
        const float s1 = sample_next(st);
        const float s2 = sample_next(st);
        float t_next = throughput * q.albedo;
        bool survive = true;
        if (bounce + 1 >= q.rr_start) {
          survive = s2 < q.rr_survive;
          t_next = t_next / q.rr_survive;
        }
        if (!survive) {
          q.out[id] = make_float2(0.0f, __uint_as_float(bounce | RDN_PATH_ROULETTE));
        } else {
          const float3 hp = R.o + R.d * R.best.t;
          const float3 nf = facing_normal(p, R.best.k, R.best.inst, R.d);
          const float3 org = offset_ray_hit(hp, nf);
          const float3 dir = cosine_sample_in_dir(nf, s0, s1);
          nr0 = make_float4(org.x, org.y, org.z, 1.1920929e-7f);
          nr1 = make_float4(dir.x, dir.y, dir.z, 3.40282347e+38f);
          ns = make_uint4(id, tlas, __float_as_uint(t_next), 0u);
          keep = true;
        }
      }
    }
    const uint32_t slot = warp_append(q.queue_count + bounce, keep);
    if (keep) {
      out_rays[2 * (size_t)slot] = nr0;
      out_rays[2 * (size_t)slot + 1] = nr1;
      out_state[slot] = ns;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && q.segment_counts) q.segment_counts[bounce] = n;
}

// The same bounce with dynamic fetch (ordered walks only, q.refill > 0): every
// lane keeps its own resumable query (LaneWalk) and the warp claims new queue
// entries for its idle lanes whenever at least q.refill of them are idle, so
// that a few long paths do not hold a whole warp. Rays of different scenes and
// directions are mixed anyway, so no coherence is lost by refilling. The
// shading and the warp-aggregated append run for the lanes that finished in
// the round; iterations are capped (error-word bit 2).
template <int MODE, bool WT>
__global__ void __launch_bounds__(128, 8) path_dynamic_kernel(TraceParams p, PathParams q, uint32_t bounce,
                                                              bool from_user, const float4* __restrict__ in_rays,
                                                              const uint4* __restrict__ in_state,
                                                              float4* __restrict__ out_rays,
                                                              uint4* __restrict__ out_state) {
  extern __shared__ uint2 smem_stack[];
  constexpr int WIDTH = MODE == MODE_WIDE4 ? 4 : 2;
  const uint32_t n = bounce == 0 ? q.count : *(volatile uint32_t*)(q.queue_count + bounce - 1);
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lanes_below = (1u << lane) - 1u;
  uint32_t* work = q.work_counter + bounce;
  uint2* stack = smem_stack + threadIdx.x;
  const uint32_t threshold = q.refill < 1u ? 1u : (q.refill > 32u ? 32u : q.refill);
  LaneWalk<WIDTH, WT> L;
  L.reset();
  uint32_t id = 0, tlas = 0;
  float throughput = 0.0f;
  bool exhausted = false;
  for (uint32_t iter = 0;; iter++) {
    if (iter >= walk_round_cap(p)) {
      if (lane == 0) atomicOr(p.error_word, 4u);
      break;
    }
    const uint32_t idle = __ballot_sync(0xffffffffu, L.phase == WALK_IDLE);
    if (!exhausted && (__popc(idle) >= threshold || idle == 0xffffffffu)) {
      const uint32_t cnt = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(work, cnt);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + cnt >= n) exhausted = true;
      if (L.phase == WALK_IDLE) {
        const uint32_t j = base + __popc(idle & lanes_below);
        if (j < n) {
          float4 r0, r1;
          if (from_user) {
            const float4* rp = q.primary_rays + 2 * (size_t)j;
            r0 = __ldg(rp);
            r1 = __ldg(rp + 1);
            id = j;
            tlas = q.tlas_idx ? __ldg(q.tlas_idx + j) : q.tlas_uniform;
            throughput = 1.0f;
          } else {
            r0 = in_rays[2 * (size_t)j];
            r1 = in_rays[2 * (size_t)j + 1];
            const uint4 st = in_state[j];
            id = st.x;
            tlas = st.y;
            throughput = __uint_as_float(st.z);
          }
          L.start(p, r0, r1, tlas, 0u);
        }
      }
    }
    if (exhausted && __ballot_sync(0xffffffffu, L.phase != WALK_IDLE) == 0u) break;
    if (L.phase != WALK_IDLE) L.advance(p, stack, blockDim.x, threshold);
    bool keep = false;
    float4 nr0 = make_float4(0.f, 0.f, 0.f, 0.f), nr1 = nr0;
    uint4 ns = make_uint4(0u, 0u, 0u, 0u);
    if (L.phase == WALK_DONE) {
      const RayCtx& R = L.R;
      if (!R.best.have) {
        q.out[id] = make_float2(throughput, __uint_as_float(bounce | RDN_PATH_ESCAPED));
      } else if (bounce == q.max_bounces) {
        q.out[id] = make_float2(0.0f, __uint_as_float(bounce));
      } else {
        uint32_t st = xxhash32(id, bounce, q.seed);
        const float s0 = sample_next(st);
        const float s1 = sample_next(st);
        const float s2 = sample_next(st);
        float t_next = throughput * q.albedo;
        bool survive = true;
        if (bounce + 1 >= q.rr_start) {
          survive = s2 < q.rr_survive;
          t_next = t_next / q.rr_survive;
        }
        if (!survive) {
          q.out[id] = make_float2(0.0f, __uint_as_float(bounce | RDN_PATH_ROULETTE));
        } else {
          const float3 hp = R.o + R.d * R.best.t;
          const float3 nf = facing_normal(p, R.best.k, R.best.inst, R.d);
          const float3 org = offset_ray_hit(hp, nf);
          const float3 dir = cosine_sample_in_dir(nf, s0, s1);
          nr0 = make_float4(org.x, org.y, org.z, 1.1920929e-7f);
          nr1 = make_float4(dir.x, dir.y, dir.z, 3.40282347e+38f);
          ns = make_uint4(id, tlas, __float_as_uint(t_next), 0u);
          keep = true;
        }
      }
      L.phase = WALK_IDLE;
    }
    const uint32_t slot = warp_append(q.queue_count + bounce, keep);
    if (keep) {
      out_rays[2 * (size_t)slot] = nr0;
      out_rays[2 * (size_t)slot + 1] = nr1;
      out_state[slot] = ns;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && q.segment_counts) q.segment_counts[bounce] = n;
}

// Primary rays into queue form (only when the executor sorts rays).
__global__ void path_prime_kernel(PathParams q, float4* __restrict__ rays, uint4* __restrict__ state) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= q.count) return;
  rays[2 * (size_t)i] = __ldg(q.primary_rays + 2 * (size_t)i);
  rays[2 * (size_t)i + 1] = __ldg(q.primary_rays + 2 * (size_t)i + 1);
  state[i] = make_uint4(i, q.tlas_idx ? __ldg(q.tlas_idx + i) : q.tlas_uniform, __float_as_uint(1.0f), 0u);
}

__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

// Sort key of queue entry i (entries at or past the live count are skipped).
__global__ void path_key_kernel(TraceParams p, PathParams q, const float4* __restrict__ rays,
                                const uint4* __restrict__ state, const uint32_t* __restrict__ n_dev) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = n_dev ? *n_dev : q.count;
  if (i >= n) return;
  const float4 r0 = rays[2 * (size_t)i], r1 = rays[2 * (size_t)i + 1];
  const uint32_t tlas = state[i].y;
  const uint32_t oct = (r1.x < 0.0f ? 1u : 0u) | (r1.y < 0.0f ? 2u : 0u) | (r1.z < 0.0f ? 4u : 0u);
  uint32_t key = (tlas << 3) | oct;
  if (q.sort_key == 2) {
    uint32_t cell = 0;
    if (tlas < p.n_binding) {
      const uint32_t h = __ldg(p.tlas_binding + tlas);
      const uint32_t root = h < p.n_tlas_root ? __ldg(p.tlas_bvh_root + h) : INVALID_NEXT;
      if (root != INVALID_NEXT) {
        const float* b = reinterpret_cast<const float*>(p.tlas_forest + root);
        const float lo[3] = {__ldg(b), __ldg(b + 1), __ldg(b + 2)}, hi[3] = {__ldg(b + 4), __ldg(b + 5), __ldg(b + 6)};
        const float o[3] = {r0.x, r0.y, r0.z};
        uint32_t c[3];
        for (int a = 0; a < 3; a++) {
          const float ext = hi[a] - lo[a];
          const float f = ext > 0.0f ? (o[a] - lo[a]) / ext * 16.0f : 0.0f;
          c[a] = f <= 0.0f ? 0u : (f >= 15.0f ? 15u : (uint32_t)f);
        }
        cell = spread4(c[0]) | (spread4(c[1]) << 1) | (spread4(c[2]) << 2);
      }
    }
    key = (key << 12) | cell;
  }
  q.keys[i] = key;
  q.idx[i] = i;
}

__global__ void path_gather_kernel(PathParams q, const float4* __restrict__ in_rays, const uint4* __restrict__ in_state,
                                   float4* __restrict__ out_rays, uint4* __restrict__ out_state,
                                   const uint32_t* __restrict__ n_dev) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = n_dev ? *n_dev : q.count;
  if (i >= n) return;
  const uint32_t j = q.idx[i];
  out_rays[2 * (size_t)i] = in_rays[2 * (size_t)j];
  out_rays[2 * (size_t)i + 1] = in_rays[2 * (size_t)j + 1];
  out_state[i] = in_state[j];
}

}  // namespace

size_t paths_scratch_bytes(uint32_t count, uint32_t max_bounces, uint32_t sort_key) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t n = count;
  size_t bytes = 256 + up(sizeof(uint32_t) * 2 * (max_bounces + 1)) + 2 * up(n * 32) + 2 * up(n * 16);
  if (sort_key) bytes += 2 * up(n * 4) + sort_scratch_bytes(count);
  return bytes;
}

void paths_bind_scratch(PathParams& q, void* scratch) {
  auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t n = q.count;
  char* s = static_cast<char*>(scratch);
  q.queue_count = reinterpret_cast<uint32_t*>(s + 256);
  q.work_counter = q.queue_count + (q.max_bounces + 1);
  size_t off = 256 + up(sizeof(uint32_t) * 2 * (q.max_bounces + 1));
  q.rays_a = s + off;
  off += up(n * 32);
  q.rays_b = s + off;
  off += up(n * 32);
  q.state_a = s + off;
  off += up(n * 16);
  q.state_b = s + off;
  off += up(n * 16);
  if (q.sort_key) {
    q.keys = reinterpret_cast<uint32_t*>(s + off);
    off += up(n * 4);
    q.idx = reinterpret_cast<uint32_t*>(s + off);
    off += up(n * 4);
    q.sort_scratch = s + off;
  }
}

namespace {
// kernel variant: 0 batch, 1 dynamic fetch, 2 batch with local-memory stacks
int path_variant(int mode, const TraceParams& p, const PathParams& q) {
  if (mode == MODE_THREADED) return 0;
  if (q.refill != 0) return 1;
  return p.local_stack ? 2 : 0;
}
template <bool WT>
const void* path_fn_wt(int mode, int variant) {
  if (mode == MODE_WIDE4)
    return variant == 1 ? (const void*)path_dynamic_kernel<MODE_WIDE4, WT>
                        : (variant == 2 ? (const void*)path_kernel<MODE_WIDE4, true, WT>
                                        : (const void*)path_kernel<MODE_WIDE4, false, WT>);
  if (mode == MODE_BINARY)
    return variant == 1 ? (const void*)path_dynamic_kernel<MODE_BINARY, WT>
                        : (variant == 2 ? (const void*)path_kernel<MODE_BINARY, true, WT>
                                        : (const void*)path_kernel<MODE_BINARY, false, WT>);
  return (const void*)path_kernel<MODE_THREADED, false, WT>;
}
const void* path_fn(int mode, int variant, bool wt) {
  return wt ? path_fn_wt<true>(mode, variant) : path_fn_wt<false>(mode, variant);
}

// One bounce launch of the variant chosen by path_variant.
template <bool WT>
void launch_bounce(int mode, int variant, uint32_t grid, uint32_t block, size_t smem, cudaStream_t stream,
                   const TraceParams& p, const PathParams& q, uint32_t b, bool from_user, const float4* in_r,
                   const uint4* in_s, float4* out_r, uint4* out_s) {
  if (mode == MODE_WIDE4 && variant == 1)
    path_dynamic_kernel<MODE_WIDE4, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else if (mode == MODE_WIDE4 && variant == 2)
    path_kernel<MODE_WIDE4, true, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else if (mode == MODE_WIDE4)
    path_kernel<MODE_WIDE4, false, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else if (mode == MODE_BINARY && variant == 1)
    path_dynamic_kernel<MODE_BINARY, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else if (mode == MODE_BINARY && variant == 2)
    path_kernel<MODE_BINARY, true, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else if (mode == MODE_BINARY)
    path_kernel<MODE_BINARY, false, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
  else
    path_kernel<MODE_THREADED, false, WT><<<grid, block, smem, stream>>>(p, q, b, from_user, in_r, in_s, out_r, out_s);
}
}  // namespace

cudaError_t prepare_paths(const TraceParams& p, const PathParams& q, int mode, uint32_t block, int sm_count,
                          uint32_t* grid) {
  if (block == 0) block = 64;
  const int variant = path_variant(mode, p, q);
  const size_t smem = mode != MODE_THREADED && variant != 2 ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done[2][3][3] = {};
  const void* fn = path_fn(mode, variant, p.watertight != 0);
  cudaError_t e = raise_smem_limit(attr_done[p.watertight ? 1 : 0][variant][mode], {fn});
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  // persistent grid, never larger than the primary queue needs
  uint32_t g = (uint32_t)(sm_count * per_sm);
  const uint32_t need = (q.count + block - 1) / block;
  *grid = g > need ? need : g;
  return cudaSuccess;
}

cudaError_t record_paths(const TraceParams& p, const PathParams& q, int mode, uint32_t block, uint32_t grid,
                         cudaStream_t stream) {
  if (block == 0) block = 64;
  if (q.count == 0 || grid == 0) return cudaSuccess;
  const int variant = path_variant(mode, p, q);
  const size_t smem = mode != MODE_THREADED && variant != 2 ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  cudaError_t e = cudaMemsetAsync(q.queue_count, 0, sizeof(uint32_t) * 2 * (q.max_bounces + 1), stream);
  if (e != cudaSuccess) return e;
  float4* ra = static_cast<float4*>(q.rays_a);
  float4* rb = static_cast<float4*>(q.rays_b);
  uint4* sa = static_cast<uint4*>(q.state_a);
  uint4* sb = static_cast<uint4*>(q.state_b);
  const uint32_t eg = (q.count + 255) / 256;
  if (q.sort_key) {
    path_prime_kernel<<<eg, 256, 0, stream>>>(q, ra, sa);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  for (uint32_t b = 0; b <= q.max_bounces; b++) {
    const float4* in_r;
    const uint4* in_s;
    float4* out_r;
    uint4* out_s;
    bool from_user = false;
    if (q.sort_key) {
      // regroup the queue in A by key into B, trace B, append to A
      const uint32_t* n_dev = b == 0 ? nullptr : q.queue_count + b - 1;
      path_key_kernel<<<eg, 256, 0, stream>>>(p, q, ra, sa, n_dev);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = radix_sort_u32(q.keys, q.idx, q.count, q.key_bits, q.sort_scratch, stream, n_dev);
      if (e != cudaSuccess) return e;
      path_gather_kernel<<<eg, 256, 0, stream>>>(q, ra, sa, rb, sb, n_dev);
      e = cudaGetLastError();
      if (e != cudaSuccess) return e;
      in_r = rb;
      in_s = sb;
      out_r = ra;
      out_s = sa;
    } else {
      from_user = b == 0;
      in_r = (b & 1) ? rb : ra;
      in_s = (b & 1) ? sb : sa;
      out_r = (b & 1) ? ra : rb;
      out_s = (b & 1) ? sa : sb;
    }
    if (p.watertight)
      launch_bounce<true>(mode, variant, grid, block, smem, stream, p, q, b, from_user, in_r, in_s, out_r, out_s);
    else
      launch_bounce<false>(mode, variant, grid, block, smem, stream, p, q, b, from_user, in_r, in_s, out_r, out_s);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace rdn
