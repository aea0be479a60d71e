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
//   primary_kernel: one thread per pixel, persistent warps that claim 4x8
//     pixel tiles (4 wide, 8 tall) from a counter. Pinhole ray -> closest hit -> geometric normal facing the ray ->
//     offset_ray_hit origin -> one shadow ray to the point light and one
//     cosine-weighted bounce ray. The shadow queue and the two bins of the
//     bounce queue (grazing rays at its front, steep rays at its back) are
//     filled through warp ballots and one 64-bit atomicAdd per warp, so the
//     queues come out compacted without a separate scan pass.
//   secondary_kernel: persistent warps that fetch 32 queue entries at a time
//     from a global work counter; the grazing bounce rays, then the steep
//     ones (closest hit, the long walks), occupy the first half of the index
//     space and shadow rays (first-hit search) the second, so warps stay
//     homogeneous and the kernel ends on short work. Results scatter to the
//     pixel records.
//
// Built with -fmad=false: all shading arithmetic is IEEE f32 in the same
// order as the oracle, so secondary rays are bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "shade.cuh"
#include "traverse.cuh"
#include "wavefront.h"

namespace rdn {
namespace {

using namespace dev;

// LOCAL: the traversal stack lives in the thread's local memory (L1-cached)
// instead of shared memory, so that the stack no longer limits occupancy.
// TIER picks the register budget through the launch bounds: 0 = the
// compiler's default for 128-thread blocks (64 registers, some spills),
// 1 = at least 7 blocks of 128 per SM (72 registers, no spills, 28 warps),
// 2 = at least 9 blocks (56 registers, 36 warps, more spills).
constexpr int min_blocks(int tier) { return tier == 1 ? 7 : (tier == 2 ? 9 : 0); }

// Bounce rays leaving their surface at a cosine of at least 1/2 (three
// quarters of a cosine-weighted sample) go to the back bin of the bounce
// queue; the grazing quarter, the longest walks, to its front.
constexpr float kSteepBounceCos = 0.5f;

// Queue entry of the j-th bounce ray of the secondary kernel's index space:
// the n_front grazing rays from the queue's front, then the steep ones from
// its back (entry cap - 1 down).
__device__ __forceinline__ uint32_t bounce_entry(uint32_t j, uint32_t n_front, uint32_t cap) {
  return j < n_front ? j : cap - 1u - (j - n_front);
}

template <int MODE, bool LOCAL, int TIER, bool WT>
__global__ void __launch_bounds__(128, min_blocks(TIER)) primary_kernel(TraceParams p, WavefrontParams w) {
  extern __shared__ uint2 smem_stack[];
  uint2 local_stack[LOCAL ? kLocalStackEntries : 1];
  uint2* const stack = LOCAL ? local_stack : smem_stack + threadIdx.x;
  const uint32_t stride = LOCAL ? 1u : blockDim.x;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t tiles_x = (w.width + 3u) / 4u;
  const uint32_t tiles = tiles_x * ((w.height + 7u) / 8u);
  // persistent: each warp claims 4x8 pixel tiles from a counter until none is
  // left, so that a warp that finishes early does not wait for its block
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(w.tile_counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= tiles) break;
    const uint32_t px = (tile % tiles_x) * 4u + (lane & 3u);
    const uint32_t py = (tile / tiles_x) * 8u + (lane >> 2);
    const bool valid = px < w.width && py < w.height;

    bool want = false;
    float3 org = make_float3(0.f, 0.f, 0.f), ldir = org, bdir = org;
    float dist = 0.0f, bcos = 0.0f;
    if (valid) {
      // camera ray (pixel centre), the same f32 steps as the host generator
      const float sx = (((float)px + 0.5f) / (float)w.width * 2.0f - 1.0f) * w.tan_half * w.aspect;
      const float sy = (1.0f - ((float)(py + w.row0) + 0.5f) / (float)w.frame_height * 2.0f) * w.tan_half;
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
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, w.tlas, stack, stride, bad);
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
        const float3 nf = facing_normal(p, R.best.k, R.best.inst, d);
        org = offset_ray_hit(hp, nf);
        const float3 L = w.light - org;
        const float dist2 = dot3(L, L);
        dist = sqrtf(dist2);
        ldir = normalize3(L);
        out.direct = fmaxf(0.0f, dot3(nf, ldir)) / dist2;  // kept only if the light is visible
        uint32_t state = xxhash32(px, py + w.row0, w.sample_index * 3u);
        const float s0 = sample_next(state);
        const float s1 = sample_next(state);
        bdir = cosine_sample_in_dir(nf, s0, s1);
        bcos = dot3(bdir, nf);
        want = true;
      }
      w.out[(size_t)py * w.width + px] = out;
    }
    // compacted appends: shadow rays to their queue; bounce rays to two bins of
    // theirs, grazing ones (the longer walks) from its front and steep ones
    // from its back, so that a warp of the secondary kernel traces rays of
    // like walk lengths. One 64-bit atomic per warp counts both bins (low and
    // high word); the shadow slot is the sum of the two bases plus the lane's
    // rank, so the shadow queue stays dense. Every lane of the warp is here.
    const bool steep = want && bcos >= kSteepBounceCos;
    const uint32_t m_want = __ballot_sync(0xffffffffu, want), m_steep = __ballot_sync(0xffffffffu, steep);
    const uint32_t m_front = m_want & ~m_steep;
    unsigned long long bases = 0ull;
    if (lane == 0 && m_want)
      bases = atomicAdd(w.bins, (unsigned long long)__popc(m_front) | ((unsigned long long)__popc(m_steep) << 32));
    bases = __shfl_sync(0xffffffffu, bases, 0);
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t front = (uint32_t)bases + __popc(m_front & below);
    const uint32_t back = (uint32_t)(bases >> 32) + __popc(m_steep & below);
    const uint32_t slot = (uint32_t)bases + (uint32_t)(bases >> 32) + __popc(m_want & below);
    if (want) {
      const uint32_t pix = py * w.width + px;
      float4* sq = reinterpret_cast<float4*>(w.shadow_rays) + 2 * (size_t)slot;
      sq[0] = make_float4(org.x, org.y, org.z, F32_EPSILON);
      sq[1] = make_float4(ldir.x, ldir.y, ldir.z, dist);
      const uint32_t bslot = steep ? w.width * w.height - 1u - back : front;
      float4* bq = reinterpret_cast<float4*>(w.bounce_rays) + 2 * (size_t)bslot;
      bq[0] = make_float4(org.x, org.y, org.z, F32_EPSILON);
      bq[1] = make_float4(bdir.x, bdir.y, bdir.z, F32_MAX);
      w.shadow_pixel[slot] = pix;
      w.bounce_pixel[bslot] = pix;
    }
  }
}

template <int MODE, bool LOCAL, int TIER, bool WT>
__global__ void __launch_bounds__(128, min_blocks(TIER)) secondary_kernel(TraceParams p, WavefrontParams w) {
  extern __shared__ uint2 smem_stack[];
  uint2 local_stack[LOCAL ? kLocalStackEntries : 1];
  uint2* const stack = LOCAL ? local_stack : smem_stack + threadIdx.x;
  const uint32_t stride = LOCAL ? 1u : blockDim.x;
  const unsigned long long bins = *(volatile unsigned long long*)w.bins;
  const uint32_t n_front = (uint32_t)bins, n = n_front + (uint32_t)(bins >> 32);
  const uint32_t cap = w.width * w.height;
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
      // bounce rays first: they are the longest walks, and a persistent kernel
      // that ends on short shadow rays leaves fewer warps waiting for a last
      // long batch (1.66 -> 1.54 ms on the 1080p frame)
      const bool shadow = j >= n;
      const uint32_t q = shadow ? j - n : bounce_entry(j, n_front, cap);
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
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(p, R, w.tlas, stack, stride, bad);
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

// Secondary rays with dynamic fetch (ordered walks only). In the batch
// schedule above a warp takes 32 rays and waits for the slowest of them:
// diffuse bounce rays differ several-fold in work, and most lanes idle while
// the last ray finishes. Here every lane keeps its own resumable traversal
// state (TLAS walk, instance, geometry, BLAS stack). Lanes walk their BLAS in
// the same speculative near-first loop as traverse_ray; a lane that finishes
// leaves the loop, and once at least `w.refill` lanes have left it the others
// pause at the end of their current round so that the warp can claim new queue
// entries for its idle lanes (one atomicAdd) and start them. Per ray the tests
// and their order are traverse_ray's, so every result equals the batch
// schedule's up to the order in which exact-distance ties are met. Iterations
// are capped far above any real traversal; a warp that reaches a cap sets bit
// 2 of the error word and stops.
constexpr uint32_t kMaxWarpIterations = 1u << 24;

template <int MODE, bool WT>
__global__ void __launch_bounds__(128, 8) secondary_dynamic_kernel(TraceParams p, WavefrontParams w) {
  extern __shared__ uint2 smem_stack[];
  constexpr int WIDTH = MODE == MODE_WIDE4 ? 4 : 2;
  const unsigned long long bins = *(volatile unsigned long long*)w.bins;
  const uint32_t n_front = (uint32_t)bins, n = n_front + (uint32_t)(bins >> 32);
  const uint32_t cap = w.width * w.height;
  const uint32_t total = 2u * n;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lanes_below = (1u << lane) - 1u;
  if (blockIdx.x == 0 && threadIdx.x == 0 && w.ray_counts) {
    w.ray_counts[0] = w.width * w.height;
    w.ray_counts[1] = n;
    w.ray_counts[2] = n;
  }
  uint2* stack = smem_stack + threadIdx.x;
  const uint32_t stride = blockDim.x;
  const uint32_t threshold = w.refill < 1u ? 1u : (w.refill > 32u ? 32u : w.refill);
  LaneWalk<WIDTH, WT> L;
  L.reset();
  uint32_t q = 0;
  bool exhausted = false;
  for (uint32_t iter = 0;; iter++) {
    if (iter >= (p.iteration_limit ? p.iteration_limit : kMaxWarpIterations)) {
      if (lane == 0) atomicOr(p.error_word, 4u);
      break;
    }
    // refill idle lanes from the queue
    const uint32_t idle = __ballot_sync(0xffffffffu, L.phase == WALK_IDLE);
    if (!exhausted && (__popc(idle) >= threshold || idle == 0xffffffffu)) {
      const uint32_t cnt = __popc(idle);
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(w.work_counter, cnt);
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + cnt >= total) exhausted = true;
      if (L.phase == WALK_IDLE) {
        const uint32_t j = base + __popc(idle & lanes_below);
        if (j < total) {
          q = j;  // bounce rays first, as in the batch schedule
          const bool shadow = j >= n;
          const float4* rq = reinterpret_cast<const float4*>(shadow ? w.shadow_rays : w.bounce_rays) +
                             2 * (size_t)(shadow ? j - n : bounce_entry(j, n_front, cap));
          L.start(p, rq[0], rq[1], w.tlas, shadow ? TF_END_SEARCH : 0u);
        }
      }
    }
    if (exhausted && __ballot_sync(0xffffffffu, L.phase != WALK_IDLE) == 0u) break;
    if (L.phase != WALK_IDLE) L.advance(p, stack, stride, threshold);
    if (L.phase == WALK_DONE) {
      const RayCtx& R = L.R;
      if (q >= n) {
        PixelResult* o = w.out + w.shadow_pixel[q - n];
        o->light = R.best.have ? 2u : 1u;
        if (R.best.have) o->direct = 0.0f;
      } else if (R.best.have) {
        PixelResult* o = w.out + w.bounce_pixel[bounce_entry(q, n_front, cap)];
        const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + R.best.geom_slot));
        o->bounce_prim = __ldg(p.redirect + R.best.k) - gm.z;
        o->bounce_t = R.best.t;
      }
      L.phase = WALK_IDLE;
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
  w.bins = reinterpret_cast<unsigned long long*>(s + 8);
  w.tile_counter = reinterpret_cast<uint32_t*>(s + 16);
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

namespace {
template <int MODE, bool LOCAL, int TIER, bool WT>
cudaError_t launch_wavefront_mode(const TraceParams& p, const WavefrontParams& w, uint32_t block, int sm_count,
                                  uint32_t phases, cudaStream_t stream) {
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done{0};
  cudaError_t e = raise_smem_limit(
      attr_done, {(const void*)primary_kernel<MODE, LOCAL, TIER, WT>, (const void*)secondary_kernel<MODE, LOCAL, TIER, WT>,
                  (const void*)secondary_dynamic_kernel<MODE == MODE_THREADED ? MODE_BINARY : MODE, WT>});
  if (e != cudaSuccess) return e;
  if (phases & 1u) {
    e = cudaMemsetAsync(w.queue_count, 0, 64, stream);
    if (e != cudaSuccess) return e;
    // persistent primary grid: as many resident blocks as fill every SM, or
    // fewer when the frame has fewer 4x8 tiles than resident warps
    int per_sm1 = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm1, primary_kernel<MODE, LOCAL, TIER, WT>, (int)block, smem);
    if (e != cudaSuccess) return e;
    if (per_sm1 < 1) per_sm1 = 1;
    const uint64_t tiles = (uint64_t)((w.width + 3) / 4) * ((w.height + 7) / 8);
    const uint64_t need = (tiles * 32 + block - 1) / block;
    const uint32_t grid1 = (uint32_t)std::min<uint64_t>((uint64_t)sm_count * per_sm1, need);
    primary_kernel<MODE, LOCAL, TIER, WT><<<grid1, block, smem, stream>>>(p, w);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (!(phases & 2u)) return cudaSuccess;
  e = cudaMemsetAsync(w.work_counter, 0, 64, stream);
  if (e != cudaSuccess) return e;
  // persistent secondary grid: enough resident blocks to fill every SM
  const bool dynamic = MODE != MODE_THREADED && w.refill != 0u && !LOCAL;
  int per_sm = 0;
  constexpr int DMODE = MODE == MODE_THREADED ? MODE_BINARY : MODE;  // the threaded walk has no dynamic form
  if (dynamic)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, secondary_dynamic_kernel<DMODE, WT>, (int)block, smem);
  else
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, secondary_kernel<MODE, LOCAL, TIER, WT>, (int)block, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const uint32_t grid2 = (uint32_t)(sm_count * per_sm);
  if (dynamic) secondary_dynamic_kernel<DMODE, WT><<<grid2, block, smem, stream>>>(p, w);
  else secondary_kernel<MODE, LOCAL, TIER, WT><<<grid2, block, smem, stream>>>(p, w);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_wavefront(const TraceParams& p, const WavefrontParams& w, int mode, uint32_t block,
                             int sm_count, uint32_t phases, cudaStream_t stream) {
  if (phases == 0) phases = 3;
  if (block == 0) block = 64;
  const size_t n = (size_t)w.width * w.height;
  if (n == 0) return cudaSuccess;
  // the local-memory stack holds kLocalStackEntries entries; deeper trees keep the shared-memory stack
  const bool local = w.local_stack && mode != MODE_THREADED && p.stack_depth <= kLocalStackEntries;
  // register tiers apply to the local-stack kernels
  const uint32_t tier = local ? w.register_tier : 0u;
#define RDN_WF(M, L, T)                                                                      \
  return p.watertight ? launch_wavefront_mode<M, L, T, true>(p, w, block, sm_count, phases, stream) \
                      : launch_wavefront_mode<M, L, T, false>(p, w, block, sm_count, phases, stream)
  if (mode == MODE_WIDE4) {
    if (!local) RDN_WF(MODE_WIDE4, false, 0);
    if (tier == 1) RDN_WF(MODE_WIDE4, true, 1);
    if (tier == 2) RDN_WF(MODE_WIDE4, true, 2);
    RDN_WF(MODE_WIDE4, true, 0);
  }
  if (mode == MODE_BINARY) {
    if (!local) RDN_WF(MODE_BINARY, false, 0);
    if (tier == 1) RDN_WF(MODE_BINARY, true, 1);
    if (tier == 2) RDN_WF(MODE_BINARY, true, 2);
    RDN_WF(MODE_BINARY, true, 0);
  }
  RDN_WF(MODE_THREADED, false, 0);
#undef RDN_WF
}

}  // namespace rdn
