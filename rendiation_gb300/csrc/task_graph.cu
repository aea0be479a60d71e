// Device task graph for sm_103a (see task_graph.h for the reference map).
//
// One execute round runs, for each group in order:
//   drain    commit the active / empty / removed bump counters and move the
//            removed indices to the end of the empty pool (prepare_execution)
//   poll     one thread per active task: run its program, then finish it
//            (wake the parent or clean up) or put it to sleep
//   compact  commit the active list and keep the tasks still
//            NOT_FINISHED_WAKEN, in order (GO_TO_SLEEP becomes SLEEP), in one
//            pass over 1024-entry tiles with decoupled look-back
// The compaction of group g and the drain of group g + 1 run in one launch
// (bookkeep_kernel), so a round of n groups takes 2n launches.
// The committed sizes live in a 64 B control block per group in device memory:
// no host round trip inside a round, and a sequence of rounds can be captured
// into a CUDA graph. The drain's last-block pattern (a ticket counter) lets the
// first blocks read the old sizes while only the last one writes the new ones.
// record_until_empty captures the rounds as the body of a WHILE conditional
// node that a one-warp check ends once no group has an active task.
// Programs: the built-in chain program runs in poll_chain_kernel, the trace
// program in poll_kernel; an external program's poll kernel (include/rdn_task.cuh) is launched by the
// callback registered for its group, at the same point of the round.
//
// Deviations from the reference, both at exhaustion only: a bump list or the
// empty pool that is full rejects the push or pop and sets an error bit,
// where the reference's bound check admits one access past the end
// (bump_allocator.rs:254-258, 296-300).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "ao.cuh"
#include "task_graph.h"
#include "task_graph_device.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;
using namespace task;

constexpr uint32_t kTile = 1024;
constexpr uint32_t kCompactThreads = 256;
constexpr uint32_t kPollThreads = 128;


__device__ __forceinline__ void put_ray(const Rec& b, float3 o, float tmin, float3 d, float tmax) {
  b[0] = __float_as_uint(o.x);
  b[1] = __float_as_uint(o.y);
  b[2] = __float_as_uint(o.z);
  b[3] = __float_as_uint(tmin);
  b[4] = __float_as_uint(d.x);
  b[5] = __float_as_uint(d.y);
  b[6] = __float_as_uint(d.z);
  b[7] = __float_as_uint(tmax);
}

// Payload of a chain's child (the closure of a .then stage), written to the
// child's record b of `words` words (validated: >= 16 for the AO operations).
__device__ void child_payload(uint32_t op, const Rec& self, const TraceParams& P, const AoEnv& A, const Rec& b,
                              uint32_t words) {
  uint32_t px, py;
  if (op == TASK_SPAWN_AO_PRIMARY && ao_pixel(A, self[0], px, py)) {
    float3 o, d;
    ao_camera_ray(A, px, py, o, d);
    put_ray(b, o, F32_EPSILON, d, F32_MAX);
    ao_count(A, 0, true);
    b[8] = RAY_FLAG_CULL_BACK;
    b[9] = 0xFFFFFFFFu;
    b[10] = A.tlas;
    b[11] = A.sbt_closest[0];
    b[12] = A.sbt_miss;
    b[13] = __float_as_uint(0.0f);
    for (uint32_t w = 14; w < words; w++) b[w] = 0u;
    return;
  }
  if (op == TASK_SPAWN_AO_PRIMARY || op == TASK_SPAWN_AO_OCCLUSION) {
    if (op == TASK_SPAWN_AO_PRIMARY || self[17] >= A.n_instances || self[16] >= A.n_triangles) {
      // past the frame, or not a closest-hit payload: an empty trace call
      // that resolves at once
      put_ray(b, make_float3(0.0f, 0.0f, 0.0f), 1.0f, make_float3(0.0f, 0.0f, 1.0f), 0.0f);
      b[8] = 0u;
      b[9] = 0u;
      b[10] = 0u;
      b[11] = b[12] = 0xFFFFFFFFu;
      b[13] = __float_as_uint(1.0f);
      for (uint32_t w = 14; w < words; w++) b[w] = 0u;
      return;
    }
    const float3 ro = make_float3(__uint_as_float(self[0]), __uint_as_float(self[1]), __uint_as_float(self[2]));
    const float3 rd = make_float3(__uint_as_float(self[4]), __uint_as_float(self[5]), __uint_as_float(self[6]));
    const float t = __uint_as_float(self[18]);
    const float3 hit = ro + rd * t;
    const float3 n = ao_shading_normal(A, P.tlas_data + self[17], self[16], __uint_as_float(self[19]),
                                       __uint_as_float(self[20]), ro, hit);
    const float3 dir = ao_direction(n, ao_sample(A));
    put_ray(b, hit, AO_TEST_MIN, dir, AO_TEST_MAX);
    ao_count(A, 1, true);
    b[8] = RAY_FLAG_END_SEARCH;
    b[9] = 0xFFFFFFFFu;
    b[10] = self[10];
    b[11] = A.sbt_closest[1];
    b[12] = A.sbt_miss;
    b[13] = __float_as_uint(1.0f);
    for (uint32_t w = 14; w < words; w++) b[w] = 0u;
    return;
  }
  for (uint32_t w = 0; w < words; w++) b[w] = 0u;
}

__device__ __forceinline__ void apply_map(uint32_t op, const Rec& self, const Rec& child, const AoEnv& A) {
  if (op == TASK_MAP_AO_ACCUMULATE) {
    uint32_t x, y;
    if (ao_pixel(A, self[0], x, y)) ao_accumulate(A, y * A.width + x, __uint_as_float(child[kTraceUser]));
  } else if (op == TASK_MAP_STORE_CHILD) {
    for (uint32_t w = 0; w < 3; w++) self[kTraceUser + w] = child[kTraceUser + w];
  } else if (op == TASK_MAP_STORE_ZERO) {
    self[kTraceUser] = __float_as_uint(0.0f);
  } else if (op == TASK_MAP_STORE_ONE) {
    self[kTraceUser] = __float_as_uint(1.0f);
  }
}

// BaseShaderFuture.then(spawn).then(spawn)...map: the base future resolves on
// its first poll only; a stage whose upstream resolved spawns its child and
// polls it at once; a stage resolves in the poll that reads its finished child.
__device__ bool poll_chain(const TaskGraphDev& G, uint32_t g, uint32_t idx, const TraceParams& P, const AoEnv& A) {
  const TaskGroupDev& T = G.g[g];
  const Rec L = task_locals(T, idx);
  const Rec self = task_payload(T, idx);
  const uint32_t n_spawn = T.n_spawn;
  // the future's words are independent loads: issue them together
  uint32_t l[1 + kTaskMaxSpawns];
#pragma unroll
  for (uint32_t k = 0; k <= kTaskMaxSpawns; k++) l[k] = k <= n_spawn ? L[k] : 0u;
  bool r = l[0] == 0u;
  if (r) L[0] = 1u;
  Rec child{nullptr, 0};
#pragma unroll
  for (uint32_t k = 0; k < kTaskMaxSpawns; k++) {
    if (k >= n_spawn) break;
    const uint32_t cg = T.spawn_type[k];
    if (r) {
      const uint32_t h = spawn_task(G, cg, g, idx);
      if (h != TASK_HANDLE_UNINIT) {
        const TaskGroupDev& C = G.g[cg];
        child_payload(T.spawn_op[k], self, P, A, task_payload(C, h), C.payload_words);
      }
      L[1 + k] = h;
      l[1 + k] = h;
    }
    r = false;
    const uint32_t h = l[1 + k];
    if (h != TASK_HANDLE_UNINIT && h != TASK_HANDLE_RESOLVED && poll_child(G, cg, h)) {
      child = task_payload(G.g[cg], h);
      L[1 + k] = TASK_HANDLE_RESOLVED;
      r = true;
    }
  }
  if (r) apply_map(T.map_op, self, child, A);
  return r;
}

// The ray-trace task (trace_task.rs:150-360): the first poll traverses and
// spawns the closest-hit or miss task of its trace call (resolving at once
// when there is none to spawn); the task resolves in the poll that finds that
// child finished, taking back the child's user payload.
template <int MODE, bool WT>
__device__ bool poll_trace(const TaskGraphDev& G, uint32_t g, uint32_t idx, const TraceParams& P, uint2* stack,
                           uint32_t stride) {
  const TaskGroupDev& T = G.g[g];
  const Rec L = task_locals(T, idx);
  const Rec self = task_payload(T, idx);
  uint32_t sub_group = L[5], sub_id = L[6], terminated = L[7];
  if (sub_id == TRACE_SUB_NOT_SPAWNED) {
    RayCtx R;
    R.o = make_float3(__uint_as_float(self[0]), __uint_as_float(self[1]), __uint_as_float(self[2]));
    R.tmin = __uint_as_float(self[3]);
    R.d = make_float3(__uint_as_float(self[4]), __uint_as_float(self[5]), __uint_as_float(self[6]));
    R.tmax = __uint_as_float(self[7]);
    R.ray_flags = self[8];
    R.cull_mask = self[9];
    bool bad;
    traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, self[10], stack, stride, bad);
    if (bad) atomicOr(P.error_word, 2u);
    uint32_t target = TRACE_SUB_NOT_SPAWNED;
    if (R.best.have) {
      if (!(R.ray_flags & RAY_FLAG_SKIP_CLOSEST) && self[11] < G.n_groups &&
          G.g[self[11]].payload_words >= kClosestWords)
        target = self[11];
    } else if (self[12] < G.n_groups && G.g[self[12]].payload_words >= kTraceCallWords) {
      target = self[12];
    }
    if (target != TRACE_SUB_NOT_SPAWNED) {
      const uint32_t h = spawn_task(G, target, g, idx);
      sub_group = target;
      sub_id = h == TASK_HANDLE_UNINIT ? TRACE_SUB_SPAWN_FAILED : h;
      L[5] = sub_group;
      L[6] = sub_id;
      if (h != TASK_HANDLE_UNINIT) {
        const TaskGroupDev& C = G.g[target];
        const Rec b = task_payload(C, h);
        for (uint32_t w = 0; w < kTraceCallWords; w++) b[w] = self[w];
        uint32_t w = kTraceCallWords;
        if (R.best.have) {
          const uint4 gm = __ldg(reinterpret_cast<const uint4*>(P.tri_root + R.best.geom_slot));
          const uint32_t tri = __ldg(P.redirect + R.best.k);
          b[16] = tri;
          b[17] = R.best.inst;
          b[18] = __float_as_uint(R.best.t);
          b[19] = __float_as_uint(R.best.u);
          b[20] = __float_as_uint(R.best.v);
          b[21] = R.best.s < 0.0f ? 0xFFu : 0xFEu;
          b[22] = gm.y;
          b[23] = tri - gm.z;
          w = kClosestWords;
        }
        for (; w < C.payload_words; w++) b[w] = 0u;
      }
    }
  }
  bool resolved = false;
  if (sub_id == TRACE_SUB_SPAWN_FAILED || sub_id == TRACE_SUB_NOT_SPAWNED) {
    if (!terminated) {
      L[7] = 1u;
      terminated = 1u;
      resolved = true;
    }
  }
  if (!terminated) {
    if (poll_child(G, sub_group, sub_id)) {
      const Rec cp = task_payload(G.g[sub_group], sub_id);
      const uint32_t u0 = cp[kTraceUser], u1 = cp[kTraceUser + 1], u2 = cp[kTraceUser + 2];
      self[kTraceUser] = u0;
      self[kTraceUser + 1] = u1;
      self[kTraceUser + 2] = u2;
      L[7] = 1u;
      resolved = true;
    }
  }
  return resolved;
}

// One thread per active entry of group g: poll(idx) runs the task's program,
// then the poll is finalised.
template <class Poll>
__device__ __forceinline__ void poll_active(const TaskGraphDev& G, uint32_t g, const Poll& poll) {
  const TaskGroupDev& T = G.g[g];
  const GroupCtl* c = T.ctl;
  const uint32_t n = c->active.size;
  const uint32_t* list = T.active[c->sel];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t idx = list[i];
    // the parent is read now, and its state line fetched into L2, so that a
    // resolving task does not wait for them at the end
    const uint32_t pi = T.parent_index[idx], pt = T.parent_type[idx];
    if (pi != TASK_NO_PARENT && pt < G.n_groups)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(G.g[pt].state + pi));
    finalize(G, g, idx, poll(idx), pi, pt);
  }
}

// Trace polls: persistent warps take 32 consecutive active entries at a time
// from the group's poll counter, so a warp whose rays end early takes more and
// the grid is sized by residency, not by the pool's capacity.
template <class Poll>
__device__ __forceinline__ void poll_active_fetch(const TaskGraphDev& G, uint32_t g, const Poll& poll) {
  const TaskGroupDev& T = G.g[g];
  GroupCtl* c = T.ctl;
  const uint32_t n = c->active.size;
  const uint32_t* list = T.active[c->sel];
  const uint32_t lane = threadIdx.x & 31u;
  for (;;) {
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(&c->poll_next, 32u);
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (base >= n) break;
    const uint32_t i = base + lane;
    if (i < n) {
      const uint32_t idx = list[i];
      const uint32_t pi = T.parent_index[idx], pt = T.parent_type[idx];
      if (pi != TASK_NO_PARENT && pt < G.n_groups)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(G.g[pt].state + pi));
      finalize(G, g, idx, poll(idx), pi, pt);
    }
  }
}

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(kPollThreads, 8) poll_kernel(const TaskGraphDev* __restrict__ Gp, uint32_t g,
                                                            TraceParams P, AoEnv) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const TaskGraphDev& G = *Gp;
  poll_active_fetch(G, g,
                    [&](uint32_t idx) { return poll_trace<MODE, WT>(G, g, idx, P, stack_ptr, stack_stride); });
}

// Chain groups alone: without the traversal the kernel fits twice the resident
// warps of poll_kernel, and its polls are chains of dependent loads that more
// warps hide.
__global__ void __launch_bounds__(kPollThreads, 8) poll_chain_kernel(const TaskGraphDev* __restrict__ Gp, uint32_t g,
                                                                    TraceParams P, AoEnv A) {
  const TaskGraphDev& G = *Gp;
  poll_active(G, g, [&](uint32_t idx) { return poll_chain(G, g, idx, P, A); });
}

__device__ __forceinline__ uint32_t commit_alloc(uint32_t size, uint32_t bump, uint32_t cap) {
  return bump > cap - size ? cap : size + bump;
}
__device__ __forceinline__ uint32_t commit_dealloc(uint32_t size, uint32_t bump) {
  return bump > size ? 0u : size - bump;
}

// prepare_execution of group T, one of nb blocks: commit the three bump lists,
// drain removed -> empty; the last block writes the committed sizes and opens
// the group's next compaction (tile counter 0, next epoch).
__device__ __forceinline__ void drain_part(const TaskGroupDev& T, uint32_t b, uint32_t nb, uint32_t* ticket) {
  GroupCtl* c = T.ctl;
  __shared__ uint32_t s_removed, s_empty, s_last;
  if (threadIdx.x == 0) {
    s_removed = commit_alloc(c->removed.size, c->removed.bump, T.cap);
    s_empty = commit_dealloc(c->empty.size, c->empty.bump);
  }
  __syncthreads();
  const uint32_t n = s_removed, off = s_empty;
  for (uint32_t i = b * blockDim.x + threadIdx.x; i < n; i += nb * blockDim.x)
    if (off + i < T.cap) T.empty[off + i] = T.removed[i];
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == nb - 1;
  __syncthreads();
  if (s_last && threadIdx.x == 0) {
    __threadfence();
    c->active.size = commit_alloc(c->active.size, c->active.bump, T.cap);
    c->active.bump = 0u;
    c->empty.size = min(T.cap, off + n);
    c->empty.bump = 0u;
    c->removed.size = 0u;
    c->removed.bump = 0u;
    c->drain_n = n;
    c->drain_off = off;
    c->tile_next = 0u;
    c->poll_next = 0u;
    c->epoch = c->epoch + 1u;
    *ticket = 0u;
  }
}

// dispatch_allocate_init_task's commits (active: allocate, empty: deallocate).
__global__ void commit_spawn_kernel(TaskGroupDev T) {
  GroupCtl* c = T.ctl;
  c->active.size = commit_alloc(c->active.size, c->active.bump, T.cap);
  c->active.bump = 0u;
  c->empty.size = commit_dealloc(c->empty.size, c->empty.bump);
  c->empty.bump = 0u;
}

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* warp_sums) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
  if (lane == 0) warp_sums[warp] = v;
  __syncthreads();
  uint32_t t = 0;
  for (uint32_t w = 0; w < blockDim.x / 32; w++) t += warp_sums[w];
  __syncthreads();
  return t;
}

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

constexpr unsigned long long kTileAggregate = 1ull, kTileInclusive = 2ull;
constexpr uint32_t kLookbackLimit = 1u << 22;  // predecessor polls before a tile gives up

// One 1024-entry tile of the compaction (see compact_part).
__device__ __forceinline__ void compact_tile(const TaskGroupDev& T, GroupCtl* c, uint32_t tile, uint32_t n,
                                             uint32_t used, uint32_t sel, uint32_t* err, uint32_t& s_excl,
                                             uint32_t* warp_sums) {
  const uint32_t s_epoch = c->epoch & 0x3FFFFFFFu;
  const uint32_t* list = T.active[sel];
  const uint32_t base = tile * kTile;
  constexpr uint32_t kPer = kTile / kCompactThreads;
  uint32_t idx[kPer];
  bool keep[kPer];
  uint32_t kept = 0;
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++) {
    const uint32_t i = base + j * kCompactThreads + threadIdx.x;
    idx[j] = 0u;
    keep[j] = false;
    if (i < n) {
      idx[j] = list[i];
      const uint32_t st = T.state[idx[j]];
      if (st == TASK_GO_TO_SLEEP) T.state[idx[j]] = TASK_NOT_FINISHED_SLEEP;
      keep[j] = st == TASK_NOT_FINISHED_WAKEN;
    }
    kept += keep[j];
  }
  const uint32_t total = block_sum(kept, warp_sums);
  if (threadIdx.x < 32) {
    // warp 0: publish the tile's count, then look back 32 descriptors at a
    // time (lane l reads tile p - l) until the nearest inclusive prefix
    const uint32_t lane = threadIdx.x;
    const unsigned long long ep = (unsigned long long)s_epoch << 34;
    uint32_t excl = 0;
    if (tile == 0) {
      if (lane == 0) st_release(T.tile_desc, ep | (kTileInclusive << 32) | total);
    } else {
      if (lane == 0) st_release(T.tile_desc + tile, ep | (kTileAggregate << 32) | total);
      int p = (int)tile - 1;
      uint32_t polls = 0;
      while (p >= 0) {
        const int q = p - (int)lane;
        bool ready = true, incl = true;
        uint32_t val = 0;
        if (q >= 0) {
          const unsigned long long v = ld_acquire(T.tile_desc + q);
          const unsigned long long status = (v >> 32) & 3ull;
          ready = (uint32_t)(v >> 34) == s_epoch && status != 0ull;
          incl = status == kTileInclusive;
          val = (uint32_t)v;
        }
        if (!__all_sync(0xFFFFFFFFu, ready)) {
          if (++polls > kLookbackLimit) {  // uniform across the warp
            if (lane == 0) atomicOr(err, TASK_ERR_LOOKBACK);
            break;
          }
          continue;
        }
        const uint32_t incl_mask = __ballot_sync(0xFFFFFFFFu, incl);
        // lanes up to the nearest inclusive descriptor (the lowest such lane) contribute
        const uint32_t stop = incl_mask ? (uint32_t)(__ffs(incl_mask) - 1) : 31u;
        uint32_t part = lane <= stop ? val : 0u;
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
        excl += part;
        if (incl_mask) break;
        p -= 32;
      }
      if (lane == 0) st_release(T.tile_desc + tile, ep | (kTileInclusive << 32) | (excl + total));
    }
    if (lane == 0) s_excl = excl;
  }
  __syncthreads();
  uint32_t* dst = T.active[sel ^ 1u];
  uint32_t offset = s_excl;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++) {
    const uint32_t ballot = __ballot_sync(0xFFFFFFFFu, keep[j]);
    if (lane == 0) warp_sums[warp] = __popc(ballot);
    __syncthreads();
    uint32_t before = offset;
    for (uint32_t w = 0; w < warp; w++) before += warp_sums[w];
    if (keep[j]) dst[before + __popc(ballot & ((1u << lane) - 1u))] = idx[j];
    uint32_t round = 0;
    for (uint32_t w = 0; w < kCompactThreads / 32; w++) round += warp_sums[w];
    __syncthreads();
    offset += round;
  }
  if (threadIdx.x == 0 && tile == (used ? used - 1u : 0u)) {
    c->compact_n = n;
    c->src_sel = sel;
    c->sel = sel ^ 1u;
    c->active.size = used ? s_excl + total : 0u;
    c->active.bump = 0u;
  }
}

// Commit of the active list and its compaction (ActiveTaskCompact) in one
// pass: each block takes the next 1024-entry tile, keeps the tasks still
// NOT_FINISHED_WAKEN (GO_TO_SLEEP becomes SLEEP), publishes its count and
// finds its offset by looking back over the descriptors of the tiles before
// it (decoupled look-back, Merrill and Garland 2016), then writes its kept
// indices, in order, to the other active buffer. Tiles are handed out in
// block arrival order, so every tile a block waits for belongs to a block
// that is already running. The block of the last tile writes the new size.
__device__ __forceinline__ void compact_part(const TaskGroupDev& T, uint32_t* err) {
  GroupCtl* c = T.ctl;
  __shared__ uint32_t s_tile, s_n, s_sel, s_epoch, s_excl, warp_sums[kCompactThreads / 32];
  if (threadIdx.x == 0) {
    s_n = commit_alloc(c->active.size, c->active.bump, T.cap);
    s_sel = c->sel;
    s_epoch = c->epoch & 0x3FFFFFFFu;
  }
  __syncthreads();
  const uint32_t n = s_n, sel = s_sel;
  const uint32_t used = (n + kTile - 1) / kTile;
  // a block arriving after the last tile's block finished reads a size no
  // larger than the one the tiles were cut from, and takes no tile
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(&c->tile_next, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    __syncthreads();
    if (tile >= (used ? used : 1u)) return;
    compact_tile(T, c, tile, n, used, sel, err, s_excl, warp_sums);
  }
}

// Bookkeeping between two polls, one launch: blocks [0, nc) compact group Tc
// after its poll, blocks [nc, nc + nd) drain group Td before its poll. The two
// groups' lists are disjoint, so the reference's order (compact g, then
// prepare g + 1) holds. nc = 0 or nd = 0 runs one part alone.
__global__ void __launch_bounds__(kCompactThreads) bookkeep_kernel(TaskGroupDev Tc, uint32_t nc, TaskGroupDev Td,
                                                                   uint32_t nd, uint32_t* ticket, uint32_t* err) {
  if (blockIdx.x < nc) compact_part(Tc, err);
  else drain_part(Td, blockIdx.x - nc, nd, ticket);
}

// TaskGroupExecutorResource::init: empty pool = 1..cap, fallback task 0.
__global__ void init_kernel(TaskGroupDev T) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < T.cap; i += gridDim.x * blockDim.x)
    T.empty[i] = i + 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    GroupCtl* c = T.ctl;
    c->empty.size = T.cap;
    T.state[0] = TASK_NOT_FINISHED_WAKEN;
    T.parent_index[0] = TASK_NO_PARENT;
    T.parent_type[0] = TASK_NO_PARENT;
    const Rec L = task_locals(T, 0);
    for (uint32_t k = 0; k < kTaskMaxSpawns; k++) L[1 + k] = TASK_HANDLE_UNINIT;
    L[5] = L[6] = TRACE_SUB_NOT_SPAWNED;
  }
}

__global__ void spawn_init_kernel(const TaskGraphDev* __restrict__ Gp, uint32_t g, uint32_t count,
                                  uint32_t init_op) {
  const TaskGraphDev& G = *Gp;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const uint32_t h = spawn_task(G, g, TASK_NO_PARENT, TASK_NO_PARENT);
    if (h != TASK_HANDLE_UNINIT) {
      const TaskGroupDev& T = G.g[g];
      const Rec b = task_payload(T, h);
      b[0] = init_op == TASK_INIT_INDEX ? i : 0u;
      for (uint32_t w = 1; w < T.payload_words; w++) b[w] = 0u;
    }
  }
}

// Drain loop of a captured graph (a WHILE conditional node): the round counter
// is reset before the loop; after each round one warp looks for an active
// entry in any group (committed or pushed since), and the loop ends when there
// is none or after max_rounds rounds. Without an active task no later round
// can change anything: only a polled task spawns or wakes another, so the
// graph is then either empty or holds tasks that wait for children whose
// spawn failed (RDN_TASK_ERROR_NO_FREE_SLOT).
__global__ void loop_reset_kernel(uint32_t* rounds) { *rounds = 0u; }

__global__ void loop_check_kernel(const TaskGraphDev* __restrict__ G, uint32_t* rounds, uint32_t max_rounds,
                                  cudaGraphConditionalHandle handle) {
  bool busy = false;
  for (uint32_t g = threadIdx.x; g < G->n_groups; g += 32) {
    const GroupCtl* c = G->g[g].ctl;
    busy |= c->active.size + c->active.bump != 0u;
  }
  busy = __any_sync(0xFFFFFFFFu, busy);
  if (threadIdx.x == 0) {
    const uint32_t r = *rounds + 1u;
    *rounds = r;
    cudaGraphSetConditional(handle, busy && r < max_rounds ? 1u : 0u);
  }
}

uint32_t tiles_of(uint32_t cap) { return (cap + kTile - 1) / kTile; }

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_poll_wt(const TaskGraphDev* G, uint32_t g, const TraceParams& P, const AoEnv& A, uint32_t grid,
                           cudaStream_t st) {
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)P.stack_depth * kPollThreads * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t e = raise_smem_limit(attr_done, {(const void*)poll_kernel<MODE, LOCAL, WT>});
  if (e != cudaSuccess) return e;
  poll_kernel<MODE, LOCAL, WT><<<grid, kPollThreads, smem, st>>>(G, g, P, A);
  return cudaGetLastError();
}

template <int MODE, bool LOCAL>
cudaError_t launch_poll(const TaskGraphDev* G, uint32_t g, const TraceParams& P, const AoEnv& A, uint32_t grid,
                        cudaStream_t st) {
  return P.watertight ? launch_poll_wt<MODE, LOCAL, true>(G, g, P, A, grid, st)
                      : launch_poll_wt<MODE, LOCAL, false>(G, g, P, A, grid, st);
}

bool op_reads_trace_payload(uint32_t op) {
  return op == TASK_MAP_AO_ACCUMULATE || op == TASK_MAP_STORE_CHILD;
}

}  // namespace

TaskGraph::~TaskGraph() {
  for (void* p : allocs_) cudaFree(p);
}

std::string TaskGraph::validate(const std::vector<TaskGroupDesc>& groups, uint32_t capacity) {
  const uint32_t n = (uint32_t)groups.size();
  if (n == 0 || n > kTaskMaxGroups) return "a task graph holds 1 to 16 task groups";
  if (capacity == 0) return "capacity must be at least 1";
  for (uint32_t g = 0; g < n; g++) {
    const TaskGroupDesc& d = groups[g];
    if (d.program > TASK_PROGRAM_EXTERNAL) return "unknown task program";
    if (d.program == TASK_PROGRAM_EXTERNAL && (d.n_spawn != 0 || d.map_op != TASK_MAP_NONE))
      return "an external program spawns and maps in its own poll kernel: n_spawn 0, map_op NONE";
    if (d.max_in_flight == 0) return "max_in_flight must be at least 1";
    if ((uint64_t)d.max_in_flight * capacity >= (1ull << 28)) return "max_in_flight * capacity too large";
    if (d.payload_words == 0 || d.payload_words > kTaskMaxPayloadWords) return "payload_words must be 1..32";
    if (d.program == TASK_PROGRAM_TRACE && d.payload_words < kTraceCallWords)
      return "a trace task needs a payload of at least 16 words";
    if (d.n_spawn > kTaskMaxSpawns) return "a chain has at most 4 spawn stages";
    if (d.map_op > TASK_MAP_STORE_ONE) return "unknown map operation";
    const uint32_t* last_child = nullptr;
    for (uint32_t k = 0; k < d.n_spawn; k++) {
      if (d.spawn_type[k] >= n) return "spawn stage names a task group that does not exist";
      if (d.spawn_op[k] > TASK_SPAWN_AO_OCCLUSION) return "unknown spawn payload operation";
      const TaskGroupDesc& cd = groups[d.spawn_type[k]];
      if (d.spawn_op[k] != TASK_SPAWN_ZERO && cd.program != TASK_PROGRAM_TRACE)
        return "a trace-call payload must go to a trace task group";
      if (d.spawn_op[k] == TASK_SPAWN_AO_OCCLUSION && d.payload_words < kClosestWords)
        return "the occlusion-ray stage reads a closest-hit payload of 24 words";
      last_child = &d.spawn_type[k];
    }
    if (op_reads_trace_payload(d.map_op)) {
      if (!last_child || groups[*last_child].payload_words < kTraceCallWords)
        return "the map operation reads the user payload of a trace-call child";
    }
    if ((d.map_op == TASK_MAP_STORE_CHILD || d.map_op == TASK_MAP_STORE_ZERO || d.map_op == TASK_MAP_STORE_ONE) &&
        d.payload_words < kTraceCallWords)
      return "the map operation writes a trace-call user payload (16 words)";
  }
  return "";
}

std::string TaskGraph::create(const std::vector<TaskGroupDesc>& groups, uint32_t capacity, int sm_count,
                              cudaStream_t st) {
  const std::string bad = validate(groups, capacity);
  if (!bad.empty()) return bad;
  const uint32_t n = (uint32_t)groups.size();
  desc_ = groups;
  ext_fn_.assign(n, nullptr);
  ext_user_.assign(n, nullptr);
  sm_count_ = sm_count > 0 ? sm_count : 1;
  std::memset(&dev_, 0, sizeof(dev_));
  dev_.n_groups = n;
  // control blocks + error word + per-group tickets (2 per group)
  void* ctl = nullptr;
  cudaError_t e = cudaMalloc(&ctl, sizeof(GroupCtl) * n + 256);
  if (e != cudaSuccess) return std::string("cudaMalloc: ") + cudaGetErrorString(e);
  allocs_.push_back(ctl);
  e = cudaMemsetAsync(ctl, 0, sizeof(GroupCtl) * n + 256, st);
  if (e != cudaSuccess) return std::string("cudaMemsetAsync: ") + cudaGetErrorString(e);
  GroupCtl* ctls = static_cast<GroupCtl*>(ctl);
  dev_.error = reinterpret_cast<uint32_t*>(ctls + n);
  for (uint32_t g = 0; g < n; g++) {
    const TaskGroupDesc& d = groups[g];
    TaskGroupDev& T = dev_.g[g];
    T.cap = d.max_in_flight * capacity;
    T.payload_words = d.payload_words;
    T.program = d.program;
    T.n_spawn = d.n_spawn;
    T.map_op = d.map_op;
    for (uint32_t k = 0; k < kTaskMaxSpawns; k++) {
      T.spawn_type[k] = d.spawn_type[k];
      T.spawn_op[k] = d.spawn_op[k];
    }
    const size_t rec = (size_t)T.cap + 1;
    const size_t words = rec * 3 + rec * d.payload_words + rec * kTaskLocalWords + (size_t)T.cap * 4 +
                         2 * (size_t)tiles_of(T.cap) + 66;
    void* mem = nullptr;
    e = cudaMalloc(&mem, words * 4);
    if (e != cudaSuccess) return std::string("cudaMalloc: ") + cudaGetErrorString(e);
    allocs_.push_back(mem);
    e = cudaMemsetAsync(mem, 0, words * 4, st);
    if (e != cudaSuccess) return std::string("cudaMemsetAsync: ") + cudaGetErrorString(e);
    uint32_t* w = static_cast<uint32_t*>(mem);
    T.state = w;
    w += rec;
    T.parent_type = w;
    w += rec;
    T.parent_index = w;
    w += rec;
    T.payload = w;
    w += rec * d.payload_words;
    T.locals = w;
    w += rec * kTaskLocalWords;
    T.active[0] = w;
    w += T.cap;
    T.active[1] = w;
    w += T.cap;
    T.removed = w;
    w += T.cap;
    T.empty = w;
    w += T.cap;
    w += (reinterpret_cast<uintptr_t>(w) & 7u) ? 1 : 0;  // 8-byte aligned tile descriptors
    T.tile_desc = reinterpret_cast<unsigned long long*>(w);
    T.ctl = ctls + g;
    const uint32_t grid = std::min<uint32_t>((T.cap + 255) / 256, (uint32_t)sm_count_ * 8);
    init_kernel<<<grid, 256, 0, st>>>(T);
    e = cudaGetLastError();
    if (e != cudaSuccess) return std::string("init launch: ") + cudaGetErrorString(e);
  }
  // the kernels read the group table from device memory (indexed by group at
  // run time, which kernel parameters do not support without a local copy)
  void* table = nullptr;
  e = cudaMalloc(&table, sizeof(TaskGraphDev));
  if (e != cudaSuccess) return std::string("cudaMalloc: ") + cudaGetErrorString(e);
  allocs_.push_back(table);
  dev_ptr_ = static_cast<TaskGraphDev*>(table);
  e = cudaMemcpyAsync(dev_ptr_, &dev_, sizeof(TaskGraphDev), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e);
  return "";
}

// compact group gc (kNone: no compaction) and drain group gd (kNone: none) in one launch
cudaError_t TaskGraph::bookkeep(uint32_t gc, uint32_t gd, cudaStream_t st) {
  constexpr uint32_t kNone = 0xFFFFFFFFu;
  // persistent blocks: the compaction's take tiles in turn, the drain's stride over the removed list
  const uint32_t nc = gc == kNone ? 0u : std::min<uint32_t>(tiles_of(dev_.g[gc].cap), (uint32_t)sm_count_ * 8);
  uint32_t nd = 0;
  if (gd != kNone)
    nd = std::max<uint32_t>(1, std::min<uint32_t>((dev_.g[gd].cap + 255) / 256, (uint32_t)sm_count_));
  if (nc + nd == 0) return cudaSuccess;
  const TaskGroupDev& Tc = dev_.g[gc == kNone ? 0u : gc];
  const TaskGroupDev& Td = dev_.g[gd == kNone ? 0u : gd];
  bookkeep_kernel<<<nc + nd, kCompactThreads, 0, st>>>(Tc, nc, Td, nd, dev_.error + 2 + 2 * (gd == kNone ? 0u : gd),
                                                       dev_.error);
  return cudaGetLastError();
}

cudaError_t TaskGraph::prepare(uint32_t g, cudaStream_t st) { return bookkeep(0xFFFFFFFFu, g, st); }

cudaError_t TaskGraph::compact(uint32_t g, cudaStream_t st) { return bookkeep(g, 0xFFFFFFFFu, st); }

cudaError_t TaskGraph::poll(uint32_t g, const TraceParams* p, int mode, const AoEnv* ao, cudaStream_t st) {
  const TaskGroupDev& T = dev_.g[g];
  // chain polls: one thread per possible active entry (blocks past the
  // committed size exit at once; their polls are chains of dependent loads
  // that want every task's loads in flight); trace polls: persistent warps
  // that fetch entries, so that divergent rays do not hold a block's slot
  const uint32_t cap_blocks = std::max<uint32_t>(1, (T.cap + kPollThreads - 1) / kPollThreads);
  const uint32_t grid = cap_blocks;
  TraceParams P;
  AoEnv A;
  if (p)
    P = *p;
  else
    std::memset(&P, 0, sizeof(P));
  if (ao)
    A = *ao;
  else
    std::memset(&A, 0, sizeof(A));
  const TaskGraphDev* G = dev_ptr_;
  if (T.program == TASK_PROGRAM_EXTERNAL) {
    if (!ext_fn_[g]) return cudaErrorInvalidValue;
    return ext_fn_[g](G, g, T.cap, st, ext_user_[g]) == 0 ? cudaGetLastError() : cudaErrorLaunchFailure;
  }
  if (T.program == TASK_PROGRAM_CHAIN) {
    poll_chain_kernel<<<grid, kPollThreads, 0, st>>>(G, g, P, A);
    return cudaGetLastError();
  }
  // the trace poll's launch bounds guarantee 8 resident blocks per SM
  const uint32_t tgrid = std::min<uint32_t>(cap_blocks, (uint32_t)sm_count_ * 8);
  if (!p) return launch_poll<MODE_THREADED, false>(G, g, P, A, tgrid, st);
  if (mode == MODE_WIDE4)
    return P.local_stack ? launch_poll<MODE_WIDE4, true>(G, g, P, A, tgrid, st)
                         : launch_poll<MODE_WIDE4, false>(G, g, P, A, tgrid, st);
  if (mode == MODE_BINARY)
    return P.local_stack ? launch_poll<MODE_BINARY, true>(G, g, P, A, tgrid, st)
                         : launch_poll<MODE_BINARY, false>(G, g, P, A, tgrid, st);
  return launch_poll<MODE_THREADED, false>(G, g, P, A, tgrid, st);
}

cudaError_t TaskGraph::dispatch_init(uint32_t group, uint32_t count, uint32_t init_op, cudaStream_t st) {
  cudaError_t e = prepare(group, st);
  if (e != cudaSuccess || count == 0) return e;
  const uint32_t grid = std::min<uint32_t>((count + 255) / 256, (uint32_t)sm_count_ * 8);
  spawn_init_kernel<<<grid, 256, 0, st>>>(dev_ptr_, group, count, init_op);
  commit_spawn_kernel<<<1, 1, 0, st>>>(dev_.g[group]);
  return cudaGetLastError();
}

// A round is, for each group in order, prepare (drain), poll, compact. The
// compaction of group g and the drain of group g + 1 touch disjoint lists and
// share one launch, so a round of n groups takes 2n launches.
cudaError_t TaskGraph::execute(uint32_t rounds, const TraceParams* p, int mode, const AoEnv* ao, cudaStream_t st) {
  const uint32_t n = dev_.n_groups;
  for (uint32_t r = 0; r < rounds; r++) {
    cudaError_t e = prepare(0, st);
    for (uint32_t g = 0; g < n && e == cudaSuccess; g++) {
      e = poll(g, p, mode, ao, st);
      if (e == cudaSuccess) e = bookkeep(g, g + 1 < n ? g + 1 : 0xFFFFFFFFu, st);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t TaskGraph::states(uint32_t* wake, uint32_t* empty, cudaStream_t st) {
  for (uint32_t g = 0; g < dev_.n_groups; g++) {
    cudaError_t e = prepare(g, st);
    if (e == cudaSuccess) e = compact(g, st);
    if (e != cudaSuccess) return e;
  }
  std::vector<GroupCtl> h(dev_.n_groups);
  cudaError_t e =
      cudaMemcpyAsync(h.data(), dev_.g[0].ctl, sizeof(GroupCtl) * dev_.n_groups, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  for (uint32_t g = 0; g < dev_.n_groups; g++) {
    wake[g] = h[g].active.size;
    empty[g] = h[g].empty.size;
  }
  return cudaSuccess;
}

cudaError_t TaskGraph::debug(uint32_t group, std::vector<uint32_t>& active, std::vector<uint32_t>& empty,
                             std::vector<uint32_t>& task_states, cudaStream_t st) {
  for (uint32_t g = 0; g < dev_.n_groups; g++) {
    cudaError_t e = prepare(g, st);
    if (e == cudaSuccess) e = compact(g, st);
    if (e != cudaSuccess) return e;
  }
  const TaskGroupDev& T = dev_.g[group];
  GroupCtl h;
  cudaError_t e = cudaMemcpyAsync(&h, T.ctl, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  active.assign(h.active.size, 0);
  empty.assign(h.empty.size, 0);
  task_states.assign((size_t)T.cap + 1, 0);
  if (h.active.size)
    e = cudaMemcpyAsync(active.data(), T.active[h.sel], 4 * (size_t)h.active.size, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && h.empty.size)
    e = cudaMemcpyAsync(empty.data(), T.empty, 4 * (size_t)h.empty.size, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(task_states.data(), T.state, 4 * ((size_t)T.cap + 1), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

cudaError_t TaskGraph::record_until_empty(uint32_t max_rounds, const TraceParams* p, int mode, const AoEnv* ao,
                                          cudaStream_t cap) {
  uint32_t* rounds = dev_.error + 40;
  loop_reset_kernel<<<1, 1, 0, cap>>>(rounds);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  cudaStreamCaptureStatus status;
  cudaGraph_t graph = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t n_deps = 0;
  e = cudaStreamGetCaptureInfo(cap, &status, nullptr, &graph, &deps, nullptr, &n_deps);
  if (e != cudaSuccess) return e;
  if (status != cudaStreamCaptureStatusActive) return cudaErrorStreamCaptureImplicit;
  cudaGraphConditionalHandle handle;
  e = cudaGraphConditionalHandleCreate(&handle, graph, 1u, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return e;
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};  // the remaining members zero
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  e = cudaGraphAddNode(&node, graph, deps, nullptr, n_deps, &cp);
  if (e != cudaSuccess) return e;
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  e = cudaStreamUpdateCaptureDependencies(cap, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
  if (e != cudaSuccess) return e;
  cudaStream_t bs = nullptr;
  e = cudaStreamCreateWithFlags(&bs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return e;
  e = cudaStreamBeginCaptureToGraph(bs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t rec = execute(1, p, mode, ao, bs);
    if (rec == cudaSuccess) {
      loop_check_kernel<<<1, 32, 0, bs>>>(dev_ptr_, rounds, max_rounds, handle);
      rec = cudaGetLastError();
    }
    e = cudaStreamEndCapture(bs, &body);
    if (rec != cudaSuccess) e = rec;
  }
  cudaStreamDestroy(bs);
  return e;
}

std::string TaskGraph::check_external() const {
  for (uint32_t g = 0; g < dev_.n_groups; g++)
    if (desc_[g].program == TASK_PROGRAM_EXTERNAL && !ext_fn_[g])
      return "task group " + std::to_string(g) + " runs an external program: register its poll with rdn_task_graph_set_poll";
  return "";
}

cudaError_t TaskGraph::read_error(uint32_t* flags, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(flags, dev_.error, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

}  // namespace rdn
