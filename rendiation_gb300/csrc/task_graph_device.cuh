// Device-side primitives of the task graph (task_graph.cu), shared with task
// programs compiled outside librdn (include/rdn_task.cuh): the record layout,
// warp-aggregated bump counters, spawn / wake / cleanup / poll of a child, and
// the poll finalisation. See task_graph.h for the reference map.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "task_graph.h"

namespace rdn {
namespace task {

// Payload and local words are stored word-major (structure of arrays): word w
// of record i at [w * (cap + 1) + i]. Neighbouring lanes mostly hold
// neighbouring records (indices leave and return to the empty pool in warp
// order), so a warp's accesses to one word coalesce.
struct Rec {
  uint32_t* base;
  uint32_t stride;
  __device__ __forceinline__ uint32_t& operator[](uint32_t w) const { return base[(size_t)w * stride]; }
};
__device__ __forceinline__ Rec task_locals(const TaskGroupDev& T, uint32_t i) { return Rec{T.locals + i, T.cap + 1}; }
__device__ __forceinline__ Rec task_payload(const TaskGroupDev& T, uint32_t i) {
  return Rec{T.payload + i, T.cap + 1};
}

// Fetch-and-increment of a bump counter, aggregated over the converged lanes
// that name the same counter: one atomic per (warp, counter), each lane gets a
// distinct old value. Tens of thousands of tasks push to the same few counters
// in one launch; per-lane atomics on one address serialise.
__device__ __forceinline__ uint32_t agg_inc(uint32_t* ctr) {
  const uint32_t active = __activemask();
  const uint32_t peers = __match_any_sync(active, reinterpret_cast<unsigned long long>(ctr));
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(ctr, (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1u));
}

// DeviceBumpAllocationInvocationInstance::bump_allocate into the active list.
__device__ __forceinline__ void push_active(const TaskGraphDev& G, const TaskGroupDev& T, uint32_t idx) {
  GroupCtl* c = T.ctl;
  const uint32_t size = c->active.size;
  const uint32_t b = agg_inc(&c->active.bump);
  if (b < T.cap - size)
    T.active[c->sel][size + b] = idx;
  else
    atomicOr(G.error, TASK_ERR_ACTIVE_FULL);
}

// TaskGroupDeviceInvocationInstance::spawn_new_task_dyn: pop a free index,
// write the record (state, parent, initial future state), push the index to
// the active list. Returns TASK_HANDLE_UNINIT when the pool is empty. The
// caller writes the payload (task_payload) in the same launch: the pushed
// index is polled only after the next commit.
__device__ inline uint32_t spawn_task(const TaskGraphDev& G, uint32_t g, uint32_t parent_type, uint32_t parent_index) {
  const TaskGroupDev& T = G.g[g];
  GroupCtl* c = T.ctl;
  const uint32_t esize = c->empty.size;
  const uint32_t b = agg_inc(&c->empty.bump);
  if (b >= esize) {
    atomicOr(G.error, TASK_ERR_NO_FREE_SLOT);
    return TASK_HANDLE_UNINIT;
  }
  const uint32_t idx = T.empty[esize - b - 1];
  T.state[idx] = TASK_NOT_FINISHED_WAKEN;
  T.parent_index[idx] = parent_index;
  T.parent_type[idx] = parent_type;
  const Rec L = task_locals(T, idx);
  L[0] = 0u;
  for (uint32_t k = 0; k < kTaskMaxSpawns; k++) L[1 + k] = TASK_HANDLE_UNINIT;
  L[5] = TRACE_SUB_NOT_SPAWNED;
  L[6] = TRACE_SUB_NOT_SPAWNED;
  L[7] = 0u;
  push_active(G, T, idx);
  return idx;
}

// wake_task_dyn: a task still in the active list (GO_TO_SLEEP) is only
// re-flagged; a sleeping one is pushed again.
__device__ __forceinline__ void wake_task(const TaskGraphDev& G, uint32_t g, uint32_t idx) {
  const TaskGroupDev& T = G.g[g];
  const bool in_active = T.state[idx] == TASK_GO_TO_SLEEP;
  T.state[idx] = TASK_NOT_FINISHED_WAKEN;
  if (!in_active) push_active(G, T, idx);
}

// cleanup_finished_task_state_and_payload
__device__ __forceinline__ void cleanup_task(const TaskGraphDev& G, uint32_t g, uint32_t idx) {
  const TaskGroupDev& T = G.g[g];
  GroupCtl* c = T.ctl;
  const uint32_t size = c->removed.size;
  const uint32_t b = agg_inc(&c->removed.bump);
  if (b < T.cap - size)
    T.removed[size + b] = idx;
  else
    atomicOr(G.error, TASK_ERR_REMOVED_FULL);
  T.state[idx] = TASK_NOT_EXIST;
}

// poll_task_dyn: a finished child is cleaned up; its payload stays readable
// until the removed list is drained at the child group's next round.
__device__ __forceinline__ bool poll_child(const TaskGraphDev& G, uint32_t g, uint32_t idx) {
  if (G.g[g].state[idx] != TASK_FINISHED) return false;
  cleanup_task(G, g, idx);
  return true;
}

// Poll finalisation of the polling pipeline (task_group.rs:130-165).
__device__ __forceinline__ void finalize(const TaskGraphDev& G, uint32_t g, uint32_t idx, bool resolved, uint32_t pi,
                                         uint32_t pt) {
  const TaskGroupDev& T = G.g[g];
  if (!resolved) {
    T.state[idx] = TASK_GO_TO_SLEEP;
    return;
  }
  T.state[idx] = TASK_FINISHED;
  if (pi == TASK_NO_PARENT)
    cleanup_task(G, g, idx);
  else if (pt < G.n_groups)
    wake_task(G, pt, pi);
}

}  // namespace task
}  // namespace rdn
