/*
 * rdn_task.cuh — task programs of your own for librdn's device task graph.
 *
 * The reference's tasks are shader futures (shader/task-graph/src/future/*.rs)
 * that its EDSL compiles into the polling pipeline of each task group
 * (runtime/task_group.rs:56-170). Here such a future is CUDA C++: a task group
 * created with RDN_TASK_PROGRAM_EXTERNAL is polled by a kernel compiled in your
 * own translation unit from this header, with the same record layout, spawn /
 * wake / cleanup rules and poll finalisation as librdn's built-in programs.
 *
 *   struct MyTask {
 *     struct Params { ... };                        // passed by value to every poll
 *     __device__ static bool poll(const rdn_task::Ctx& t, const Params& p);
 *   };                                              // true = resolved
 *   extern "C" rdn_status my_poll(const void* g, uint32_t group, uint32_t cap, void* s, void* user) {
 *     return rdn_task::launch<MyTask>(g, group, cap, s, MyTask::Params{...});
 *   }
 *   rdn_task_graph_set_poll(graph, group, my_poll, user);
 *
 * A poll runs once per round for every active task of the group. It reads and
 * writes the task's payload words and its 8 local words (the future's state;
 * at spawn: word 0 = 0, words 1..4 = RDN_TASK_HANDLE_UNINIT, 5..6 = 0xFFFFFFFF,
 * 7 = 0), spawns children (with the task as parent; a child that resolves
 * wakes it), and polls a child, which cleans the child up when it has
 * finished. Returning true finishes the task: its parent is woken, or a root
 * task is cleaned up. Build with nvcc, -I include -I rendiation_gb300/csrc.
 */
#ifndef RDN_TASK_CUH
#define RDN_TASK_CUH

#include <cuda_runtime.h>

#include <cstdint>

#include "rdn.h"
#include "task_graph_device.cuh"

#define RDN_TASK_HANDLE_UNINIT 0xFFFFFFFEu   /* a spawn found the child group's pool full */
#define RDN_TASK_HANDLE_RESOLVED 0xFFFFFFFFu

namespace rdn_task {

using Rec = rdn::task::Rec;  // word w of a record: rec[w]

struct Ctx {
  const rdn::TaskGraphDev* graph;
  uint32_t group;  // this task's group
  uint32_t index;  // this task's record

  __device__ Rec payload() const { return rdn::task::task_payload(graph->g[group], index); }
  __device__ Rec locals() const { return rdn::task::task_locals(graph->g[group], index); }
  __device__ uint32_t payload_words(uint32_t g) const { return graph->g[g].payload_words; }
  // Spawns a task of group `child_group` with this task as its parent; its
  // payload is zero until written through child_payload(). Returns the child's
  // handle, or RDN_TASK_HANDLE_UNINIT when that group has no free record (the
  // graph's error word then has RDN_TASK_ERROR_NO_FREE_SLOT).
  __device__ uint32_t spawn(uint32_t child_group) const {
    if (child_group >= graph->n_groups) return RDN_TASK_HANDLE_UNINIT;
    const uint32_t h = rdn::task::spawn_task(*graph, child_group, group, index);
    if (h != RDN_TASK_HANDLE_UNINIT) {
      const Rec b = child_payload(child_group, h);
      for (uint32_t w = 0; w < graph->g[child_group].payload_words; w++) b[w] = 0u;
    }
    return h;
  }
  __device__ Rec child_payload(uint32_t child_group, uint32_t handle) const {
    return rdn::task::task_payload(graph->g[child_group], handle);
  }
  // True when the child has finished; the child is then cleaned up, and its
  // payload stays readable through child_payload() until this launch ends.
  __device__ bool poll_child(uint32_t child_group, uint32_t handle) const {
    if (child_group >= graph->n_groups || handle == RDN_TASK_HANDLE_UNINIT || handle == RDN_TASK_HANDLE_RESOLVED)
      return false;
    return rdn::task::poll_child(*graph, child_group, handle);
  }
};

// One thread per active task of group g; finalises every poll as librdn's
// built-in programs do.
template <class Program>
__global__ void __launch_bounds__(128) poll_kernel(const rdn::TaskGraphDev* __restrict__ graph, uint32_t g,
                                                   typename Program::Params params) {
  const rdn::TaskGroupDev& T = graph->g[g];
  const rdn::GroupCtl* c = T.ctl;
  const uint32_t n = c->active.size;
  const uint32_t* list = T.active[c->sel];
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t idx = list[i];
    const uint32_t pi = T.parent_index[idx], pt = T.parent_type[idx];
    const bool resolved = Program::poll(Ctx{graph, g, idx}, params);
    rdn::task::finalize(*graph, g, idx, resolved, pi, pt);
  }
}

// Launches Program's poll over group `group` (the arguments of an
// rdn_task_poll_fn) on `stream`.
template <class Program>
inline rdn_status launch(const void* graph_device, uint32_t group, uint32_t group_capacity, void* stream,
                         const typename Program::Params& params) {
  const uint32_t grid = group_capacity ? (group_capacity + 127) / 128 : 1;
  poll_kernel<Program><<<grid, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const rdn::TaskGraphDev*>(graph_device), group, params);
  return cudaGetLastError() == cudaSuccess ? RDN_OK : RDN_ERR_CUDA;
}

}  // namespace rdn_task

#endif /* RDN_TASK_CUH */
