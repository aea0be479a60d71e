// A task program compiled outside librdn through include/rdn_task.cuh, used by
// tests/test_task_graph_ext.py. Countdown: payload word 0 = n. The first poll
// resolves at once when n == 0; otherwise it spawns a child of its own group
// with n - 1 and waits for it, resolving in the poll that finds it finished.
#include "rdn_task.cuh"

struct Countdown {
  struct Params {
    uint32_t unused;
  };
  __device__ static bool poll(const rdn_task::Ctx& t, const Params&) {
    const rdn_task::Rec L = t.locals(), P = t.payload();
    if (L[0] == 0u) {
      L[0] = 1u;
      const uint32_t n = P[0];
      if (n == 0u) return true;
      const uint32_t h = t.spawn(t.group);
      if (h != RDN_TASK_HANDLE_UNINIT) t.child_payload(t.group, h)[0] = n - 1u;
      L[1] = h;
      return false;
    }
    if (t.poll_child(t.group, L[1])) {
      L[1] = RDN_TASK_HANDLE_RESOLVED;
      return true;
    }
    return false;
  }
};

extern "C" rdn_status countdown_poll(const void* graph, uint32_t group, uint32_t cap, void* stream, void* user) {
  (void)user;
  return rdn_task::launch<Countdown>(graph, group, cap, stream, Countdown::Params{0});
}
