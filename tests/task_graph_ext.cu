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

// A ray-query pipeline of external programs around librdn's built-in trace
// task: ray generation (payload word 0 = ray index) spawns a trace task with
// the ray's trace call (trace-call payload layout of rdn.h; the user payload
// word carries the ray index) and waits for it; the closest-hit program
// records (t, u, v, primitive) of its payload, the miss program (tmax, 0, 0,
// miss). The host passes the buffers and groups through `user`.
struct QueryParams {
  const float4* rays;  // 2 per ray: origin, tmin / direction, tmax
  float4* out;         // per ray
  uint32_t count, trace_group, closest_group, miss_group, ray_flags, cull_mask;
};

struct RayGen {
  using Params = QueryParams;
  __device__ static bool poll(const rdn_task::Ctx& t, const Params& p) {
    const rdn_task::Rec L = t.locals(), P = t.payload();
    if (L[0] == 0u) {
      L[0] = 1u;
      const uint32_t i = P[0];
      if (i >= p.count) return true;
      const uint32_t h = t.spawn(p.trace_group);
      if (h != RDN_TASK_HANDLE_UNINIT) {
        const rdn_task::Rec c = t.child_payload(p.trace_group, h);
        const float4 a = p.rays[2 * i], b = p.rays[2 * i + 1];
        c[0] = __float_as_uint(a.x);
        c[1] = __float_as_uint(a.y);
        c[2] = __float_as_uint(a.z);
        c[3] = __float_as_uint(a.w);
        c[4] = __float_as_uint(b.x);
        c[5] = __float_as_uint(b.y);
        c[6] = __float_as_uint(b.z);
        c[7] = __float_as_uint(b.w);
        c[8] = p.ray_flags;
        c[9] = p.cull_mask;
        c[10] = 0u;
        c[11] = p.closest_group;
        c[12] = p.miss_group;
        c[13] = i;
      }
      L[1] = h;
      return false;
    }
    if (t.poll_child(p.trace_group, L[1])) {
      L[1] = RDN_TASK_HANDLE_RESOLVED;
      return true;
    }
    return false;
  }
};

struct RecordHit {
  using Params = QueryParams;
  __device__ static bool poll(const rdn_task::Ctx& t, const Params& p) {
    const rdn_task::Rec P = t.payload();
    const uint32_t i = P[13];
    if (i < p.count)
      p.out[i] = make_float4(__uint_as_float(P[18]), __uint_as_float(P[19]), __uint_as_float(P[20]),
                             __uint_as_float(P[23]));
    return true;
  }
};

struct RecordMiss {
  using Params = QueryParams;
  __device__ static bool poll(const rdn_task::Ctx& t, const Params& p) {
    const rdn_task::Rec P = t.payload();
    const uint32_t i = P[13];
    if (i < p.count) p.out[i] = make_float4(__uint_as_float(P[7]), 0.0f, 0.0f, __uint_as_float(0xFFFFFFFFu));
    return true;
  }
};

extern "C" rdn_status raygen_poll(const void* graph, uint32_t group, uint32_t cap, void* stream, void* user) {
  return rdn_task::launch<RayGen>(graph, group, cap, stream, *static_cast<const QueryParams*>(user));
}
extern "C" rdn_status record_hit_poll(const void* graph, uint32_t group, uint32_t cap, void* stream, void* user) {
  return rdn_task::launch<RecordHit>(graph, group, cap, stream, *static_cast<const QueryParams*>(user));
}
extern "C" rdn_status record_miss_poll(const void* graph, uint32_t group, uint32_t cap, void* stream, void* user) {
  return rdn_task::launch<RecordMiss>(graph, group, cap, stream, *static_cast<const QueryParams*>(user));
}
