/*
 * rdn_trace.cuh — ray queries with an any-hit program of your own.
 *
 * The reference calls a user any-hit shader for every candidate hit on
 * non-opaque geometry (RayAnyHitBehavior, api/ty.rs:134-136;
 * traverse_gpu.rs:296-367): accept it, ignore it, and/or end the search. librdn's
 * entry points take fixed policies (RDN_ANYHIT_*); this header lets a CUDA
 * kernel of your own trace rays through librdn's traversal with any functor in
 * their place:
 *
 *   struct AlphaTest {
 *     const uint32_t* bits;
 *     __device__ uint32_t operator()(const rdn_query::Params&, const rdn_query::AnyHitInfo& h) const {
 *       return bit(bits, h.triangle) ? rdn_query::ACCEPT : 0u;
 *     }
 *   };
 *   rdn_query::Params p;                                  // once per build, on the host
 *   size_t n = sizeof(p);
 *   rdn_trace_params(ctx, RDN_TRAVERSAL_ORDERED_WIDE, &p, &n);
 *   ... in a kernel: rdn_query::Hit h = rdn_query::trace<rdn::MODE_WIDE4>(p, ray, tlas, flags, mask, AlphaTest{bits});
 *
 * The functor runs inside the walk with the same order and range rules as the
 * built-in policies, so a functor that restates a policy returns that
 * policy's hits bit for bit. Build with nvcc, -I include -I rendiation_gb300/csrc.
 */
#ifndef RDN_TRACE_CUH
#define RDN_TRACE_CUH

#include <cuda_runtime.h>

#include <cstdint>

#include "rdn.h"
#include "traverse.cuh"

namespace rdn_query {

using Params = rdn::TraceParams;
using AnyHitInfo = rdn::dev::AnyHitInfo;
constexpr uint32_t ACCEPT = rdn::dev::ANYHIT_ACCEPT;  // commit the hit (it becomes the closest so far)
constexpr uint32_t END_SEARCH = rdn::dev::ANYHIT_END;  // stop the query after this candidate

struct Hit {
  float t, u, v;
  uint32_t prim;      // primitive index within its geometry, RDN_MISS on a miss
  uint32_t geometry;  // geometry index within the BLAS
  uint32_t instance;  // TLAS instance slot
  uint32_t hit_kind;  // RDN_HIT_KIND_*; 0 on a miss
  bool unbound_tlas;  // the ray named a TLAS index that is not bound
};

// One query: MODE rdn::MODE_THREADED (the reference's order) or
// rdn::MODE_WIDE4 / rdn::MODE_BINARY (ordered walks; Params from
// rdn_trace_params with that traversal, whose stack fits this thread's
// local array). Params asked for with RDN_INTERSECT_WATERTIGHT select the
// watertight triangle test (both forms are compiled into the caller's kernel).
template <int MODE, class AnyHit>
__device__ inline Hit trace(const Params& p, const rdn_ray& ray, uint32_t tlas, uint32_t ray_flags,
                            uint32_t cull_mask, const AnyHit& anyhit) {
  uint2 stack[MODE == rdn::MODE_THREADED ? 1 : rdn::kLocalStackEntries];
  rdn::dev::RayCtx R;
  R.o = make_float3(ray.org[0], ray.org[1], ray.org[2]);
  R.tmin = ray.tmin;
  R.d = make_float3(ray.dir[0], ray.dir[1], ray.dir[2]);
  R.tmax = ray.tmax;
  R.ray_flags = ray_flags;
  R.cull_mask = cull_mask;
  bool bad;
  if (p.watertight)
    rdn::dev::traverse_ray<MODE, false, AnyHit, true>(p, R, tlas, stack, 1u, bad, anyhit);
  else
    rdn::dev::traverse_ray<MODE, false, AnyHit, false>(p, R, tlas, stack, 1u, bad, anyhit);
  Hit h;
  h.unbound_tlas = bad;
  if (R.best.have) {
    const uint4 gm = __ldg(reinterpret_cast<const uint4*>(p.tri_root + R.best.geom_slot));
    h.t = R.best.t;
    h.u = R.best.u;
    h.v = R.best.v;
    h.prim = __ldg(p.redirect + R.best.k) - gm.z;
    h.geometry = gm.y;
    h.instance = R.best.inst;
    h.hit_kind = R.best.s < 0.0f ? RDN_HIT_KIND_BACK_FACING_TRIANGLE : RDN_HIT_KIND_FRONT_FACING_TRIANGLE;
  } else {
    h.t = R.tmax;
    h.u = h.v = 0.0f;
    h.prim = h.geometry = h.instance = RDN_MISS;
    h.hit_kind = 0u;
  }
  return h;
}

}  // namespace rdn_query

#endif /* RDN_TRACE_CUH */
