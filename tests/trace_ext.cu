// Kernels of a caller's own that trace through librdn's traversal with
// any-hit programs of their own (include/rdn_trace.cuh), used by
// tests/test_trace_ext.py: EvenPrims restates RDN_ANYHIT_ACCEPT_EVEN_PRIMS;
// CutOut is a procedural alpha test (accept a hit when u + v < 0.5).
#include "rdn_trace.cuh"

struct EvenPrims {
  __device__ uint32_t operator()(const rdn_query::Params&, const rdn_query::AnyHitInfo& h) const {
    return (h.primitive & 1u) ? 0u : rdn_query::ACCEPT;
  }
};

struct CutOut {
  __device__ uint32_t operator()(const rdn_query::Params&, const rdn_query::AnyHitInfo& h) const {
    return h.u + h.v < 0.5f ? rdn_query::ACCEPT : 0u;
  }
};

template <int MODE, class AnyHit>
__global__ void trace_kernel(rdn_query::Params p, const rdn_ray* rays, float4* out, uint32_t n, uint32_t flags,
                             uint32_t mask) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const rdn_query::Hit h = rdn_query::trace<MODE>(p, rays[i], 0u, flags, mask, AnyHit{});
  out[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.prim));
}

template <int MODE, class AnyHit>
static int launch(const rdn_query::Params& p, const rdn_ray* rays, float4* out, uint32_t n, uint32_t flags,
                  uint32_t mask, cudaStream_t s) {
  trace_kernel<MODE, AnyHit><<<(n + 127) / 128, 128, 0, s>>>(p, rays, out, n, flags, mask);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

// anyhit: 0 EvenPrims, 1 CutOut; mode: rdn::MODE_THREADED or rdn::MODE_WIDE4
extern "C" int trace_custom(const void* params, const void* rays, void* out, uint32_t n, uint32_t anyhit,
                            uint32_t mode, uint32_t flags, uint32_t mask, void* stream) {
  const rdn_query::Params& p = *static_cast<const rdn_query::Params*>(params);
  const rdn_ray* r = static_cast<const rdn_ray*>(rays);
  float4* o = static_cast<float4*>(out);
  const cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (mode == rdn::MODE_WIDE4)
    return anyhit ? launch<rdn::MODE_WIDE4, CutOut>(p, r, o, n, flags, mask, s)
                  : launch<rdn::MODE_WIDE4, EvenPrims>(p, r, o, n, flags, mask, s);
  return anyhit ? launch<rdn::MODE_THREADED, CutOut>(p, r, o, n, flags, mask, s)
                : launch<rdn::MODE_THREADED, EvenPrims>(p, r, o, n, flags, mask, s);
}
