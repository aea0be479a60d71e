// Fused path-tracing frame for sm_103a: the reference path tracer's ray
// generation (path_tracing/ray_gen.rs:89-211), closest hit with its shadow
// trace (ray_hit.rs:12-103), shadow closest hit / miss (mod.rs:197-209) and
// miss (ray_miss.rs:10-28) as one kernel, one thread per pixel, warps over 8x4
// pixel tiles. Each thread walks its path with one traversal call site: the
// core ray and the shadow ray of a hit take turns through it, so the kernel
// holds one inlined traversal instead of two. Built with -fmad=false: see
// pt.cuh.
#include <cuda_runtime.h>

#include <cstdint>

#include "pt.cuh"
#include "traverse.cuh"

namespace rdn {
namespace {

using namespace dev;

template <int MODE, bool LOCAL, bool WT>
__global__ void __launch_bounds__(128) pt_kernel(TraceParams P, PtEnv E) {
  RDN_TRAVERSAL_STACK(LOCAL);
  const AoEnv& A = E.view;
  uint32_t x, y;
  const bool valid = ao_pixel(A, blockIdx.x * blockDim.x + threadIdx.x, x, y);
  uint32_t core = 0, shadow = 0;
  if (valid) {
    const uint32_t sample = ao_sample(A);
    float3 o, d;
    ao_camera_ray(A, x, y, o, d);
    float3 throughput = splat3(1.0f), radiance = splat3(0.0f);
    // state of a hit carried across its shadow trace
    float3 hit = splat3(0.0f), sn = hit, origin = hit, ldir = hit, lrad = hit;
    uint32_t sm_id = 0;
    uint32_t depth = 0;
    bool shadow_phase = false, bad = false;
    while (depth < E.max_depth) {
      RayCtx R;
      R.o = shadow_phase ? origin : o;
      R.d = shadow_phase ? ldir : d;
      R.tmin = F32_EPSILON;
      R.tmax = F32_MAX;  // core: RayRange::default; shadow: the directional light's distance
      R.ray_flags = shadow_phase ? RAY_FLAG_END_SEARCH : RAY_FLAG_CULL_BACK;
      R.cull_mask = 0xFFFFFFFFu;
      bool b;
      traverse_ray<MODE, false, BuiltinAnyHit, WT>(P, R, A.tlas, stack_ptr, stack_stride, b);
      bad |= b;
      if (!shadow_phase) {
        core++;
        if (!R.best.have) {  // miss shader, then the ray generation's miss branch
          const float3 s = pt_miss(E, d);
          radiance = make_float3((throughput.x * s.x + 0.0f) + radiance.x, (throughput.y * s.y + 0.0f) + radiance.y,
                                 (throughput.z * s.z + 0.0f) + radiance.z);
          break;
        }
        // closest hit, first part: light sample and shadow ray
        hit = o + d * R.best.t;
        const DeviceInstance* inst = P.tlas_data + R.best.inst;
        float3 gn;
        sn = hit_normals(A, inst, __ldg(P.redirect + R.best.k), R.best.u, R.best.v, o, hit, gn);
        sm_id = __ldg(&inst->instance_custom_index);
        uint32_t ls = xxhash32(x, y, sample * 2u);
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
        ldir = neg3(dir);
        const float pdf_l = 1.0f * pmf;
        lrad = light_ok ? illum / pdf_l : splat3(0.0f);
        origin = offset_ray_hit(hit, gn);
        if (light_ok) {
          shadow_phase = true;
          continue;
        }
      } else {
        shadow++;
        if (R.best.have) lrad = splat3(0.0f);  // shadow closest hit
        shadow_phase = false;
      }
      // closest hit, map: BRDF sample, direct light through the BRDF
      const float3 view = neg3(d);
      const PtSurface s = pt_surface(E, sm_id);
      uint32_t bs = xxhash32(x, y, sample * 3u);
      float3 brdf;
      float pdf;
      const float3 sdir = pt_sample(s, view, sn, bs, brdf, pdf);
      const float3 brdf_l = pt_bsdf(s, view, ldir, sn);
      const float light_dot = fabsf(dot3(sn, ldir));
      const float3 sampled = make_float3((light_dot * brdf_l.x) * lrad.x, (light_dot * brdf_l.y) * lrad.y,
                                         (light_dot * brdf_l.z) * lrad.z);
      // ray generation's hit branch
      if (pdf == 0.0f) depth = E.max_depth;
      depth = depth + 1u;
      const float cosv = dot3(sdir, sn);
      const float pdf_c = fmaxf(pdf, PT_MIN_PDF);
      throughput = make_float3(((throughput.x * cosv) * brdf.x) / pdf_c, ((throughput.y * cosv) * brdf.y) / pdf_c,
                               ((throughput.z * cosv) * brdf.z) / pdf_c);
      radiance = make_float3(throughput.x * sampled.x + radiance.x, throughput.y * sampled.y + radiance.y,
                             throughput.z * sampled.z + radiance.z);
      o = origin;
      d = sdir;
    }
    if (bad) atomicOr(P.error_word, 2u);
    const uint32_t pixel = y * A.width + x;
    pt_accumulate(E, pixel, pt_tone_map(E, radiance));
    if (E.radiance) E.radiance[pixel] = make_float4(radiance.x, radiance.y, radiance.z, (float)core);
  }
  if (A.ray_counts) {
    const uint32_t c = __reduce_add_sync(0xffffffffu, core), s = __reduce_add_sync(0xffffffffu, shadow);
    if ((threadIdx.x & 31u) == 0u) {
      if (c) atomicAdd(A.ray_counts + 0, c);
      if (s) atomicAdd(A.ray_counts + 1, s);
    }
  }
}

template <int MODE, bool LOCAL, bool WT>
cudaError_t launch_variant_wt(const TraceParams& p, const PtEnv& e, cudaStream_t st) {
  const uint32_t block = e.view.block ? e.view.block : 128;
  const uint32_t grid = (ao_dispatch_count(e.view.width, e.view.height) + block - 1) / block;
  const size_t smem = MODE != MODE_THREADED && !LOCAL ? (size_t)p.stack_depth * block * sizeof(uint2) : 0;
  static std::atomic<uint64_t> attr_done{0};
  const cudaError_t err = raise_smem_limit(attr_done, {(const void*)pt_kernel<MODE, LOCAL, WT>});
  if (err != cudaSuccess) return err;
  pt_kernel<MODE, LOCAL, WT><<<grid, block, smem, st>>>(p, e);
  return cudaGetLastError();
}

template <int MODE, bool LOCAL>
cudaError_t launch_variant(const TraceParams& p, const PtEnv& e, cudaStream_t st) {
  return p.watertight ? launch_variant_wt<MODE, LOCAL, true>(p, e, st) : launch_variant_wt<MODE, LOCAL, false>(p, e, st);
}

}  // namespace

cudaError_t launch_pt(const TraceParams& p, const PtEnv& e, int mode, cudaStream_t st) {
  if (e.view.width == 0 || e.view.height == 0) return cudaSuccess;
  if (mode == MODE_WIDE4)
    return p.local_stack ? launch_variant<MODE_WIDE4, true>(p, e, st) : launch_variant<MODE_WIDE4, false>(p, e, st);
  if (mode == MODE_BINARY)
    return p.local_stack ? launch_variant<MODE_BINARY, true>(p, e, st) : launch_variant<MODE_BINARY, false>(p, e, st);
  return launch_variant<MODE_THREADED, false>(p, e, st);
}

}  // namespace rdn
