/* A host program that uses the library through its C ABI only (include/rdn.h
 * plus the CUDA runtime for device buffers), the way a Rust, Go or C++ host
 * binds it: one triangle geometry, one identity instance, a build, one batch
 * trace and, when a frame file is given, one frame of the path tracer's first
 * bounce (rdn_wavefront_shadow_bounce), and when a second file is given, one
 * sample of the reference path tracer (rdn_path_tracing_render), results
 * written to a file.
 *
 *   c_client <input> <output> <traversal> <device_build> [<frame> [<path-traced frame>]]
 *
 * input:  u32 vertex_count, u32 index_count (0 = non-indexed), u32 ray_count,
 *         f32 positions[3 * vertex_count], u32 indices[index_count],
 *         f32 rays[8 * ray_count] (org, tmin, dir, tmax)
 * frame:  u32 width, u32 height, u32 sample_index, f32 camera[14] (origin,
 *         forward, right, up, tan_half, aspect), f32 light[3]
 * path-traced frame: u32 width, u32 height, u32 sample_count, u32 max_path_depth,
 *         f32 view_projection_inv[16], f32 camera_position[3], f32 light[6]
 *         (illuminance, direction)
 * output: rdn_hit[ray_count], rdn_hit_ext[ray_count], u32 error_flags, and with
 *         a frame: rdn_pixel_result[width * height], u32 rays[3] (primary,
 *         shadow, bounce), u32 error_flags; with a path-traced frame: u8
 *         rgba[4 * width * height], u32 rays[2] (core, shadow), u32 error_flags
 *
 * Exit codes: 0 ok, 1 usage or file error, 2 an rdn_* call failed (its status
 * and rdn_last_error are printed), 3 a CUDA runtime call failed. */
#include <cuda_runtime_api.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rdn.h"

static rdn_ctx* ctx = NULL;

#define CHECK(x)                                                                                 \
  do {                                                                                           \
    rdn_status s_ = (x);                                                                         \
    if (s_ != RDN_OK) {                                                                          \
      fprintf(stderr, "%s failed: status %d: %s\n", #x, (int)s_, ctx ? rdn_last_error(ctx) : ""); \
      return 2;                                                                                  \
    }                                                                                            \
  } while (0)
#define CUCHECK(x)                                                      \
  do {                                                                  \
    cudaError_t e_ = (x);                                               \
    if (e_ != cudaSuccess) {                                            \
      fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));   \
      return 3;                                                         \
    }                                                                   \
  } while (0)

static int read_all(FILE* f, void* dst, size_t bytes) { return bytes == 0 || fread(dst, 1, bytes, f) == bytes; }

int main(int argc, char** argv) {
  if (argc < 5 || argc > 7) {
    fprintf(stderr, "usage: %s <input> <output> <traversal> <device_build> [<frame> [<path-traced frame>]]\n",
            argv[0]);
    return 1;
  }
  const uint32_t traversal = (uint32_t)atoi(argv[3]);
  const uint32_t device_build = (uint32_t)atoi(argv[4]);
  FILE* in = fopen(argv[1], "rb");
  if (!in) return 1;
  uint32_t head[3];
  if (!read_all(in, head, sizeof head)) return 1;
  const uint32_t nv = head[0], ni = head[1], nr = head[2];
  float* pos = (float*)malloc(12 * (size_t)nv + 4);
  uint32_t* idx = (uint32_t*)malloc(4 * (size_t)ni + 4);
  rdn_ray* rays = (rdn_ray*)malloc(sizeof(rdn_ray) * (size_t)nr + 4);
  if (!pos || !idx || !rays) return 1;
  if (!read_all(in, pos, 12 * (size_t)nv) || !read_all(in, idx, 4 * (size_t)ni) ||
      !read_all(in, rays, sizeof(rdn_ray) * (size_t)nr))
    return 1;
  fclose(in);
  if (rdn_api_version() != RDN_API_VERSION) {
    fprintf(stderr, "header and library disagree on the API version\n");
    return 1;
  }

  CHECK(rdn_create(&ctx, 0));
  rdn_geometry g;
  memset(&g, 0, sizeof g);
  g.type = 0; /* triangles */
  g.flags = RDN_GEOMETRY_OPAQUE;
  g.positions = pos;
  g.vertex_count = nv;
  g.index_count = ni;
  g.indices = ni ? idx : NULL;
  uint32_t blas = 0, tlas = 0;
  CHECK(rdn_blas_create(ctx, &g, 1, &blas));
  rdn_instance inst;
  memset(&inst, 0, sizeof inst);
  inst.transform[0] = inst.transform[5] = inst.transform[10] = inst.transform[15] = 1.0f;
  inst.mask = 0xFFu;
  inst.blas_handle = blas;
  CHECK(rdn_tlas_create(ctx, &inst, 1, &tlas));
  CHECK(rdn_bind_tlas(ctx, &tlas, 1));
  rdn_build_opts opts;
  memset(&opts, 0, sizeof opts);
  opts.blas_bin_size = 4;
  opts.device_build = device_build;
  CHECK(rdn_build(ctx, &opts));

  rdn_ray* d_rays = NULL;
  rdn_hit* d_hits = NULL;
  rdn_hit_ext* d_ext = NULL;
  CUCHECK(cudaMalloc((void**)&d_rays, sizeof(rdn_ray) * (size_t)nr + 32));
  CUCHECK(cudaMalloc((void**)&d_hits, sizeof(rdn_hit) * (size_t)nr + 16));
  CUCHECK(cudaMalloc((void**)&d_ext, sizeof(rdn_hit_ext) * (size_t)nr + 16));
  CUCHECK(cudaMemcpy(d_rays, rays, sizeof(rdn_ray) * (size_t)nr, cudaMemcpyHostToDevice));
  rdn_trace_desc d;
  memset(&d, 0, sizeof d);
  d.rays = d_rays;
  d.hits = d_hits;
  d.hits_ext = d_ext;
  d.count = nr;
  d.cull_mask = 0xFFu;
  d.traversal = traversal;
  CHECK(rdn_trace(ctx, &d, NULL));
  uint32_t flags = 0;
  CHECK(rdn_check_errors(ctx, NULL, &flags));

  rdn_hit* hits = (rdn_hit*)malloc(sizeof(rdn_hit) * (size_t)nr + 16);
  rdn_hit_ext* ext = (rdn_hit_ext*)malloc(sizeof(rdn_hit_ext) * (size_t)nr + 16);
  if (!hits || !ext) return 1;
  CUCHECK(cudaMemcpy(hits, d_hits, sizeof(rdn_hit) * (size_t)nr, cudaMemcpyDeviceToHost));
  CUCHECK(cudaMemcpy(ext, d_ext, sizeof(rdn_hit_ext) * (size_t)nr, cudaMemcpyDeviceToHost));
  FILE* out = fopen(argv[2], "wb");
  if (!out) return 1;
  fwrite(hits, sizeof(rdn_hit), nr, out);
  fwrite(ext, sizeof(rdn_hit_ext), nr, out);
  fwrite(&flags, 4, 1, out);

  if (argc >= 6) {
    /* one frame of the path tracer's first bounce: caller-owned scratch sized by the library */
    FILE* fr = fopen(argv[5], "rb");
    if (!fr) return 1;
    uint32_t fh[3];
    float cam[14], light[3];
    if (!read_all(fr, fh, sizeof fh) || !read_all(fr, cam, sizeof cam) || !read_all(fr, light, sizeof light))
      return 1;
    fclose(fr);
    const size_t npix = (size_t)fh[0] * fh[1];
    size_t scratch_bytes = 0;
    CHECK(rdn_wavefront_scratch_size(fh[0], fh[1], &scratch_bytes));
    void* d_scratch = NULL;
    rdn_pixel_result* d_out = NULL;
    uint32_t* d_counts = NULL;
    CUCHECK(cudaMalloc(&d_scratch, scratch_bytes));
    CUCHECK(cudaMalloc((void**)&d_out, sizeof(rdn_pixel_result) * npix + 32));
    CUCHECK(cudaMalloc((void**)&d_counts, 16));
    rdn_wavefront_desc w;
    memset(&w, 0, sizeof w);
    memcpy(w.camera.origin, cam, 12);
    memcpy(w.camera.forward, cam + 3, 12);
    memcpy(w.camera.right, cam + 6, 12);
    memcpy(w.camera.up, cam + 9, 12);
    w.camera.tan_half = cam[12];
    w.camera.aspect = cam[13];
    w.camera.width = fh[0];
    w.camera.height = fh[1];
    memcpy(w.light, light, 12);
    w.sample_index = fh[2];
    w.traversal = traversal;
    w.out = d_out;
    w.scratch = d_scratch;
    w.scratch_bytes = scratch_bytes;
    w.ray_counts = d_counts;
    CHECK(rdn_wavefront_shadow_bounce(ctx, &w, NULL));
    uint32_t wflags = 0;
    CHECK(rdn_check_errors(ctx, NULL, &wflags));
    rdn_pixel_result* px = (rdn_pixel_result*)malloc(sizeof(rdn_pixel_result) * npix + 32);
    uint32_t counts[3];
    if (!px) return 1;
    CUCHECK(cudaMemcpy(px, d_out, sizeof(rdn_pixel_result) * npix, cudaMemcpyDeviceToHost));
    CUCHECK(cudaMemcpy(counts, d_counts, sizeof counts, cudaMemcpyDeviceToHost));
    fwrite(px, sizeof(rdn_pixel_result), npix, out);
    fwrite(counts, 4, 3, out);
    fwrite(&wflags, 4, 1, out);
    free(px);
    cudaFree(d_scratch);
    cudaFree(d_out);
    cudaFree(d_counts);
  }
  if (argc >= 7) {
    /* one sample of the reference path tracer (rdn_path_tracing_render): the
     * wavefront schedule with caller-owned scratch, one directional light,
     * the default material; the RGBA8 image and the ray counts are written out */
    FILE* fp = fopen(argv[6], "rb");
    if (!fp) return 1;
    uint32_t ph[4];  /* width, height, sample_count, max_path_depth */
    float pv[16 + 3 + 6];  /* view_projection_inv, camera position, light illuminance + direction */
    if (!read_all(fp, ph, sizeof ph) || !read_all(fp, pv, sizeof pv)) return 1;
    fclose(fp);
    const size_t npix = (size_t)ph[0] * ph[1];
    size_t scratch_bytes = 0;
    CHECK(rdn_pt_scratch_size(ph[0], ph[1], &scratch_bytes));
    void* d_scratch = NULL;
    uint8_t* d_image = NULL;
    uint32_t* d_counts = NULL;
    rdn_pt_directional_light* d_light = NULL;
    CUCHECK(cudaMalloc(&d_scratch, scratch_bytes));
    CUCHECK(cudaMalloc((void**)&d_image, 4 * npix));
    CUCHECK(cudaMemset(d_image, 0, 4 * npix));
    CUCHECK(cudaMalloc((void**)&d_counts, 8));
    CUCHECK(cudaMemset(d_counts, 0, 8));
    CUCHECK(cudaMalloc((void**)&d_light, sizeof(rdn_pt_directional_light)));
    CUCHECK(cudaMemcpy(d_light, pv + 19, sizeof(rdn_pt_directional_light), cudaMemcpyHostToDevice));
    rdn_pt_desc pd;
    memset(&pd, 0, sizeof pd);
    memcpy(pd.view_projection_inv, pv, 64);
    memcpy(pd.camera_position, pv + 16, 12);
    pd.width = ph[0];
    pd.height = ph[1];
    pd.sample_count = ph[2];
    pd.max_path_depth = ph[3];
    pd.traversal = traversal;
    pd.tone_map = RDN_TONE_MAP_ACES_FILMIC;
    pd.exposure = 1.0f;
    pd.background = RDN_PT_BACKGROUND_SOLID;
    pd.lights = d_light;
    pd.light_count = 1;
    pd.image = d_image;
    pd.ray_counts = d_counts;
    pd.schedule = RDN_PT_SCHEDULE_WAVEFRONT;
    pd.scratch = d_scratch;
    pd.scratch_bytes = scratch_bytes;
    CHECK(rdn_path_tracing_render(ctx, &pd, NULL));
    uint32_t pflags = 0;
    CHECK(rdn_check_errors(ctx, NULL, &pflags));
    uint8_t* img = (uint8_t*)malloc(4 * npix + 16);
    uint32_t pcounts[2];
    if (!img) return 1;
    CUCHECK(cudaMemcpy(img, d_image, 4 * npix, cudaMemcpyDeviceToHost));
    CUCHECK(cudaMemcpy(pcounts, d_counts, sizeof pcounts, cudaMemcpyDeviceToHost));
    fwrite(img, 4, npix, out);
    fwrite(pcounts, 4, 2, out);
    fwrite(&pflags, 4, 1, out);
    free(img);
    cudaFree(d_scratch);
    cudaFree(d_image);
    cudaFree(d_counts);
    cudaFree(d_light);
  }
  fclose(out);

  cudaFree(d_rays);
  cudaFree(d_hits);
  cudaFree(d_ext);
  CHECK(rdn_destroy(ctx));
  ctx = NULL;
  free(pos);
  free(idx);
  free(rays);
  free(hits);
  free(ext);
  return 0;
}
