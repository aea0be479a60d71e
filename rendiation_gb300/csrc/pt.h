// The reference path tracer (DeviceReferencePathTracingRenderer,
// scene/rendering/gpu-ray-tracing/src/feature/path_tracing) as a fused frame
// kernel: its environment and launch.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "task_graph.h"
#include "trace_kernels.h"

namespace rdn {

// rdn_pt_material (64 B): the channels PhysicalShading::construct_shading_impl
// reads (content/lighting/transport/src/surface/microfacet/device/direct_lighting.rs:14-54).
struct PtMaterial {
  float base_color[3];
  float perceptual_roughness;
  float emissive[3];
  float metallic;
  float specular[3];
  float reflectance;
  uint32_t workflow;  // 0 metallic-roughness, 1 specular
  uint32_t reserved[3];
};
static_assert(sizeof(PtMaterial) == 64, "64 B material");

// rdn_pt_directional_light (24 B): DirectionalLightStorage's illuminance and direction.
struct PtLight {
  float illuminance[3];
  float direction[3];
};
static_assert(sizeof(PtLight) == 24, "24 B light");

constexpr uint32_t PT_TONE_NONE = 0, PT_TONE_LINEAR = 1, PT_TONE_REINHARD = 2, PT_TONE_CINEON = 3,
                   PT_TONE_ACES = 4;
constexpr uint32_t PT_BACKGROUND_SOLID = 0, PT_BACKGROUND_TEST = 1, PT_BACKGROUND_ENV_CUBE = 2;

struct PtEnv {
  AoEnv view;  // camera, frame size, sample index, TLAS, built arrays, normals, RGBA8 image, ray counts
  uint32_t max_depth;
  uint32_t tone_map;
  float exposure;
  uint32_t background;
  float bg[3];
  const PtLight* lights;
  uint32_t light_count;
  const PtMaterial* materials;
  uint32_t material_count;
  const uint32_t* sm_to_material;
  uint32_t sm_count;
  float4* radiance;  // nullable: per pixel (HDR radiance of this sample, core rays traced)
  uint32_t schedule;  // 0 one thread per pixel; 1 persistent warps refilled with pixels as paths end;
                      // 2 wavefront passes over path queues (PtWave)
  uint32_t* fetch;    // refill schedule: the frame's pixel counter (zeroed before the launch)
  uint32_t register_tier;  // refill schedule, local-stack walks: 0 compiler's choice, 1 <= 96, 2 <= 64 registers
  const float4* env;       // environment cube: 6 faces (+X -X +Y -Y +Z -Z) of env_size^2 RGBA texels, rows of t
  uint32_t env_size;
  float env_transform[16];  // Mat4, reference memory order
  float env_intensity;
};

// Wavefront schedule: path state of every pixel in HBM and queues of pixel
// indices between passes (one pass per ray kind and depth).
constexpr uint32_t kPtStateWords = 28;
constexpr uint32_t kPtMaxPasses = 2 * 64;
struct PtWave {
  uint32_t* state;     // kPtStateWords x n_pix, word-major
  uint32_t* queue[2];  // n_pix entries each: pass p reads queue[(p + 1) & 1], appends to queue[p & 1]
  uint32_t* counters;  // [0, kPtMaxPasses): entries appended by pass p; then the passes' fetch counters
  uint32_t n_pix;
};
size_t pt_scratch_bytes(uint32_t width, uint32_t height);
// Carves the scratch (256-byte aligned, pt_scratch_bytes) into a PtWave.
PtWave pt_wave_layout(void* scratch, uint32_t width, uint32_t height);

cudaError_t launch_pt(const TraceParams& p, const PtEnv& e, const PtWave* w, int mode, int sm_count, cudaStream_t st);

}  // namespace rdn
