/*
 * rdn.h — C ABI of the GB300 ray-query library (librdn.so).
 *
 * This is the drop-in boundary for the reference's ray-query path
 * (mikialex/rendiation, shader/ray-tracing). Each entry point names the
 * reference interface it replaces. The reference exposes Rust traits whose
 * device half returns shader-EDSL nodes, so the boundary a Rust host binds is
 * this C ABI: an `extern "C"` block plus a trait implementation that forwards
 * to it.
 *
 * Conventions
 *  - Every entry point returns rdn_status; nothing aborts or traps. The text
 *    of the last error of a context is available from rdn_last_error().
 *  - Source arrays passed to *_create are copied, as the reference clones its
 *    sources (naive/mod.rs:98-109).
 *  - Handles are dense u32 slots; deleting leaves an empty slot, as in the
 *    reference (naive/mod.rs:110-119).
 *  - Ray and hit buffers passed to rdn_trace are DEVICE pointers owned by the
 *    caller; work is stream-ordered on the given cudaStream_t (NULL = legacy
 *    default stream). Acceleration-structure buffers are owned by the context.
 *  - Create/delete/bind/build take the context's lock (the reference's
 *    Arc<RwLock> write lock, naive/mod.rs:497-609); traces on distinct
 *    streams may run concurrently once the structure is built. Persistent
 *    kernels that claim work from a counter of the context (the refill path
 *    tracer, the differentiable paths) allow one call of each kind in flight
 *    per context.
 */
#ifndef RDN_H
#define RDN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RDN_API_VERSION 1u

typedef int32_t rdn_status;
#define RDN_OK 0
#define RDN_ERR_INVALID_ARG (-1)
#define RDN_ERR_INVALID_HANDLE (-2)
#define RDN_ERR_OOM (-3)
#define RDN_ERR_CUDA (-4)
#define RDN_ERR_QUEUE_OVERFLOW (-5)
#define RDN_ERR_TIMEOUT (-6)
#define RDN_ERR_NOT_BUILT (-7)
#define RDN_ERR_UNSUPPORTED (-8)

/* Ray flags: the reference's RayFlagConfigRaw values (api/ty.rs:102-114). */
#define RDN_RAY_FLAG_NONE 0x00u
#define RDN_RAY_FLAG_FORCE_OPAQUE 0x01u
#define RDN_RAY_FLAG_FORCE_NON_OPAQUE 0x02u
#define RDN_RAY_FLAG_ACCEPT_FIRST_HIT_AND_END_SEARCH 0x04u
#define RDN_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER 0x08u
#define RDN_RAY_FLAG_CULL_BACK_FACING_TRIANGLES 0x10u
#define RDN_RAY_FLAG_CULL_FRONT_FACING_TRIANGLES 0x20u
#define RDN_RAY_FLAG_CULL_OPAQUE 0x40u
#define RDN_RAY_FLAG_CULL_NON_OPAQUE 0x80u
#define RDN_RAY_FLAG_SKIP_TRIANGLES 0x100u
#define RDN_RAY_FLAG_SKIP_PROCEDURAL_PRIMITIVES 0x200u

/* Instance flags (api/ty.rs:142-151) and geometry flags (api/ty.rs:153-159). */
#define RDN_INSTANCE_TRIANGLE_FACING_CULL_DISABLE 0x1u
#define RDN_INSTANCE_TRIANGLE_FLIP_FACING 0x2u
#define RDN_INSTANCE_FORCE_OPAQUE 0x4u
#define RDN_INSTANCE_FORCE_NO_OPAQUE 0x8u
#define RDN_GEOMETRY_OPAQUE 0x1u
#define RDN_GEOMETRY_NO_DUPLICATE_ANYHIT_INVOCATION 0x2u

/* Hit kinds (api/ty.rs:138-140). */
#define RDN_HIT_KIND_FRONT_FACING_TRIANGLE 0xFEu
#define RDN_HIT_KIND_BACK_FACING_TRIANGLE 0xFFu

#define RDN_MISS 0xFFFFFFFFu

typedef struct rdn_ctx rdn_ctx;

/* BottomLevelAccelerationStructureBuildSource (api/backend.rs:103-118).
 * type 0 = triangles (positions xyz f32 per vertex; indices nullable: NULL
 * means non-indexed, every 3 vertices form a triangle, naive/mod.rs:158-162);
 * type 1 = AABBs, accepted and ignored exactly as the reference's naive
 * system ignores them (naive/mod.rs:201-237). */
typedef struct rdn_geometry {
  uint32_t type;
  uint32_t flags; /* RDN_GEOMETRY_* */
  const float* positions;
  uint32_t vertex_count;
  uint32_t index_count;
  const uint32_t* indices;
} rdn_geometry;

/* TopLevelAccelerationStructureSourceInstance (api/backend.rs:160-167).
 * transform is a Mat4 in the reference's memory order (columns a, b, c, d;
 * translation in elements 12..14). */
typedef struct rdn_instance {
  float transform[16];
  uint32_t custom_index;
  uint32_t mask;
  uint32_t sbt_offset;
  uint32_t flags; /* RDN_INSTANCE_* */
  uint32_t blas_handle;
} rdn_instance;

/* TreeBuildOption (content/space/src/utils.rs:20-38) for BLAS and TLAS. The
 * reference hard-codes BLAS {max_tree_depth 50, bin_size 2} and TLAS
 * {50, 10} with SAH::new(4) (naive/mod.rs:173-177,280-284); those are the
 * defaults (a zero field selects its default). host_threads 0 = all cores. */
typedef struct rdn_build_opts {
  uint32_t blas_bin_size;
  uint32_t blas_max_depth;
  uint32_t tlas_bin_size;
  uint32_t tlas_max_depth;
  uint32_t host_threads;
  /* 1: build the triangle trees on the context's GPU (every flattened array
   * byte-identical to the host build, which follows the reference's
   * single-threaded builder); the TLAS stays on the host. 0: host build. */
  uint32_t device_build;
  uint32_t reserved[2];
} rdn_build_opts;

/* One ray, 32 B: ShaderRayTraceCallStoragePayload's origin, direction and
 * range (backend/wavefront_compute/ctx.rs:15-29). */
typedef struct rdn_ray {
  float org[3];
  float tmin;
  float dir[3];
  float tmax;
} rdn_ray;

/* Closest/any hit, 16 B. prim = primitive index within its geometry
 * (traverse_cpu.rs:160), RDN_MISS for a miss; t = world distance
 * (traverse_cpu.rs:157); u, v = barycentric weights of vertices 1 and 2
 * (geometry/mod.rs:144-154). On a miss t = the ray's tmax and u = v = 0. */
typedef struct rdn_hit {
  float t;
  float u;
  float v;
  uint32_t prim;
} rdn_hit;

/* Optional per-ray hit context, 16 B (HitCtxStorage, ctx.rs:46-57):
 * geometry index within the BLAS, instance slot (position in the built
 * instance array, traverse_gpu.rs:556-570), the instance's custom index and
 * the hit kind. All RDN_MISS (hit_kind 0) on a miss. */
typedef struct rdn_hit_ext {
  uint32_t geometry;
  uint32_t instance;
  uint32_t instance_custom;
  uint32_t hit_kind;
} rdn_hit_ext;

/* Traversal order.
 * RDN_TRAVERSAL_ORDERED (default): nearest-child-first stack traversal over
 *   64 B two-child nodes holding the reference's exact node boxes, with
 *   speculative leaf postponement (a lane that reaches a leaf keeps descending
 *   until its whole warp holds leaves, so triangle tests run together). Closest
 *   hits equal the reference's except among hits at exactly equal distance;
 *   first-hit (shadow) queries agree on hit/miss.
 * RDN_TRAVERSAL_REFERENCE: the reference's stackless threaded hit/miss walk
 *   (traverse_cpu.rs:291-319) over its own 48 B node layout; bit-identical to
 *   the reference CPU traversal, including ties and which hit ends a search.
 * RDN_TRAVERSAL_ORDERED_WIDE: as ORDERED over 128 B four-child nodes collapsed
 *   from the same tree (faster on coherent rays such as camera primaries). */
#define RDN_TRAVERSAL_ORDERED 0u
#define RDN_TRAVERSAL_REFERENCE 1u
#define RDN_TRAVERSAL_ORDERED_WIDE 2u

/* Triangle test, OR-ed into any traversal value of any entry point.
 * Without it (the default) every triangle is tested with the reference's
 * formula (geometry/mod.rs:105-155): plane distance from the normalised
 * normal, projected barycentrics. That formula is not watertight: a ray
 * through an edge shared by two triangles can miss both, and a zero-area
 * triangle (or a ray in a triangle's plane) gives t = NaN, which the
 * reference accepts as a hit.
 * RDN_INTERSECT_WATERTIGHT: the watertight f32 test of Woop, Benthin and Wald
 * (JCGT 2013) on the shared vertex values, with box tests made conservative
 * against rounding (exit distance times 1 + 2 gamma_3, Ize, JCGT 2013): no ray
 * passes between two triangles that share an edge, a NaN distance never hits,
 * facing and culling follow the reference's rules. One case keeps the
 * reference box test's NaN rule: a ray with an exactly zero direction
 * component that lies exactly in a box's face plane skips that box. Hit/miss
 * and primitive ids differ from the reference's only for rays at an
 * equal-distance tie, rays near a triangle edge, and rays the reference gives
 * a NaN distance; t and the barycentrics are this test's own f32 values. */
#define RDN_INTERSECT_WATERTIGHT 0x100u

/* Fixed any-hit policies for non-opaque geometry, standing in for a user
 * any-hit shader (RayAnyHitBehavior, api/ty.rs:134-136). */
#define RDN_ANYHIT_ACCEPT 0u
#define RDN_ANYHIT_ACCEPT_AND_END 1u
#define RDN_ANYHIT_ACCEPT_EVEN_PRIMS 2u
#define RDN_ANYHIT_PRIMITIVE_MASK 3u   /* accept a non-opaque hit when bit t of anyhit_mask is set, t the
                                          built triangle index (creation order); a data-driven alpha test */

typedef struct rdn_trace_desc {
  const rdn_ray* rays;      /* device, count entries */
  rdn_hit* hits;            /* device, count entries */
  rdn_hit_ext* hits_ext;    /* device, nullable */
  const uint32_t* tlas_idx; /* device, nullable: per-ray index into the bound TLAS list */
  uint32_t count;
  uint32_t tlas_uniform;    /* used when tlas_idx is NULL */
  uint32_t ray_flags;       /* RDN_RAY_FLAG_* */
  uint32_t cull_mask;       /* low 8 bits used */
  uint32_t traversal;       /* RDN_TRAVERSAL_* */
  uint32_t anyhit_mode;     /* RDN_ANYHIT_* */
  uint32_t block_size;      /* 0 = 64 */
  uint32_t local_stack;      /* ordered walks: 1 = per-thread traversal stacks in local memory (L1)
                                instead of shared memory, for trees whose stack fits 64 entries */
  const uint32_t* anyhit_mask; /* device, RDN_ANYHIT_PRIMITIVE_MASK: one bit per built triangle */
} rdn_trace_desc;

/* ---- device status ----------------------------------------------------- */

/* Bits of the device error word the kernels set instead of faulting. */
#define RDN_ERROR_STACK_OVERFLOW 0x1u   /* a traversal stack push past its depth (unreachable by construction) */
#define RDN_ERROR_BAD_TLAS_INDEX 0x2u   /* a ray named a TLAS index that is not bound (the ray misses) */
#define RDN_ERROR_ITERATION_LIMIT 0x4u  /* a dynamic-fetch warp reached its iteration limit and stopped */

/* Waits for `stream`, reads and clears the context's device error word
 * (*flags, nullable) and returns RDN_ERR_TIMEOUT when a warp hit its iteration
 * limit, RDN_ERR_QUEUE_OVERFLOW on a stack overflow, else RDN_OK. The
 * reference aborts instead (panic = "abort"); kernels here record and return. */
rdn_status rdn_check_errors(rdn_ctx* ctx, void* stream, uint32_t* flags);

/* Iteration cap of the dynamic-fetch loops (refill > 0) of every later launch;
 * 0 restores the built-in cap (2^24, far above any real traversal). A lower cap
 * lets a caller (or a test) bound the work of one launch: warps that reach it
 * stop, and rdn_check_errors reports RDN_ERR_TIMEOUT. */
rdn_status rdn_set_iteration_limit(rdn_ctx* ctx, uint32_t limit);

/* Counters of node visits and triangle tests, the reference's
 * BVH_VISIT_COUNT / TRI_VISIT_COUNT (traverse_cpu.rs:38-41). */
typedef struct rdn_counters {
  uint64_t node_visits;
  uint64_t tri_tests;
  uint64_t tri_hits;
  uint64_t bad_tlas_rays;
} rdn_counters;

/* ---- context ---------------------------------------------------------- */

/* Replaces NaiveSahBVHSystem::new (naive/mod.rs:508-519). device >= 0 selects a
 * CUDA device; device == -1 creates a host-only context that can build (and
 * export the built arrays) but rejects traces with RDN_ERR_UNSUPPORTED. */
rdn_status rdn_create(rdn_ctx** out, int device);
rdn_status rdn_destroy(rdn_ctx* ctx);
const char* rdn_last_error(const rdn_ctx* ctx);
uint32_t rdn_api_version(void);

/* ---- acceleration structures (GPUAccelerationStructureSystemProvider,
 *      api/backend.rs:120-142; naive/mod.rs:560-609) ------------------- */

/* create_bottom_level_acceleration_structure */
rdn_status rdn_blas_create(rdn_ctx* ctx, const rdn_geometry* geometries, uint32_t count, uint32_t* out_handle);
/* delete_bottom_level_acceleration_structure */
rdn_status rdn_blas_delete(rdn_ctx* ctx, uint32_t handle);
/* create_top_level_acceleration_structure */
rdn_status rdn_tlas_create(rdn_ctx* ctx, const rdn_instance* instances, uint32_t count, uint32_t* out_handle);
/* delete_top_level_acceleration_structure */
rdn_status rdn_tlas_delete(rdn_ctx* ctx, uint32_t handle);
/* bind_tlas; bind_tlas_max_len is u32::MAX in the reference */
rdn_status rdn_bind_tlas(rdn_ctx* ctx, const uint32_t* handles, uint32_t count);
/* Explicit build + upload (the reference builds lazily in
 * get_or_build_gpu_data, naive/mod.rs:521-537; rdn_trace does the same when
 * the structure is dirty). opts may be NULL. */
rdn_status rdn_build(rdn_ctx* ctx, const rdn_build_opts* opts);
/* Statistics of the last build. */
typedef struct rdn_build_stats {
  uint64_t device_bytes;      /* acceleration-structure bytes resident on the device */
  uint64_t triangles;
  uint64_t nodes;             /* BLAS nodes in the reference's forest */
  uint64_t sah_splits;
  uint64_t median_fallbacks;  /* degenerate binning -> BalanceTree median split */
  uint32_t max_blas_depth;
  uint32_t device_built;      /* 1 when the triangle trees were built on the GPU */
  double build_seconds;       /* SAH build + flattening, wall clock */
  double upload_seconds;
  double device_seconds;      /* device build only: span of its work on the GPU stream */
} rdn_build_stats;
rdn_status rdn_get_build_stats(const rdn_ctx* ctx, rdn_build_stats* out);

/* Copies one of the built arrays in the reference's flattened layout
 * (NaiveSahBvhCpu fields, traverse_cpu.rs:9-35) to host memory `dst` of
 * `capacity` bytes; the byte size is written to *size. which:
 * 0 tlas_binding, 1 tlas_bvh_root, 2 tlas_bvh_forest, 3 tlas_data,
 * 4 tlas_bounding, 5 blas_meta_info, 6 tri_bvh_root, 7 tri_bvh_forest,
 * 8 indices_redirect, 9 indices, 10 vertices. dst may be NULL to query. */
rdn_status rdn_get_built_array(const rdn_ctx* ctx, uint32_t which, void* dst, size_t capacity, size_t* size);

/* ---- queries -------------------------------------------------------- */

/* Batch closest/any-hit query with NaiveSahBvhCpu::traverse semantics
 * (traverse_cpu.rs:52-245), one result per ray. */
rdn_status rdn_trace(rdn_ctx* ctx, const rdn_trace_desc* desc, void* stream);

/* Same as rdn_trace, additionally accumulating node-visit and triangle-test
 * counts (slower; for measurement). */
rdn_status rdn_trace_counted(rdn_ctx* ctx, const rdn_trace_desc* desc, void* stream, rdn_counters* out);

/* Device view of the built structure for kernels of the caller's that trace
 * with include/rdn_trace.cuh (any-hit programs of their own): fills `out`
 * (host memory of *size bytes, at least the size this call reports in
 * *size when out is NULL) with the traversal parameters of `traversal`,
 * building the structure first if needed. Valid until the next rdn_build or
 * a change to the sources. The ordered walks keep their stack in a 64-entry
 * local array: RDN_ERR_UNSUPPORTED for a tree too deep for it. */
rdn_status rdn_trace_params(rdn_ctx* ctx, uint32_t traversal, void* out, size_t* size);

/* ---- wavefront executor -------------------------------------------- */

/* Pinhole camera: ray(px, py) = normalize(forward + sx*right + sy*up) with
 * sx = ((px+0.5)/width*2-1)*tan_half*aspect, sy = (1-(py+0.5)/height*2)*tan_half. */
typedef struct rdn_camera {
  float origin[3];
  float forward[3];
  float right[3];
  float up[3];
  float tan_half;
  float aspect;
  uint32_t width;
  uint32_t height;
} rdn_camera;

/* One pixel of the primary + shadow + bounce workload, 32 B. */
typedef struct rdn_pixel_result {
  uint32_t primary_prim;     /* RDN_MISS when the primary ray misses */
  float primary_t;
  uint32_t bounce_prim;      /* RDN_MISS when no bounce hit */
  float bounce_t;
  uint32_t primary_flags;    /* bit 0: primary hit */
  uint32_t light;            /* 0 no shadow ray, 1 light visible, 2 occluded */
  float direct;              /* max(0, n.l)/|L|^2 when visible, else 0 */
  uint32_t primary_instance; /* instance slot of the primary hit */
} rdn_pixel_result;

typedef struct rdn_wavefront_desc {
  rdn_camera camera;
  float light[3];
  uint32_t sample_index;     /* seeds the bounce sampler: xxhash32(px, py, 3*sample_index) */
  uint32_t tlas_uniform;
  uint32_t traversal;        /* RDN_TRAVERSAL_* */
  uint32_t block_size;       /* 0 = 64 */
  rdn_pixel_result* out;     /* device, width*height records */
  void* scratch;             /* device, >= rdn_wavefront_scratch_size() bytes, 256-byte aligned */
  size_t scratch_bytes;
  uint32_t* ray_counts;      /* device, nullable: [primary, shadow, bounce] rays traced */
  uint32_t phases;           /* 0 = both; bit 0: primary kernel (raygen, trace, shade, enqueue),
                                bit 1: secondary kernel (shadow + bounce queues of the last primary run) */
  uint32_t refill;           /* secondary schedule of the ordered walks: 0 = each warp traces 32 queued
                                rays together; k in 1..32 = each lane keeps its own traversal state and
                                a warp takes new rays whenever k lanes are idle (dynamic fetch) */
  uint32_t local_stack;      /* ordered walks: 1 = traversal stacks in the threads' local memory (L1)
                                instead of shared memory, for trees whose stack fits 64 entries */
  uint32_t register_tier;    /* local-stack kernels: 0 = 64 registers per thread, 1 = 72 (no spills,
                                fewer resident warps), 2 = 56 (more warps, more spills) */
  uint32_t speculation;      /* ordered walks: a lane holding a leaf keeps descending while more than
                                this many lanes of its warp still look for one (0 = until all have one) */
  uint32_t row_offset;       /* a band of a taller frame: camera.height rows starting at row_offset of a */
  uint32_t frame_height;     /* frame of frame_height rows (0 = camera.height: the whole frame). Camera
                                rays and samplers are those of the whole frame's rows, so bands that
                                tile a frame (one per GPU) give exactly its pixel records; out holds
                                the band's width x camera.height records */
} rdn_wavefront_desc;

/* Scratch size for the secondary-ray queues of a width x height launch. */
rdn_status rdn_wavefront_scratch_size(uint32_t width, uint32_t height, size_t* bytes);

/* RayTracingEncoderProvider::trace_ray (api/backend.rs:48-56) running the
 * fixed pipeline of the path tracer's first bounce
 * (feature/path_tracing/ray_gen.rs, ray_hit.rs): pinhole primary ray, closest
 * hit, one ACCEPT_FIRST_HIT_AND_END_SEARCH shadow ray over [EPSILON, light
 * distance] and one cosine-weighted diffuse bounce over [EPSILON, f32::MAX]
 * from offset_ray_hit origins. Two kernels, stream-ordered, no host sync. */
rdn_status rdn_wavefront_shadow_bounce(rdn_ctx* ctx, const rdn_wavefront_desc* desc, void* stream);

/* ---- batched multi-scene paths ---------------------------------------- */

/* depth_flags of a path result: bits 0..15 = bounce at which the path ended. */
#define RDN_PATH_ESCAPED 0x80000000u  /* ended by a miss: radiance = throughput (sky = 1) */
#define RDN_PATH_ROULETTE 0x40000000u /* ended by Russian roulette: radiance 0 */

typedef struct rdn_path_result {
  float radiance;
  uint32_t depth_flags;
} rdn_path_result;

/* Diffuse paths over many scenes at once: every ray carries its own index into
 * the bound TLAS list (the reference's payload tlas_idx, traverse_cpu.rs:63),
 * so all scenes share one persistent launch per bounce. Per bounce k of ray i:
 * closest hit; a miss writes radiance = throughput; a hit at k == max_bounces
 * writes 0; otherwise the sampler xxhash32(i, k, seed) gives a cosine bounce
 * around the facing geometric normal from an offset_ray_hit origin with
 * throughput *= albedo, and from bounce rr_start on the path survives with
 * probability rr_survive (throughput /= rr_survive). */
typedef struct rdn_path_desc {
  const rdn_ray* rays;          /* device, primary rays */
  const uint32_t* tlas_idx;     /* device, nullable: per-ray TLAS index */
  uint32_t count;
  uint32_t tlas_uniform;        /* used when tlas_idx is NULL */
  uint32_t max_bounces;         /* <= 16 */
  uint32_t rr_start;
  float albedo;
  float rr_survive;
  uint32_t seed;
  uint32_t traversal;           /* RDN_TRAVERSAL_* */
  uint32_t block_size;          /* 0 = 64 */
  uint32_t sort_key;            /* RDN_SORT_*: regroup each bounce's rays before tracing */
  rdn_path_result* out;         /* device, count entries */
  void* scratch;                /* device, >= rdn_paths_scratch_size() bytes, 256-byte aligned */
  size_t scratch_bytes;
  uint32_t* segment_counts;     /* device, nullable: rays traced per bounce (max_bounces + 1) */
  uint32_t refill;              /* schedule of the ordered walks: 0 = each warp traces 32 queued rays
                                   together; k in 1..32 = each lane keeps its own query and a warp takes
                                   new rays whenever k lanes are idle (dynamic fetch) */
  uint32_t local_stack;         /* ordered walks, batch schedule: 1 = traversal stacks in local memory */
  uint32_t speculation;         /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc */
} rdn_path_desc;

/* Ray-sort keys (stable radix sort of each queue before its bounce). */
#define RDN_SORT_NONE 0u
#define RDN_SORT_SCENE_OCTANT 1u        /* (TLAS index, direction octant) */
#define RDN_SORT_SCENE_OCTANT_CELL 2u   /* ... plus a 12-bit Morton cell of the origin in the scene box */

rdn_status rdn_paths_scratch_size(uint32_t count, uint32_t max_bounces, uint32_t sort_key, size_t* bytes);

/* Stream-ordered: one counter reset and max_bounces + 1 persistent launches;
 * queue sizes stay on the device (no host synchronisation). Replaces the
 * reference's per-round task polling of the path tracer
 * (feature/path_tracing/mod.rs:127-235, task_group.rs:176-278). */
rdn_status rdn_trace_paths(rdn_ctx* ctx, const rdn_path_desc* desc, void* stream);

/* The same launches captured once into an executable CUDA graph; the
 * descriptor's pointers and sizes are baked in. Launch it any number of times. */
typedef struct rdn_graph rdn_graph;
rdn_status rdn_trace_paths_graph(rdn_ctx* ctx, const rdn_path_desc* desc, rdn_graph** out);
rdn_status rdn_graph_launch(rdn_graph* graph, void* stream);
rdn_status rdn_graph_destroy(rdn_graph* graph);

/* ---- differentiable closest hit (frozen visibility) ------------------ */

/* Loss = sum over rays of (value - target)^2, value = the hit triangle's vertex
 * attribute interpolated with the barycentrics (1-u-v, u, v) of the hit, which
 * the traversal finds with the reference's test and these kernels re-solve in
 * float-float (f32 FMA) arithmetic for accuracy at grazing angles; misses add
 * nothing. Vertices are those of the built vertex array (all geometries'
 * positions in creation order, rdn_get_built_array(..., 10, ...)). */
typedef struct rdn_attr_loss_desc {
  const rdn_ray* rays;          /* device */
  uint32_t count;
  uint32_t tlas_uniform;
  const float* attributes;      /* device, one per built vertex */
  const float* targets;         /* device, one per ray; NULL = 0 */
  float* ray_value;             /* device, nullable: interpolated attribute per ray (forward) */
  float* ray_loss;              /* device, nullable: per-ray loss (forward) */
  double* loss_sum;             /* device, nullable: loss added here (forward; not reset) */
  float* grad_vertices;         /* device, 4 per built vertex: dL/dx, dL/dy, dL/dz, dL/dattr;
                                   accumulated (adjoint; the caller zeroes it) */
  float* grad_ray_origin;       /* device, nullable: 3 per ray (adjoint) */
  float* grad_ray_direction;    /* device, nullable: 3 per ray (adjoint) */
  float grad_scale;             /* upstream gradient of the loss sum (adjoint), usually 1 */
  uint32_t traversal;           /* RDN_TRAVERSAL_* */
  uint32_t block_size;          /* 0 = 64 */
  uint32_t from_record;         /* adjoint: 1 = differentiate the hits recorded by the forward in
                                   hit_tri / hit_inst instead of tracing the rays again */
  uint32_t* hit_tri;            /* device, nullable: built triangle of each ray's hit, RDN_MISS (forward) */
  uint32_t* hit_inst;           /* device, nullable: TLAS instance slot of each ray's hit (forward) */
  uint32_t local_stack;         /* ordered walks: 1 = traversal stacks in local memory */
  uint32_t speculation;         /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc */
} rdn_attr_loss_desc;

/* Forward: trace, interpolate, loss. Extends the reference's closest-hit query
 * (traverse_cpu.rs:52-245) with a differentiable attribute read-out. */
rdn_status rdn_attr_loss_forward(rdn_ctx* ctx, const rdn_attr_loss_desc* desc, void* stream);
/* Adjoint at frozen visibility: re-traces every ray (the hit is recomputed, not
 * stored) or, with from_record, takes the hits the forward wrote to hit_tri /
 * hit_inst; then scatters gradients with respect to vertex positions and
 * attributes and writes per-ray gradients with respect to origin and direction
 * (object space of the hit instance). */
rdn_status rdn_attr_loss_adjoint(rdn_ctx* ctx, const rdn_attr_loss_desc* desc, void* stream);

/* Differentiable hit query: the closest hit's distance t (the parameter along
 * the ray's direction as given, which is the reference's reported distance,
 * traverse_cpu.rs:157), its barycentrics u, v (weights of vertices 1 and 2,
 * geometry/mod.rs:144-154) and the interpolated vertex attribute
 * value = (1-u-v) a0 + u a1 + v a2 of the triangle that the traversal finds,
 * all re-solved on that triangle in float-float (f32 FMA) arithmetic, so they
 * can differ from rdn_trace's reference-formula values in the last bits, and
 * by more for rays that graze the triangle. The adjoint takes the caller's
 * upstream gradients of (t, u, v, value) per ray and returns, at frozen
 * visibility, the gradients with respect to the vertex positions (object
 * space of each BLAS, accumulated), the vertex attributes (accumulated), and
 * each ray's origin and direction (world space; the instance transform's
 * linear part is assumed affine). Misses write (tmax, 0, 0, 0) and get zero
 * gradients. No counterpart in the reference: the differentiable form of its
 * closest-hit query (traverse_cpu.rs:52-245). */
typedef struct rdn_hit_diff_desc {
  const rdn_ray* rays;          /* device */
  uint32_t count;
  uint32_t tlas_uniform;
  const float* attributes;      /* device, nullable: one per built vertex; NULL: value = 0, no attribute gradient */
  float* hit;                   /* device, nullable: 4 per ray, (t, u, v, value) (forward) */
  uint32_t* hit_tri;            /* device, nullable: built triangle of each ray's hit, RDN_MISS (forward) */
  uint32_t* hit_inst;           /* device, nullable: TLAS instance slot of each ray's hit (forward) */
  const float* grad_hit;        /* device: 4 per ray, (dL/dt, dL/du, dL/dv, dL/dvalue) (adjoint) */
  float* grad_vertices;         /* device: 4 per built vertex, (dL/dx, dL/dy, dL/dz, dL/dattr); accumulated
                                   (adjoint; the caller zeroes it) */
  float* grad_ray_origin;       /* device, nullable: 3 per ray (adjoint) */
  float* grad_ray_direction;    /* device, nullable: 3 per ray (adjoint) */
  uint32_t traversal;           /* RDN_TRAVERSAL_* (| RDN_INTERSECT_WATERTIGHT) */
  uint32_t block_size;          /* 0 = 64 */
  uint32_t from_record;         /* adjoint: 1 = differentiate the hits the forward recorded in hit_tri /
                                   hit_inst instead of tracing the rays again */
  uint32_t local_stack;         /* ordered walks: 1 = traversal stacks in local memory */
  uint32_t speculation;         /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc */
} rdn_hit_diff_desc;

rdn_status rdn_hit_diff_forward(rdn_ctx* ctx, const rdn_hit_diff_desc* desc, void* stream);
rdn_status rdn_hit_diff_adjoint(rdn_ctx* ctx, const rdn_hit_diff_desc* desc, void* stream);

/* Differentiable paths over many scenes: every path is a primary ray (with its
 * own index into the bound TLAS list) followed by up to segments-1 cosine
 * bounces generated like rdn_trace_paths's (facing normal, offset_ray_hit
 * origin, sampler xxhash32(path, segment, seed), no roulette). Each segment's
 * hit adds (value - target)^2 with the attribute interpolation above; a
 * missed segment (and every later one) has value 0. The adjoint recomputes all
 * hits by tracing each path again and treats each segment's ray as fixed:
 * gradients flow to the vertices of every hit triangle, not through the bounce
 * directions. */
typedef struct rdn_attr_path_desc {
  const rdn_ray* rays;          /* device, one primary ray per path */
  const uint32_t* tlas_idx;     /* device, nullable: per-path TLAS index */
  uint32_t count;
  uint32_t tlas_uniform;
  uint32_t segments;            /* 1..8: primary + bounces */
  uint32_t seed;
  const float* attributes;      /* device, one per built vertex */
  const float* targets;         /* device, segments per path; NULL = 0 */
  float* values;                /* device, nullable: segments per path (forward) */
  double* loss_sum;             /* device, nullable: loss added here (forward) */
  float* grad_vertices;         /* device, 4 per built vertex, accumulated (adjoint) */
  uint32_t* seg_tri;            /* device, nullable: built triangle index of each segment's hit, RDN_MISS (forward) */
  rdn_ray* seg_rays;            /* device, nullable: the ray of each segment (forward) */
  float grad_scale;
  uint32_t traversal;
  uint32_t block_size;          /* 0 = 64 */
  uint32_t from_record;         /* adjoint: 1 = differentiate the segments recorded by the forward in
                                   seg_tri / seg_inst / seg_rays (a tape) instead of tracing the paths again */
  uint32_t* seg_inst;           /* device, nullable: TLAS instance slot of each segment's hit (forward) */
  uint32_t local_stack;         /* ordered walks: 1 = traversal stacks in local memory */
  uint32_t speculation;         /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc */
} rdn_attr_path_desc;

rdn_status rdn_attr_paths_forward(rdn_ctx* ctx, const rdn_attr_path_desc* desc, void* stream);
rdn_status rdn_attr_paths_adjoint(rdn_ctx* ctx, const rdn_attr_path_desc* desc, void* stream);
/* Forward and adjoint captured once into one executable CUDA graph; each
 * launch zeroes *loss_sum and the gradient buffer (num_vertices entries of 4
 * floats) first. With grad_vertices NULL the graph holds the forward only.
 * The differentiable-path calls of one context share a device work counter:
 * order them on one stream. */
rdn_status rdn_attr_paths_graph(rdn_ctx* ctx, const rdn_attr_path_desc* desc, uint64_t num_vertices,
                                rdn_graph** out);

/* ---- parallel primitives (shader/parallel-compute) ---------------------
 * Stateless, on the calling thread's current device, stream-ordered. Scratch
 * is caller-owned device memory of at least the queried size, 256-byte aligned. */

rdn_status rdn_scan_scratch_size(uint32_t count, size_t* bytes);
/* Prefix sum of u32 (wrapping). inclusive != 0 for an inclusive scan. segment:
 * 0, or a power of two after which an inclusive scan restarts (the reference's
 * workgroup-scoped scan, prefix_scan.rs:39-114; without segments it is the
 * device-wide segmented scan of lib.rs:398-429, with no WG^2 length limit). */
rdn_status rdn_scan_u32(const uint32_t* in, uint32_t* out, uint32_t count, int inclusive, uint32_t segment,
                        void* scratch, size_t scratch_bytes, void* stream);

rdn_status rdn_compact_scratch_size(uint32_t count, size_t* bytes);
/* Stream compaction (stream_compaction.rs:3-45): out receives the values whose
 * flag is non-zero, in order, and zeros after them; *out_count (device) the
 * number kept. */
rdn_status rdn_compact_u32(const uint32_t* values, const uint32_t* flags, uint32_t* out, uint32_t* out_count,
                           uint32_t count, void* scratch, size_t scratch_bytes, void* stream);

rdn_status rdn_radix_sort_scratch_size(uint32_t count, size_t* bytes);
/* Stable LSD radix sort of u32 keys (radix_sort.rs:29-74) on their low
 * key_bits bits (1..32), carrying optional u32 values; in place. */
rdn_status rdn_radix_sort_u32(uint32_t* keys, uint32_t* values, uint32_t count, uint32_t key_bits, void* scratch,
                              size_t scratch_bytes, void* stream);

/* Allocation-free variant of rdn_wavefront_shadow_bounce; it has no
 * counterpart in the reference. For callers that cannot allocate device
 * memory (a host that hands out all device memory from its own budget fixed at
 * start-up, or a foreign-language host that only sees this C ABI): the shadow
 * and bounce queues live in one array compiled into the library, of
 * RDN_WAVEFRONT_STATIC_SCRATCH_BYTES, held on every GPU that loads the library
 * until exit. desc->scratch must be NULL and desc->scratch_bytes 0; launches
 * whose queues do not fit (rdn_wavefront_scratch_size() above the array size,
 * about 466,000 pixels) are rejected with RDN_ERR_INVALID_ARG. The call
 * allocates nothing: it never builds, so a structure created, deleted or bound
 * since its last build is RDN_ERR_NOT_BUILT (call rdn_build first, which
 * allocates). rdn_create looks up the array's device address for its device.
 * Every call reuses the same array: calls that overlap on the GPU race and
 * must be ordered by the caller. */
#define RDN_WAVEFRONT_STATIC_SCRATCH_BYTES (32u * 1024u * 1024u)
rdn_status rdn_wavefront_shadow_bounce_static(rdn_ctx* ctx, const rdn_wavefront_desc* desc, void* stream);

/* ---- device task graph (shader/task-graph) ----------------------------
 * DeviceTaskGraphBuildSource / DeviceTaskGraphExecutor (runtime/mod.rs:54-397)
 * on the GPU: each task group has a pool of max_in_flight * capacity task
 * records plus the fallback record 0, an active list, an empty-index pool and
 * a removed list. The reference's shader futures are EDSL code; here a task's
 * future is one of two built-in programs:
 *   RDN_TASK_PROGRAM_CHAIN  BaseShaderFuture, then n_spawn stages of
 *       .then(spawn a task of spawn_type[k] with self as parent, payload made
 *       by spawn_op[k]), then .map(map_op) (future/mod.rs, then.rs, task.rs,
 *       map.rs). The base future resolves on the task's first poll; a stage
 *       resolves in the poll that reads its finished child.
 *   RDN_TASK_PROGRAM_TRACE  the ray-trace task (trace_task.rs:150-360): its
 *       first poll traverses the trace call in its payload and spawns the
 *       closest-hit or miss task the call names; it resolves when that child
 *       has finished, taking back the child's user payload.
 * All calls are stream-ordered on the given stream except the read-backs,
 * which wait for it. Counts are those of the reference's
 * TaskGraphExecutionStates. */
#define RDN_TASK_MAX_GROUPS 16u
#define RDN_TASK_PROGRAM_CHAIN 0u
#define RDN_TASK_PROGRAM_TRACE 1u
#define RDN_TASK_PROGRAM_EXTERNAL 2u    /* polled by a kernel of the caller's (include/rdn_task.cuh), launched by
                                           the callback given to rdn_task_graph_set_poll */
#define RDN_TASK_SPAWN_ZERO 0u          /* zeroed child payload */
#define RDN_TASK_SPAWN_AO_PRIMARY 1u    /* AO ray generation: payload word 0 = pixel -> camera trace call */
#define RDN_TASK_SPAWN_AO_OCCLUSION 2u  /* AO primary closest hit -> occlusion-ray trace call */
#define RDN_TASK_MAP_NONE 0u
#define RDN_TASK_MAP_AO_ACCUMULATE 1u   /* running average of the child's occlusion into the AO image */
#define RDN_TASK_MAP_STORE_CHILD 2u     /* own user payload <- the child's */
#define RDN_TASK_MAP_STORE_ZERO 3u      /* own user payload <- 0.0 */
#define RDN_TASK_MAP_STORE_ONE 4u       /* own user payload <- 1.0 */
#define RDN_TASK_INIT_ZERO 0u           /* dispatch_init payload: zero */
#define RDN_TASK_INIT_INDEX 1u          /* dispatch_init payload: word 0 = dispatch index */
/* error flags of rdn_task_graph_check_errors */
#define RDN_TASK_ERROR_NO_FREE_SLOT 0x1u  /* a spawn found the group's pool full (the task stays pending) */
#define RDN_TASK_ERROR_ACTIVE_FULL 0x2u   /* an active-list push past capacity was dropped */
#define RDN_TASK_ERROR_REMOVED_FULL 0x4u  /* a removed-list push past capacity was dropped */
#define RDN_TASK_ERROR_LOOKBACK 0x8u      /* a compaction tile gave up waiting for its predecessor's count */

/* Trace-call payload words of TRACE tasks and of the closest-hit / miss tasks
 * they spawn: [0..7] origin xyz, tmin, direction xyz, tmax; [8] ray flags;
 * [9] cull mask; [10] TLAS index; [11] closest-hit group; [12] miss group
 * (0xFFFFFFFF none); [13..15] user payload. Closest-hit payloads add [16]
 * built triangle, [17] instance slot, [18] t, [19] u, [20] v, [21] hit kind,
 * [22] geometry index, [23] primitive index. */
typedef struct rdn_task_group_desc {
  uint32_t program;        /* RDN_TASK_PROGRAM_* */
  uint32_t max_in_flight;  /* >= 1 */
  uint32_t payload_words;  /* 1..32 u32 words (TRACE: >= 16) */
  uint32_t n_spawn;        /* CHAIN: 0..4 spawn stages */
  uint32_t spawn_type[4];  /* task group of each stage's child */
  uint32_t spawn_op[4];    /* RDN_TASK_SPAWN_* */
  uint32_t map_op;         /* RDN_TASK_MAP_* */
} rdn_task_group_desc;

/* Environment of the trace and AO programs, and the descriptor of an AO
 * frame: the reference's ray-traced AO renderer (feature/ao.rs). Camera ray
 * of pixel (x, y): uv = (x, y) / size + jitter / size with the jitter drawn
 * from xxhash32(x, y, sample_count), target = view_projection_inv applied to
 * ndc (2u-1, 1-2v, 1, 1), direction = normalize(target - camera_position);
 * CULL_BACK_FACING over [f32::EPSILON, f32::MAX]. A hit spawns one
 * ACCEPT_FIRST_HIT_AND_END_SEARCH occlusion ray over [0.01, 100] from the hit
 * point along tbn(shading normal) * cosine_hemisphere(hammersley(sample_count,
 * 256)); the pixel's payload is 0 when it hits and 1 otherwise (1 too when the
 * camera ray misses). The RGBA8 texel becomes
 * (old * sample_count + payload) / (sample_count + 1) while sample_count < 256. */
typedef struct rdn_ao_desc {
  float view_projection_inv[16];  /* Mat4 in the reference's memory order */
  float camera_position[3];
  uint32_t width, height;
  uint32_t sample_count;          /* samples already averaged into image */
  uint32_t tlas_uniform;
  uint32_t traversal;             /* RDN_TRAVERSAL_* */
  const float* normals;           /* device, nullable: 3 per built vertex (shading normals) */
  uint8_t* image;                 /* device, RGBA8 unorm, width * height texels, 4-byte aligned */
  uint32_t sbt_closest[2];        /* task graphs: closest-hit group of the camera and the occlusion ray */
  uint32_t sbt_miss;              /* task graphs: miss group of both rays */
  uint32_t block_size;            /* rdn_ao_render: threads per block, 32, 64 or 128 (0 = 128) */
  uint32_t* ray_counts;           /* device, nullable: [camera, occlusion] rays traced, added to */
  uint32_t* sample_counter;       /* device, nullable: when set, the frame reads its sample index from
                                     here instead of sample_count and adds one to it at its end, so
                                     that a captured frame (rdn_ao_capture) advances by itself */
  uint32_t speculation;           /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc
                                     (the fused kernel and the task graph's trace programs) */
} rdn_ao_desc;

typedef struct rdn_task_graph rdn_task_graph;
rdn_status rdn_task_graph_create(rdn_ctx* ctx, const rdn_task_group_desc* groups, uint32_t count, uint32_t capacity,
                                 void* stream, rdn_task_graph** out);
rdn_status rdn_task_graph_destroy(rdn_task_graph* graph);
/* dispatch_allocate_init_task (runtime/mod.rs:199-260): count root tasks, no parent. */
rdn_status rdn_task_graph_dispatch_init(rdn_task_graph* graph, uint32_t group, uint32_t count, uint32_t init_op,
                                        void* stream);
/* execute (runtime/mod.rs:357-397): rounds x (every group in order: prepare,
 * poll, compact). env: NULL when no group runs a TRACE program or an AO
 * operation; without AO operations only its traversal and tlas_uniform
 * fields are read. */
rdn_status rdn_task_graph_execute(rdn_task_graph* graph, uint32_t rounds, const rdn_ao_desc* env, void* stream);
/* read_back_execution_states: wake, sleep_or_finished and empty counts per
 * group (arrays of the graph's group count); waits for the stream. */
rdn_status rdn_task_graph_states(rdn_task_graph* graph, uint32_t* wake, uint32_t* sleep_or_finished,
                                 uint32_t* empty, void* stream);
/* debug_execution for one group: active list, empty pool (each up to the
 * group's max_in_flight * capacity entries) and the state of every record
 * (capacity + 1 entries; host arrays); waits for the stream. */
rdn_status rdn_task_graph_debug(rdn_task_graph* graph, uint32_t group, uint32_t* active, uint32_t* n_active,
                                uint32_t* empty, uint32_t* n_empty, uint32_t* task_states, void* stream);
rdn_status rdn_task_graph_check_errors(rdn_task_graph* graph, void* stream, uint32_t* flags);
/* Poll of an RDN_TASK_PROGRAM_EXTERNAL group: the executor calls fn once per
 * round where it would launch a built-in poll, with the device graph table,
 * the group, its max_in_flight * capacity and the stream (captures included);
 * fn launches the caller's poll kernel (rdn_task::launch in rdn_task.cuh) and
 * returns RDN_OK. */
typedef rdn_status (*rdn_task_poll_fn)(const void* graph_device, uint32_t group, uint32_t group_capacity,
                                       void* stream, void* user);
rdn_status rdn_task_graph_set_poll(rdn_task_graph* graph, uint32_t group, rdn_task_poll_fn fn, void* user);
/* dispatch_init of `count` root tasks in `group`, then rounds until no group
 * holds an active task, at most max_rounds, captured into an executable CUDA
 * graph (rdn_graph_launch / rdn_graph_destroy). The loop is a conditional node
 * that the device ends after the first round that leaves no task active: no
 * host round trip and no idle rounds. The graph is then empty, unless a spawn
 * found a pool full and its parent waits for ever (as in the reference). env is baked in, as for
 * rdn_task_graph_execute; a graph that traces needs the structure built. The
 * task graph, the built structure and the buffers env names must outlive the
 * captured graph. */
rdn_status rdn_task_graph_capture(rdn_task_graph* graph, uint32_t group, uint32_t count, uint32_t init_op,
                                  uint32_t max_rounds, const rdn_ao_desc* env, rdn_graph** out);

/* The reference's AO pipeline as a task graph (feature/ao.rs:162-313 on
 * trace_ray): group 0 ray-trace task (max_in_flight 2), 1 ray generation,
 * 2 primary closest hit, 3 occlusion closest hit, 4 miss; capacity = the
 * frame rounded up to whole 4x8 pixel tiles (4 wide, 8 tall). rdn_ao_render_graph dispatches
 * one ray-generation task per pixel of those tiles (32 consecutive tasks per
 * tile, so that a warp traces neighbouring pixels; tasks past the frame
 * resolve without tracing) and runs 8 rounds (the reference's
 * execution_round_hint). */
rdn_status rdn_ao_pipeline_create(rdn_ctx* ctx, uint32_t width, uint32_t height, void* stream,
                                  rdn_task_graph** out);
rdn_status rdn_ao_render_graph(rdn_task_graph* graph, const rdn_ao_desc* desc, void* stream);
/* The same frame as one fused kernel, one thread per pixel. */
rdn_status rdn_ao_render(rdn_ctx* ctx, const rdn_ao_desc* desc, void* stream);
/* One AO frame captured into an executable CUDA graph: the fused kernel
 * (pipeline NULL) or the task-graph pipeline's dispatch and rounds until the
 * pipeline is empty (at most 8, ended on the device). The
 * descriptor is baked in; with desc->sample_counter set, each rdn_graph_launch
 * draws the next sample. The context's structure must stay built and the
 * buffers alive while the graph is in use. */
rdn_status rdn_ao_capture(rdn_ctx* ctx, rdn_task_graph* pipeline, const rdn_ao_desc* desc, rdn_graph** out);

/* ---- Path tracing: DeviceReferencePathTracingRenderer::render
 * (scene/rendering/gpu-ray-tracing/src/feature/path_tracing/mod.rs:127-235) ----
 * One sample per pixel into a headless RGBA8 unorm buffer (the reference's
 * radiance texture, frame_state.rs:12-20):
 *   camera ray as rdn_ao_desc (xxhash32(x, y, sample_count) jitter,
 *     view_projection_inv, camera_position), CULL_BACK_FACING over
 *     [f32::EPSILON, f32::MAX], TLAS tlas_uniform        ray_gen.rs:95-161
 *   closest hit: light index floor(next * count) from the sampler
 *     xxhash32(x, y, 2 * sample_count), pmf 1 / count; a directional light
 *     lights from -direction at distance f32::MAX with radiance illuminance and
 *     pdf 1; its shadow ray ACCEPT_FIRST_HIT_AND_END_SEARCH over
 *     [f32::EPSILON, f32::MAX] from offset_ray_hit(hit, geometric normal)
 *                                                        ray_hit.rs:12-57, lighting_sampler.rs:86-125,
 *                                                        lighting_bridge.rs:213-258, ray_util.rs:5-40
 *   BRDF sample from xxhash32(x, y, 3 * sample_count): Lambertian + GGX /
 *     Smith-GGX-correlated / Schlick mixed by mix(0.2, 1, max f0), alpha =
 *     perceptual roughness^2                             ray_hit.rs:58-102, surface_bridge.rs:171-224
 *   sampled radiance |n.l| * bsdf(v, l) * light radiance / pdf (0 when occluded)
 *   ray generation: a miss adds throughput * miss radiance and ends the path;
 *     a hit multiplies throughput by cos * brdf / max(pdf, 1e-4) and adds
 *     throughput * sampled radiance; pdf == 0 ends it; at most max_path_depth
 *     core rays                                          ray_gen.rs:101-150
 *   tone map, then texel = (old * sample_count + ldr) / (sample_count + 1),
 *     alpha 1                                            ray_gen.rs:160-177, tonemap.rs:53-200
 * Every bounce of one path draws the same random numbers, as the reference's
 * closest-hit shader seeds its samplers by pixel and sample count alone. A
 * material's emissive channel reaches no pixel, as in the reference (its ray
 * generation adds the surface radiance of misses only, which is zero). atan,
 * sin, cos and pow are fixed polynomial evaluations (the oracle computes the
 * same), not the GPU backend's builtins. */
#define RDN_TONE_MAP_NONE 0u
#define RDN_TONE_MAP_LINEAR 1u
#define RDN_TONE_MAP_REINHARD 2u
#define RDN_TONE_MAP_CINEON 3u
#define RDN_TONE_MAP_ACES_FILMIC 4u  /* the reference's default (ToneMap::new, exposure 1) */
#define RDN_PT_BACKGROUND_SOLID 0u   /* PTRayMissCtx::Solid: background_color */
#define RDN_PT_BACKGROUND_TEST 1u    /* PTRayMissCtx::Test: 0.7 for direction.y > 0, else 0.3 */
#define RDN_PT_BACKGROUND_ENV_CUBE 2u /* PTRayMissCtx::EnvCube: env_cube sampled along env_transform applied to
                                        the direction (M (d, 1) / w), times env_intensity: the major axis's face
                                        (ties x, y, z), bilinear over texel centres clamped to the face, level 0
                                        (f32 weights, no filtering across faces) */
#define RDN_PT_MAX_PATH_DEPTH 3u     /* the reference's MAX_RAY_DEPTH (path_tracing/mod.rs:80) */
#define RDN_PT_SCHEDULE_PIXEL 0u     /* one thread per pixel, warps over 4x8 tiles */
#define RDN_PT_SCHEDULE_REFILL 1u    /* persistent warps; a lane whose path ends takes the next pixel (the
                                        frame uses the context's work counter: one frame in flight per context) */
#define RDN_PT_SCHEDULE_WAVEFRONT 2u /* one pass per ray kind and depth over queues of paths, the path state in
                                        the caller's scratch (rdn_pt_scratch_size): warps trace camera, bounce
                                        or shadow rays only */

/* DirectionalLightStorage's illuminance and direction (the direction light travels). */
typedef struct rdn_pt_directional_light {
  float illuminance[3];
  float direction[3];
} rdn_pt_directional_light;

/* The channels PhysicalShading::construct_shading_impl reads
 * (lighting/transport/src/surface/microfacet/device/direct_lighting.rs:14-59).
 * workflow 0 (metallic): albedo = base_color (1 - metallic), f0 = base_color
 * metallic + 0.16 reflectance^2 (1 - metallic). workflow 1 (specular): f0 =
 * specular, albedo = base_color (1 - max channel of specular). A pixel whose
 * instance has no material uses the reference's defaults (base colour 0.5,
 * roughness 0.5, metallic 0, reflectance 0.5). */
typedef struct rdn_pt_material {
  float base_color[3];
  float perceptual_roughness;
  float emissive[3];
  float metallic;
  float specular[3];
  float reflectance;
  uint32_t workflow;
  uint32_t reserved[3];
} rdn_pt_material;

typedef struct rdn_pt_desc {
  float view_projection_inv[16];  /* Mat4 in the reference's memory order */
  float camera_position[3];
  uint32_t width, height;
  uint32_t sample_count;          /* PTConfig.current_sample_count: samples already averaged into image */
  uint32_t max_path_depth;        /* PTConfig.max_path_depth (RDN_PT_MAX_PATH_DEPTH in the reference) */
  uint32_t tlas_uniform;
  uint32_t traversal;             /* RDN_TRAVERSAL_* */
  uint32_t tone_map;              /* RDN_TONE_MAP_* */
  float exposure;
  uint32_t background;            /* RDN_PT_BACKGROUND_* */
  float background_color[3];
  const rdn_pt_directional_light* lights; /* device, light_count entries (nullable when 0) */
  uint32_t light_count;
  uint32_t material_count;
  const rdn_pt_material* materials;       /* device, nullable: every instance takes the default material */
  const uint32_t* sm_to_material;         /* device, nullable: material of each instance custom index
                                             (NULL: the custom index itself); out of range -> default */
  uint32_t sm_count;                      /* entries of sm_to_material */
  uint32_t block_size;                    /* 32, 64 or 128 (0 = 128) */
  const float* normals;           /* device, nullable: 3 per built vertex (shading normals) */
  uint8_t* image;                 /* device, RGBA8 unorm, width * height texels, 4-byte aligned */
  float* radiance;                /* device, nullable, 16-byte aligned: per pixel the sample's HDR
                                     radiance (x, y, z) and the core rays of its path (w) */
  uint32_t* ray_counts;           /* device, nullable: [core, shadow] rays traced, added to */
  uint32_t schedule;              /* RDN_PT_SCHEDULE_*: how paths map to threads (no pixel changes) */
  uint32_t register_tier;         /* refill and wavefront schedules, ordered walks with local stacks:
                                     register budget per thread, 0 = compiler's choice, 1 = at most 96,
                                     2 = at most 64 (no pixel changes) */
  void* scratch;                  /* device, 256-byte aligned, >= rdn_pt_scratch_size(): wavefront schedule */
  size_t scratch_bytes;
  const float* env_cube;          /* device, 16-byte aligned: RDN_PT_BACKGROUND_ENV_CUBE's six faces (+X, -X,
                                     +Y, -Y, +Z, -Z), each env_size rows (t) of env_size RGBA f32 texels (s) */
  uint32_t env_size;
  float env_transform[16];        /* IblShaderInfoForBackground.transform, Mat4 in the reference's memory order */
  float env_intensity;            /* IblShaderInfoForBackground.intensity */
  uint32_t* sample_counter;       /* device, nullable: when set, the frame reads its sample index from here
                                     instead of sample_count and adds one to it at its end, so that a
                                     captured frame (rdn_pt_capture) advances by itself */
  uint32_t speculation;           /* ordered walks: leaf postponement threshold, as in rdn_wavefront_desc */
} rdn_pt_desc;

/* Scratch of the wavefront schedule for a width x height frame: 112 B of path
 * state and two 4 B queue entries per pixel. */
rdn_status rdn_pt_scratch_size(uint32_t width, uint32_t height, size_t* bytes);
rdn_status rdn_path_tracing_render(rdn_ctx* ctx, const rdn_pt_desc* desc, void* stream);
/* One path-traced sample captured into an executable CUDA graph: the
 * descriptor is baked in; with desc->sample_counter set each rdn_graph_launch
 * draws the next sample (PTRenderState::next_sample on the device). The
 * context's structure must stay built and the buffers alive while the graph
 * is in use; one replay at a time per context with the refill schedule. */
rdn_status rdn_pt_capture(rdn_ctx* ctx, const rdn_pt_desc* desc, rdn_graph** out);

#ifdef __cplusplus
}
#endif

#endif /* RDN_H */
