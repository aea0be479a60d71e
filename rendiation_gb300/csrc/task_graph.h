// Device task graph (the reference's shader/task-graph crate): task groups
// with pools, spawn / poll / wake, bump lists and active-list compaction, run
// as CUDA kernels. The state machine follows the reference:
//   task states, pool record              runtime/task_pool.rs:5-16,118-139,160-190
//   spawn / wake / poll / cleanup         runtime/task_group.rs:410-515
//   poll finalisation (finish, wake parent, sleep)
//                                         runtime/task_group.rs:130-165
//   execute round per group: prepare (commit + drain removed -> empty),
//   poll, commit + compaction             runtime/task_group.rs:175-278
//   bump allocate / deallocate / commit / drain
//                                         bump_allocator.rs:83-316
//   compaction keeps NOT_FINISHED_WAKEN, turns GO_TO_SLEEP into SLEEP
//                                         runtime/dispatch_compact.rs:44-116
//   pool init (empty pool 1..size, fallback task 0)
//                                         runtime/task_group.rs:351-397
//   execution states                      runtime/mod.rs:262-325
//
// Task programs replace the reference's shader futures, which are EDSL code:
// CHAIN is BaseShaderFuture, then k times .then(spawn a task with self as
// parent), then .map (future/mod.rs:118-188, then.rs, task.rs, map.rs), with
// built-in payload and map operations; TRACE is the ray-trace task
// (backend/wavefront_compute/trace_task.rs:150-360).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "trace_kernels.h"

namespace rdn {

constexpr uint32_t kTaskMaxGroups = 16;
constexpr uint32_t kTaskMaxSpawns = 4;
constexpr uint32_t kTaskLocalWords = 8;
constexpr uint32_t kTaskMaxPayloadWords = 32;

// Task states (runtime/task_pool.rs:118-139).
enum : uint32_t {
  TASK_NOT_EXIST = 0,
  TASK_NOT_FINISHED_WAKEN = 1,
  TASK_GO_TO_SLEEP = 2,
  TASK_NOT_FINISHED_SLEEP = 3,
  TASK_FINISHED = 4,
};
constexpr uint32_t TASK_NO_PARENT = 0xFFFFFFFFu;
// future/task.rs:11-12
constexpr uint32_t TASK_HANDLE_UNINIT = 0xFFFFFFFEu;
constexpr uint32_t TASK_HANDLE_RESOLVED = 0xFFFFFFFFu;
// trace_task.rs:107-108
constexpr uint32_t TRACE_SUB_NOT_SPAWNED = 0xFFFFFFFFu;
constexpr uint32_t TRACE_SUB_SPAWN_FAILED = 0xFFFFFFFEu;

// error word bits
constexpr uint32_t TASK_ERR_NO_FREE_SLOT = 0x1;  // spawn found the empty pool exhausted
constexpr uint32_t TASK_ERR_ACTIVE_FULL = 0x2;   // an active-list push past the list's capacity
constexpr uint32_t TASK_ERR_REMOVED_FULL = 0x4;  // a removed-list push past its capacity
constexpr uint32_t TASK_ERR_LOOKBACK = 0x8;      // a compaction tile waited past its limit for a predecessor

// Task local words (the reference's per-task future state): [0] base future
// polled once, [1..4] child handles of the chain's spawn stages, [5] trace
// sub-task group, [6] trace sub-task id, [7] trace has_terminated.
// Programs
// EXTERNAL: polled by a kernel compiled outside librdn (include/rdn_task.cuh)
// that a host callback launches.
enum : uint32_t { TASK_PROGRAM_CHAIN = 0, TASK_PROGRAM_TRACE = 1, TASK_PROGRAM_EXTERNAL = 2 };
// Host callback that launches an external program's poll kernel on `stream`
// for group `group` of the device graph table `graph_device` (returns 0 on success).
using ExternalPoll = int32_t (*)(const void* graph_device, uint32_t group, uint32_t group_capacity, void* stream,
                                 void* user);
// payload of a spawned child
enum : uint32_t {
  TASK_SPAWN_ZERO = 0,          // zeroed payload
  TASK_SPAWN_AO_PRIMARY = 1,    // ray-gen pixel -> camera ray trace call (feature/ao.rs:193-213)
  TASK_SPAWN_AO_OCCLUSION = 2,  // primary closest hit -> occlusion ray trace call (feature/ao.rs:244-276)
};
// operation applied when a chain resolves
enum : uint32_t {
  TASK_MAP_NONE = 0,
  TASK_MAP_AO_ACCUMULATE = 1,    // progressive average into the AO image (feature/ao.rs:215-237)
  TASK_MAP_STORE_CHILD = 2,      // own user payload <- the child's (feature/ao.rs:278)
  TASK_MAP_STORE_ZERO = 3,       // own user payload <- 0.0 (occluded; feature/ao.rs:288)
  TASK_MAP_STORE_ONE = 4,        // own user payload <- 1.0 (miss; feature/ao.rs:296)
};
// init payloads of dispatch_allocate_init_task
enum : uint32_t { TASK_INIT_ZERO = 0, TASK_INIT_INDEX = 1 };

// Payload layout of trace-call tasks (TRACE, and the closest / miss tasks it
// spawns), in u32 words:
//   [0..7]  ray: origin xyz, tmin, direction xyz, tmax (world space)
//   [8] ray flags  [9] cull mask  [10] TLAS index  [11] closest-hit group
//   [12] miss group (0xFFFFFFFF = none)
//   [13..15] user payload
//   closest-hit payload only: [16] built triangle  [17] instance slot  [18] t
//   [19] u  [20] v  [21] hit kind  [22] geometry index  [23] primitive index
constexpr uint32_t kTraceCallWords = 16;
constexpr uint32_t kClosestWords = 24;
constexpr uint32_t kTraceUser = 13;

struct ListCtl {
  uint32_t size, bump;
};
// Device-resident control block of a group, 64 B.
struct GroupCtl {
  ListCtl active, removed, empty;
  uint32_t sel;        // which active buffer holds the list
  uint32_t src_sel;    // buffer the running compaction reads
  uint32_t drain_n;    // removed entries the drain copies
  uint32_t drain_off;  // where they go in the empty pool
  uint32_t compact_n;  // committed active size the compaction reads
  uint32_t tile_next;  // next compaction tile to hand out (reset by the drain)
  uint32_t epoch;      // compaction generation: tile descriptors of older ones read as unset
  uint32_t poll_next;  // next active entry a trace poll's warp takes (reset by the drain)
  uint32_t pad[2];
};
static_assert(sizeof(GroupCtl) == 64, "64 B control block");

struct TaskGroupDev {
  uint32_t* state;
  uint32_t* parent_type;
  uint32_t* parent_index;
  uint32_t* payload;  // payload_words x (cap + 1), word-major
  uint32_t* locals;   // kTaskLocalWords x (cap + 1), word-major
  uint32_t* active[2];
  uint32_t* removed;
  uint32_t* empty;
  unsigned long long* tile_desc;  // compaction tile descriptors: epoch (30 bits) | status (2) | count (32)
  GroupCtl* ctl;
  uint32_t cap;  // max_in_flight * capacity; the pool holds cap + 1 records
  uint32_t payload_words;
  uint32_t program, n_spawn, map_op;
  uint32_t spawn_type[kTaskMaxSpawns];
  uint32_t spawn_op[kTaskMaxSpawns];
};

struct TaskGraphDev {
  TaskGroupDev g[kTaskMaxGroups];
  uint32_t n_groups;
  uint32_t* error;
};

// Ambient-occlusion environment of the built-in AO operations.
struct AoEnv {
  float vp_inv[16];  // ndc -> world (Mat4, reference memory order)
  float cam[3];      // camera world position
  uint32_t width, height, sample_count, tlas;
  uint32_t sbt_closest[2];  // closest-hit group of ray type 0 (primary) and 1 (occlusion test)
  uint32_t sbt_miss;        // miss group (miss index 0)
  uint8_t* image;           // RGBA8 unorm, width * height texels
  const float* normals;     // per built vertex, 3 floats; NULL = the geometric normal
  const uint32_t* indices;  // built vertex indices
  const float* vertices;    // built vertex positions
  uint32_t n_instances;     // TLAS instance slots
  uint32_t n_triangles;     // built triangles
  uint32_t* ray_counts;     // nullable: [camera, occlusion] rays traced
  const uint32_t* sample_dev;  // nullable: the sample index, read at run time instead of sample_count
  uint32_t block;              // fused kernel: threads per block (32, 64 or 128)
};

// Ray-generation tasks of a w x h AO frame: whole 4x8 pixel tiles, 32 per tile.
__host__ __device__ inline uint32_t ao_dispatch_count(uint32_t w, uint32_t h) {
  return ((w + 3) / 4) * ((h + 7) / 8) * 32;
}

struct TaskGroupDesc {
  uint32_t program = TASK_PROGRAM_CHAIN;
  uint32_t max_in_flight = 1;
  uint32_t payload_words = 1;
  uint32_t n_spawn = 0;
  uint32_t spawn_type[kTaskMaxSpawns] = {0, 0, 0, 0};
  uint32_t spawn_op[kTaskMaxSpawns] = {0, 0, 0, 0};
  uint32_t map_op = TASK_MAP_NONE;
};

// Host side: device memory of all groups, and the launch sequences of the
// reference's executor.
class TaskGraph {
 public:
  ~TaskGraph();
  // The descriptor checks of create(), without a device: "" when valid.
  static std::string validate(const std::vector<TaskGroupDesc>& groups, uint32_t capacity);
  // Validates, allocates and initialises (TaskGroupExecutorResource::init).
  std::string create(const std::vector<TaskGroupDesc>& groups, uint32_t capacity, int sm_count, cudaStream_t st);
  // dispatch_allocate_init_task (runtime/mod.rs:217-260)
  cudaError_t dispatch_init(uint32_t group, uint32_t count, uint32_t init_op, cudaStream_t st);
  // execute (runtime/mod.rs:357-397); trace / AO programs read p and ao.
  cudaError_t execute(uint32_t rounds, const TraceParams* p, int mode, const AoEnv* ao, cudaStream_t st);
  // prepare_execution_and_compact_living_task on every group, then the sizes
  // (runtime/mod.rs:262-325); waits for the stream.
  cudaError_t states(uint32_t* wake, uint32_t* empty, cudaStream_t st);
  // debug_execution (runtime/mod.rs:327-355): compacts, then copies one group's
  // active list, empty pool and task states; waits for the stream.
  cudaError_t debug(uint32_t group, std::vector<uint32_t>& active, std::vector<uint32_t>& empty,
                    std::vector<uint32_t>& task_states, cudaStream_t st);
  cudaError_t read_error(uint32_t* flags, cudaStream_t st);
  void set_external(uint32_t g, ExternalPoll fn, void* user) {
    ext_fn_[g] = fn;
    ext_user_[g] = user;
  }
  // "" when every EXTERNAL group has a poll callback
  std::string check_external() const;
  // Into the stream being captured: rounds until no group holds a task, at
  // most max_rounds, as a WHILE conditional node (the device decides after
  // each round; the host issues nothing per round).
  cudaError_t record_until_empty(uint32_t max_rounds, const TraceParams* p, int mode, const AoEnv* ao,
                                 cudaStream_t capturing);

  uint32_t group_count() const { return dev_.n_groups; }
  uint32_t group_cap(uint32_t g) const { return dev_.g[g].cap; }
  const std::vector<TaskGroupDesc>& groups() const { return desc_; }

 private:
  cudaError_t prepare(uint32_t g, cudaStream_t st);
  cudaError_t compact(uint32_t g, cudaStream_t st);
  cudaError_t bookkeep(uint32_t gc, uint32_t gd, cudaStream_t st);
  cudaError_t poll(uint32_t g, const TraceParams* p, int mode, const AoEnv* ao, cudaStream_t st);

  TaskGraphDev dev_{};
  TaskGraphDev* dev_ptr_ = nullptr;  // device copy of dev_
  std::vector<ExternalPoll> ext_fn_;
  std::vector<void*> ext_user_;
  std::vector<TaskGroupDesc> desc_;
  std::vector<void*> allocs_;
  int sm_count_ = 1;
};

// Fused AO frame (ao.cu): every pixel of a.width x a.height, one launch.
cudaError_t launch_ao(const TraceParams& p, const AoEnv& a, int mode, cudaStream_t st);
// Adds one to a device sample counter (the end of a frame that reads it).
cudaError_t launch_ao_advance(uint32_t* counter, cudaStream_t st);

}  // namespace rdn
