// Device build of the triangle BVH forest: the reference's binned SAH tree
// (content/space/src/bvh/strategy.rs:11-43,202-284 with SAH::new(4); degenerate
// binning falls back to BalanceTree's median split, strategy.rs:66-87 and
// apply.rs:19-45), flattened exactly as NaiveSahBvhSource::build flattens it
// (shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/mod.rs:
// 122-260 for the geometry arrays, :338-386 for the forest, :611-632 for the
// threaded links), plus the two-child, four-child and triangle-record layouts
// of the traversal kernels. The arrays equal the host build's byte for byte.
//
// The reference builds one node at a time, depth first, on one thread. Here
// every geometry's tree is built together, one tree level per round:
//   prepare   each node of the level decides leaf / split (count > bin_size and
//             depth < max_depth, utils.rs:35-37) and claims warp tasks of 256
//             primitives ("chunks") of its range;
//   box       nodes whose box is not known yet (roots, median-split children)
//             reduce their primitives' boxes;
//   stats     per chunk: the 4 centroid buckets on the longest axis of the
//             node box, their counts and boxes, merged into the node;
//   decide    per node: the reference's 3-candidate SAH choice (or the median
//             fallback when 3 buckets are empty), the two children, and each
//             chunk's per-bucket offset inside the node (warp scan);
//   select    median-split nodes run Rust's select_nth_unstable_by
//             restatement on one thread each;
//   scatter   SAH nodes write their primitives in bucket order, stable inside
//             a bucket (warp ballots), then copy the range back.
// Boxes are merged with integer atomics on an order-preserving key of the
// float, so a union does not depend on the order primitives arrive in. The
// reference's pre-order numbering is recovered afterwards from subtree sizes
// (bottom-up) and a top-down pass, and the two-child node / leaf numbering from
// one scan over the pre-order inner-node flags. Compiled with -fmad=false: the
// bucket, area and cost arithmetic must round exactly as the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "device_build.h"
#include "parallel.h"
#include "rust_select.h"

namespace rdn {
namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr uint32_t kChunk = 256;
constexpr uint32_t kBlock = 256;
constexpr uint32_t kWarps = kBlock / 32;
constexpr uint32_t F_BOX_PENDING = 1u, F_ACTIVE = 2u, F_FALLBACK = 4u;

// Order-preserving int key of a float (no NaN reaches a box: boxes start
// empty and grow with NaN-ignoring min/max). -0.0 orders below +0.0.
__host__ __device__ __forceinline__ int key_of(float f) {
#ifdef __CUDA_ARCH__
  const int i = __float_as_int(f);
#else
  int i;
  std::memcpy(&i, &f, 4);
#endif
  return i >= 0 ? i : (i ^ 0x7FFFFFFF);
}
__host__ __device__ __forceinline__ float val_of(int k) {
  const int i = k >= 0 ? k : (k ^ 0x7FFFFFFF);
#ifdef __CUDA_ARCH__
  return __int_as_float(i);
#else
  float f;
  std::memcpy(&f, &i, 4);
  return f;
#endif
}

struct BNode {  // 64 B, one per tree node during the build
  int lo[3], hi[3];   // box as keys
  uint32_t start, end;  // range in the global primitive order
  uint32_t depth, left;  // left child id (right = left + 1), NONE for a leaf
  uint32_t tree, flags;
  uint32_t cbase, nchunks;
  uint32_t pad[2];
};
static_assert(sizeof(BNode) == 64, "64 B build node");

struct LevelCounters {  // one per tree level, zeroed before the first level
  uint32_t chunks, children, big, pad;
};
struct BuildCounters {
  unsigned long long sah, fallback;
  uint32_t bad_index, pad;
};

struct F3 {
  float x, y, z;
};
struct NodeBox {
  F3 lo, hi;
};

__device__ __forceinline__ NodeBox box_of(const BNode& n) {
  return NodeBox{{val_of(n.lo[0]), val_of(n.lo[1]), val_of(n.lo[2])}, {val_of(n.hi[0]), val_of(n.hi[1]), val_of(n.hi[2])}};
}
__device__ __forceinline__ float comp(const F3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ int split_axis(const NodeBox& b) {  // Box3::longest_axis
  const float x = b.hi.x - b.lo.x, y = b.hi.y - b.lo.y, z = b.hi.z - b.lo.z;
  if (x > y) return x > z ? 0 : 2;
  return y > z ? 1 : 2;
}
__device__ __forceinline__ uint32_t bucket_of(float value, float start, float step) {
  // ((value - start) / step).floor() as usize, clamped to the last bucket
  const float f = floorf((value - start) / step);
  const uint32_t b = (f > 0.0f) ? (f >= 4.0f ? 4u : (uint32_t)f) : 0u;
  return b >= 4 ? 3u : b;
}
__device__ __forceinline__ float sah_area(const NodeBox& b) {  // 2 * (w*h + w*d + h*d)
  const float w = b.hi.x - b.lo.x, h = b.hi.y - b.lo.y, d = b.hi.z - b.lo.z;
  return 2.0f * (w * h + w * d + h * d);
}
__device__ __forceinline__ float half_area(const NodeBox& b) {  // collapse order of the four-child layout
  const float w = b.hi.x - b.lo.x, h = b.hi.y - b.lo.y, d = b.hi.z - b.lo.z;
  return w * h + w * d + h * d;
}
__device__ __forceinline__ NodeBox empty_box() {
  return NodeBox{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
}
__device__ __forceinline__ void grow(NodeBox& b, const NodeBox& o) {
  b.lo = {fminf(b.lo.x, o.lo.x), fminf(b.lo.y, o.lo.y), fminf(b.lo.z, o.lo.z)};
  b.hi = {fmaxf(b.hi.x, o.hi.x), fmaxf(b.hi.y, o.hi.y), fmaxf(b.hi.z, o.hi.z)};
}
__device__ __forceinline__ void set_box(BNode& n, const NodeBox& b) {
  n.lo[0] = key_of(b.lo.x);
  n.lo[1] = key_of(b.lo.y);
  n.lo[2] = key_of(b.lo.z);
  n.hi[0] = key_of(b.hi.x);
  n.hi[1] = key_of(b.hi.y);
  n.hi[2] = key_of(b.hi.z);
}

// Centre keys of one axis with the reference's comparator
// (partial_cmp(..).unwrap_or(Less) on the centre coordinate).
struct CentreLess {
  const float* key;
  __host__ __device__ bool operator()(const uint32_t& a, const uint32_t& b) const {
    const float ka = key[a], kb = key[b];
    return ka != ka || kb != kb || ka < kb;  // a NaN on either side compares Less
  }
};

// ---- geometry preparation ----------------------------------------------

// Global vertex indices (BLAS concatenation, naive/mod.rs:155-186), the
// primitive boxes (BuildPrimitive::new, utils.rs:40-66: grow an empty box by
// the 3 vertices) and centres (box centre), SoA centres for the bucket pass.
__global__ void prepare_primitives_kernel(uint32_t N, uint32_t G, const uint32_t* __restrict__ g_prim_start,
                                          const uint32_t* __restrict__ g_vstart, const uint32_t* __restrict__ g_vcount,
                                          const uint32_t* __restrict__ g_indexed, uint32_t* __restrict__ idx,
                                          const float* __restrict__ vtx, float4* __restrict__ pbox,
                                          float* __restrict__ cen, uint32_t* __restrict__ order,
                                          BuildCounters* ctr) {
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = G;  // last g with g_prim_start[g] <= p
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) / 2;
      if (g_prim_start[mid] <= p) lo = mid;
      else hi = mid;
    }
    const uint32_t g = lo, local = p - g_prim_start[g], vs = g_vstart[g], vc = g_vcount[g];
    NodeBox b = empty_box();
    for (int k = 0; k < 3; k++) {
      uint32_t raw = g_indexed[g] ? idx[3 * (size_t)p + k] : 3 * local + k;
      if (raw >= vc) {
        atomicAdd(&ctr->bad_index, 1u);
        raw = 0;
      }
      idx[3 * (size_t)p + k] = vs + raw;
      if (vc) {
        const float* v = vtx + 3 * (size_t)(vs + raw);
        const F3 q = {v[0], v[1], v[2]};
        grow(b, NodeBox{q, q});
      }
    }
    pbox[2 * (size_t)p] = make_float4(b.lo.x, b.lo.y, b.lo.z, 0.0f);
    pbox[2 * (size_t)p + 1] = make_float4(b.hi.x, b.hi.y, b.hi.z, 0.0f);
    cen[p] = (b.lo.x + b.hi.x) * 0.5f;
    cen[N + p] = (b.lo.y + b.hi.y) * 0.5f;
    cen[2 * (size_t)N + p] = (b.lo.z + b.hi.z) * 0.5f;
    order[p] = p;
  }
}

// ---- one tree level -----------------------------------------------------

__device__ __forceinline__ uint32_t warp_inclusive_u32(uint32_t v, uint32_t lane) {
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (uint32_t)o) v += t;
  }
  return v;
}

// Warp-aggregated claim on a counter: all 32 lanes call, each with its own
// amount (0 allowed); one atomic per warp instead of one per lane (a level
// of 250 k nodes would otherwise serialise on the counter's address).
__device__ __forceinline__ uint32_t warp_claim(uint32_t* ctr, uint32_t amount, uint32_t lane) {
  const uint32_t inc = warp_inclusive_u32(amount, lane);
  const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(ctr, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + inc - amount;
}

// Level L holds nodes [lvl[L], lvl[L+1]) of the pool. The bounds live on the
// device: level L's last kernel writes lvl[L+2], so that the host can queue
// several levels without reading anything back. Kernels of an empty level
// (past the last one) find no node and return. Node loops step a whole warp
// at a time (warp-uniform bounds) so that the lanes can aggregate atomics.
__global__ void level_prepare_kernel(const uint32_t* __restrict__ lvl, uint32_t L, uint32_t bin_size,
                                     uint32_t max_depth, BNode* __restrict__ pool, uint32_t* __restrict__ acc_cnt,
                                     int* __restrict__ acc_box, uint32_t* __restrict__ chunk_node,
                                     LevelCounters* lcs) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lb = lvl[L], W = lvl[L + 1] - lb;
  LevelCounters* lc = lcs + L;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < W; i0 += stride) {
    const uint32_t i = i0 + lane;
    uint32_t nch = 0;
    bool active = false;
    if (i < W) {
      BNode& n = pool[lb + i];
      const uint32_t count = n.end - n.start;
      active = n.depth < max_depth && count > bin_size;
      const bool need = active || (n.flags & F_BOX_PENDING);
      nch = need ? (count + kChunk - 1) / kChunk : 0;
      n.flags = (n.flags & ~(F_ACTIVE | F_FALLBACK)) | (active ? F_ACTIVE : 0u);
      n.left = NONE;
      n.nchunks = nch;
    }
    const uint32_t base = warp_claim(&lc->chunks, nch, lane);
    if (i < W) pool[lb + i].cbase = nch ? base : 0u;
    // chunk -> node map: small ranges by their own lane, long ones by the whole warp
    if (nch && nch <= 32)
      for (uint32_t j = 0; j < nch; j++) chunk_node[base + j] = lb + i;
    uint32_t wide = __ballot_sync(0xffffffffu, nch > 32);
    while (wide) {
      const uint32_t src = __ffs(wide) - 1;
      wide &= wide - 1;
      const uint32_t b = __shfl_sync(0xffffffffu, base, src), c = __shfl_sync(0xffffffffu, nch, src);
      for (uint32_t j = lane; j < c; j += 32) chunk_node[b + j] = lb + i0 + src;
    }
    if (active) {
      for (int b = 0; b < 4; b++) acc_cnt[4 * (size_t)i + b] = 0;
      for (int b = 0; b < 4; b++)
        for (int k = 0; k < 3; k++) {
          acc_box[24 * (size_t)i + 6 * b + k] = key_of(INFINITY);
          acc_box[24 * (size_t)i + 6 * b + 3 + k] = key_of(-INFINITY);
        }
    }
  }
}

__device__ __forceinline__ void chunk_range(const BNode& n, uint32_t c, uint32_t& s, uint32_t& e) {
  s = n.start + (c - n.cbase) * kChunk;
  e = min(n.end, s + kChunk);
}

// Boxes of nodes whose box is still unknown: min/max of the primitive boxes.
__global__ void level_box_kernel(const LevelCounters* lcs, uint32_t L, BNode* __restrict__ pool,
                                 const uint32_t* __restrict__ chunk_node, const uint32_t* __restrict__ order,
                                 const float4* __restrict__ pbox) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t total = lcs[L].chunks;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t id = chunk_node[c];
    const BNode n = pool[id];
    if (!(n.flags & F_BOX_PENDING)) continue;
    uint32_t s, e;
    chunk_range(n, c, s, e);
    int lo[3] = {key_of(INFINITY), key_of(INFINITY), key_of(INFINITY)};
    int hi[3] = {key_of(-INFINITY), key_of(-INFINITY), key_of(-INFINITY)};
    for (uint32_t i = s + lane; i < e; i += 32) {
      const uint32_t p = order[i];
      const float4 a = pbox[2 * (size_t)p], b = pbox[2 * (size_t)p + 1];
      lo[0] = min(lo[0], key_of(a.x));
      lo[1] = min(lo[1], key_of(a.y));
      lo[2] = min(lo[2], key_of(a.z));
      hi[0] = max(hi[0], key_of(b.x));
      hi[1] = max(hi[1], key_of(b.y));
      hi[2] = max(hi[2], key_of(b.z));
    }
    for (int k = 0; k < 3; k++) {
      lo[k] = __reduce_min_sync(0xffffffffu, lo[k]);
      hi[k] = __reduce_max_sync(0xffffffffu, hi[k]);
    }
    if (lane < 3) {
      atomicMin(&pool[id].lo[lane], lo[lane]);
      atomicMax(&pool[id].hi[lane], hi[lane]);
    }
  }
}

struct SplitPlane {
  int axis;
  float a0, step;
};
__device__ __forceinline__ SplitPlane plane_of(const BNode& n) {
  const NodeBox nb = box_of(n);
  SplitPlane sp;
  sp.axis = split_axis(nb);
  sp.a0 = comp(nb.lo, sp.axis);
  const float a1 = comp(nb.hi, sp.axis);
  sp.step = (a1 - sp.a0) / 4.0f;
  return sp;
}

// Bucket counts and boxes of each chunk, merged into the node.
__global__ void level_stats_kernel(const uint32_t* __restrict__ lvl, uint32_t L, uint32_t N,
                                   const LevelCounters* lcs, const BNode* __restrict__ pool,
                                   const uint32_t* __restrict__ chunk_node, const uint32_t* __restrict__ order,
                                   const float4* __restrict__ pbox, const float* __restrict__ cen,
                                   uint32_t* __restrict__ chunk_cnt, uint32_t* __restrict__ acc_cnt,
                                   int* __restrict__ acc_box) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lb = lvl[L];
  const uint32_t total = lcs[L].chunks;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t id = chunk_node[c];
    const BNode n = pool[id];
    if (!(n.flags & F_ACTIVE)) continue;
    const SplitPlane sp = plane_of(n);
    const float* ck = cen + (size_t)sp.axis * N;
    uint32_t s, e;
    chunk_range(n, c, s, e);
    uint32_t cnt[4] = {0, 0, 0, 0};
    int bx[4][6];
#pragma unroll
    for (int b = 0; b < 4; b++) {
      bx[b][0] = bx[b][1] = bx[b][2] = key_of(INFINITY);
      bx[b][3] = bx[b][4] = bx[b][5] = key_of(-INFINITY);
    }
    for (uint32_t i = s + lane; i < e; i += 32) {
      const uint32_t p = order[i];
      const uint32_t bk = bucket_of(ck[p], sp.a0, sp.step);
      const float4 a = pbox[2 * (size_t)p], b = pbox[2 * (size_t)p + 1];
      const int k[6] = {key_of(a.x), key_of(a.y), key_of(a.z), key_of(b.x), key_of(b.y), key_of(b.z)};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (bk == (uint32_t)q) {
          cnt[q]++;
          bx[q][0] = min(bx[q][0], k[0]);
          bx[q][1] = min(bx[q][1], k[1]);
          bx[q][2] = min(bx[q][2], k[2]);
          bx[q][3] = max(bx[q][3], k[3]);
          bx[q][4] = max(bx[q][4], k[4]);
          bx[q][5] = max(bx[q][5], k[5]);
        }
      }
    }
    const uint32_t li = id - lb;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const uint32_t tot = __reduce_add_sync(0xffffffffu, cnt[q]);
      int r[6];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        r[k] = __reduce_min_sync(0xffffffffu, bx[q][k]);
        r[3 + k] = __reduce_max_sync(0xffffffffu, bx[q][3 + k]);
      }
      if (lane == 0) chunk_cnt[4 * (size_t)c + q] = tot;
      if (tot) {
        if (lane == 0) atomicAdd(&acc_cnt[4 * (size_t)li + q], tot);
        if (lane < 3) atomicMin(&acc_box[24 * (size_t)li + 6 * q + lane], r[lane]);
        else if (lane < 6) atomicMax(&acc_box[24 * (size_t)li + 6 * q + lane], r[lane]);
      }
    }
  }
}

// Nodes with more chunks than this leave their chunk prefix to
// level_big_prefix_kernel (a block per node); smaller ones are scanned by
// their own thread.
constexpr uint32_t kBigChunks = 8;

// The reference's split decision for one active node (strategy.rs:202-284):
// the 4 buckets' counts and boxes, then either BalanceTree's median split
// (3 empty buckets, strategy.rs:67-87) or the first strictly cheaper of the 3
// SAH candidates. Fills the two children; returns true for the median split.
__device__ __forceinline__ bool decide_split(const BNode& n, uint32_t i, const uint32_t* __restrict__ acc_cnt,
                                             const int* __restrict__ acc_box, BNode& l, BNode& r) {
  uint32_t cnt[4];
  NodeBox bb[4];
  for (int q = 0; q < 4; q++) {
    cnt[q] = acc_cnt[4 * (size_t)i + q];
    const int* k = acc_box + 24 * (size_t)i + 6 * q;
    bb[q] = NodeBox{{val_of(k[0]), val_of(k[1]), val_of(k[2])}, {val_of(k[3]), val_of(k[4]), val_of(k[5])}};
  }
  const int empties = (cnt[0] == 0) + (cnt[1] == 0) + (cnt[2] == 0) + (cnt[3] == 0);
  bool fallback = false;
  if (empties == 3) {
    // BalanceTree: median by centre on the same axis; child boxes come from
    // the next level's box pass
    fallback = true;
    const uint32_t mid = (n.end + n.start) / 2;
    l.start = n.start;
    l.end = mid;
    r.start = mid;
    r.end = n.end;
    l.flags = r.flags = F_BOX_PENDING;
    set_box(l, empty_box());
    set_box(r, empty_box());
  } else {
    // candidate j puts buckets 0..=j left; the first strictly cheaper
    // candidate wins, candidate 0 when no cost is below +inf
    float best_cost = INFINITY;
    NodeBox best_l = empty_box(), best_r = empty_box();
    uint32_t best_lc = 0;
    for (int j = 0; j < 3; j++) {
      NodeBox lb_ = empty_box(), rb_ = empty_box();
      uint32_t lc_ = 0, rc_ = 0;
      for (int p = 0; p <= j; p++) {
        grow(lb_, bb[p]);
        lc_ += cnt[p];
      }
      for (int p = j + 1; p < 4; p++) {
        grow(rb_, bb[p]);
        rc_ += cnt[p];
      }
      const float cost = sah_area(lb_) * (float)lc_ + sah_area(rb_) * (float)rc_;
      if (j == 0 || cost < best_cost) {
        best_l = lb_;
        best_r = rb_;
        best_lc = lc_;
      }
      if (cost < best_cost) best_cost = cost;
    }
    l.start = n.start;
    l.end = n.start + best_lc;
    r.start = n.start + best_lc;
    r.end = n.end;
    l.flags = r.flags = 0;
    set_box(l, best_l);
    set_box(r, best_r);
  }
  l.depth = r.depth = n.depth + 1;
  l.tree = r.tree = n.tree;
  l.left = r.left = NONE;
  return fallback;
}

// One thread per node of the level: the split decision, the two children
// (slots claimed per warp), and the exclusive per-bucket prefix of the node's
// chunk counts (big nodes: appended to big_list for the block-wide scan).
__global__ void level_decide_kernel(const uint32_t* __restrict__ lvl, uint32_t L, BNode* __restrict__ pool,
                                    const uint32_t* __restrict__ acc_cnt, const int* __restrict__ acc_box,
                                    const uint4* __restrict__ chunk_cnt, uint4* __restrict__ chunk_prefix,
                                    LevelCounters* lcs, BuildCounters* bc, uint32_t* __restrict__ big_list,
                                    uint32_t big_cap) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lb = lvl[L], next_base = lvl[L + 1], W = next_base - lb;
  LevelCounters* lc = lcs + L;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < W; i0 += stride) {
    const uint32_t i = i0 + lane;
    BNode n;
    bool active = false, fallback = false;
    BNode l{}, r{};
    if (i < W) {
      n = pool[lb + i];
      active = (n.flags & F_ACTIVE) != 0;
      if (active) fallback = decide_split(n, i, acc_cnt, acc_box, l, r);
    }
    const uint32_t base = next_base + warp_claim(&lc->children, active ? 2u : 0u, lane);
    const uint32_t n_sah = __popc(__ballot_sync(0xffffffffu, active && !fallback));
    const uint32_t n_med = __popc(__ballot_sync(0xffffffffu, active && fallback));
    if (lane == 0 && n_sah) atomicAdd(&bc->sah, (unsigned long long)n_sah);
    if (lane == 0 && n_med) atomicAdd(&bc->fallback, (unsigned long long)n_med);
    const bool big = active && !fallback && n.nchunks > kBigChunks;
    const uint32_t slot = warp_claim(&lc->big, big ? 1u : 0u, lane);
    if (!active) continue;
    pool[base] = l;
    pool[base + 1] = r;
    pool[lb + i].left = base;
    if (fallback) pool[lb + i].flags = n.flags | F_FALLBACK;
    if (fallback || n.nchunks == 0) continue;
    if (big && slot < big_cap) {
      big_list[slot] = lb + i;
      continue;
    }
    uint4 run = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t j = 0; j < n.nchunks; j++) {
      const uint4 v = chunk_cnt[n.cbase + j];
      chunk_prefix[n.cbase + j] = run;
      run.x += v.x;
      run.y += v.y;
      run.z += v.z;
      run.w += v.w;
    }
  }
}

// Exclusive per-bucket prefix of the chunk counts of the big nodes, one block
// per node: each thread takes kPerThread consecutive chunks of a tile, the
// block scans the thread totals (warp shuffles, then the warp totals).
constexpr uint32_t kPerThread = 4;
__global__ void __launch_bounds__(kBlock) level_big_prefix_kernel(const LevelCounters* lcs, uint32_t L,
                                                                  const BNode* __restrict__ pool,
                                                                  const uint32_t* __restrict__ big_list,
                                                                  uint32_t big_cap, const uint4* __restrict__ chunk_cnt,
                                                                  uint4* __restrict__ chunk_prefix) {
  __shared__ uint4 warp_total[kWarps];
  __shared__ uint4 carry_s;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t nbig = min(lcs[L].big, big_cap);
  for (uint32_t b = blockIdx.x; b < nbig; b += gridDim.x) {
    const BNode n = pool[big_list[b]];
    uint4 carry = make_uint4(0u, 0u, 0u, 0u);
    for (uint32_t t0 = 0; t0 < n.nchunks; t0 += kBlock * kPerThread) {
      const uint32_t j0 = t0 + threadIdx.x * kPerThread;
      uint4 v[kPerThread];
      uint4 sum = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (uint32_t k = 0; k < kPerThread; k++) {
        v[k] = j0 + k < n.nchunks ? chunk_cnt[n.cbase + j0 + k] : make_uint4(0u, 0u, 0u, 0u);
        sum.x += v[k].x;
        sum.y += v[k].y;
        sum.z += v[k].z;
        sum.w += v[k].w;
      }
      uint4 inc = sum;  // inclusive scan of the thread totals inside the warp
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, inc.x, o), y = __shfl_up_sync(0xffffffffu, inc.y, o);
        const uint32_t z = __shfl_up_sync(0xffffffffu, inc.z, o), w = __shfl_up_sync(0xffffffffu, inc.w, o);
        if (lane >= (uint32_t)o) {
          inc.x += x;
          inc.y += y;
          inc.z += z;
          inc.w += w;
        }
      }
      if (lane == 31) warp_total[warp] = inc;
      __syncthreads();
      uint4 before = carry;  // carry + earlier warps of the tile
      for (uint32_t q = 0; q < warp; q++) {
        const uint4 t = warp_total[q];
        before.x += t.x;
        before.y += t.y;
        before.z += t.z;
        before.w += t.w;
      }
      uint4 run = make_uint4(before.x + inc.x - sum.x, before.y + inc.y - sum.y, before.z + inc.z - sum.z,
                             before.w + inc.w - sum.w);
#pragma unroll
      for (uint32_t k = 0; k < kPerThread; k++) {
        if (j0 + k < n.nchunks) chunk_prefix[n.cbase + j0 + k] = run;
        run.x += v[k].x;
        run.y += v[k].y;
        run.z += v[k].z;
        run.w += v[k].w;
      }
      if (threadIdx.x == kBlock - 1) carry_s = run;  // the last thread's running total ends the tile
      __syncthreads();
      carry = carry_s;
      __syncthreads();
    }
  }
}

// Median split: Rust's select_nth_unstable_by on the node's range, one thread per node.
__global__ void level_select_kernel(const uint32_t* __restrict__ lvl, uint32_t L, uint32_t N,
                                    const BNode* __restrict__ pool, const float* __restrict__ cen,
                                    uint32_t* __restrict__ order) {
  const uint32_t lb = lvl[L], W = lvl[L + 1] - lb;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < W; i += gridDim.x * blockDim.x) {
    const BNode n = pool[lb + i];
    if (!(n.flags & F_FALLBACK)) continue;
    const uint32_t count = n.end - n.start;
    if (count / 2 == 0) continue;
    const int axis = split_axis(box_of(n));
    RustSelectNth<uint32_t, CentreLess> sel(CentreLess{cen + (size_t)axis * N});
    sel.run(order + n.start, count, count / 2);
  }
}

// SAH nodes: each chunk writes its primitives to their bucket-ordered slots.
__global__ void level_scatter_kernel(const uint32_t* __restrict__ lvl, uint32_t L, uint32_t N,
                                     const LevelCounters* lcs, const BNode* __restrict__ pool,
                                     const uint32_t* __restrict__ chunk_node, const uint32_t* __restrict__ order,
                                     const float* __restrict__ cen, const uint32_t* __restrict__ acc_cnt,
                                     const uint32_t* __restrict__ chunk_prefix, uint32_t* __restrict__ scratch) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t lb = lvl[L];
  const uint32_t total = lcs[L].chunks;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t id = chunk_node[c];
    const BNode n = pool[id];
    if ((n.flags & (F_ACTIVE | F_FALLBACK)) != F_ACTIVE) continue;
    const SplitPlane sp = plane_of(n);
    const float* ck = cen + (size_t)sp.axis * N;
    const uint32_t li = id - lb;
    uint32_t base[4];
    uint32_t run = n.start;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      base[q] = run + chunk_prefix[4 * (size_t)c + q];
      run += acc_cnt[4 * (size_t)li + q];
    }
    uint32_t s, e;
    chunk_range(n, c, s, e);
    for (uint32_t i0 = s; i0 < e; i0 += 32) {
      const uint32_t i = i0 + lane;
      const bool valid = i < e;
      const uint32_t p = valid ? order[i] : 0u;
      const uint32_t bk = valid ? bucket_of(ck[p], sp.a0, sp.step) : 4u;
      uint32_t dest = 0;
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const uint32_t m = __ballot_sync(0xffffffffu, bk == (uint32_t)q);
        if (bk == (uint32_t)q) dest = base[q] + __popc(m & lt_mask);
        base[q] += __popc(m);
      }
      if (valid) scratch[dest] = p;
    }
  }
}

// Also closes the level: the next level's end is its start plus the children
// that level_decide_kernel created (decide ran before this launch).
__global__ void level_copyback_kernel(uint32_t* __restrict__ lvl, uint32_t L, const LevelCounters* lcs,
                                      const BNode* __restrict__ pool, const uint32_t* __restrict__ chunk_node,
                                      const uint32_t* __restrict__ scratch, uint32_t* __restrict__ order) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t total = lcs[L].chunks;
  if (blockIdx.x == 0 && threadIdx.x == 0) lvl[L + 2] = lvl[L + 1] + lcs[L].children;
  for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < total; c += (gridDim.x * blockDim.x) >> 5) {
    const BNode n = pool[chunk_node[c]];
    if ((n.flags & (F_ACTIVE | F_FALLBACK)) != F_ACTIVE) continue;
    uint32_t s, e;
    chunk_range(n, c, s, e);
    for (uint32_t i = s + lane; i < e; i += 32) order[i] = scratch[i];
  }
}

// ---- numbering and emission --------------------------------------------

__global__ void subtree_size_kernel(uint32_t lb, uint32_t W, const BNode* __restrict__ pool, uint32_t* __restrict__ size) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W) return;
  const uint32_t l = pool[lb + i].left;
  size[lb + i] = l == NONE ? 1u : 1u + size[l] + size[l + 1];
}

__global__ void preorder_roots_kernel(uint32_t G, const uint32_t* __restrict__ bvh_start, uint32_t* __restrict__ pre) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < G) pre[g] = bvh_start[g];
}

__global__ void preorder_level_kernel(uint32_t lb, uint32_t W, const BNode* __restrict__ pool,
                                      const uint32_t* __restrict__ size, uint32_t* __restrict__ pre) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W) return;
  const uint32_t l = pool[lb + i].left;
  if (l == NONE) return;
  const uint32_t me = pre[lb + i];
  pre[l] = me + 1;
  pre[l + 1] = me + 1 + size[l];
}

__global__ void inner_flags_kernel(uint32_t T, const BNode* __restrict__ pool, const uint32_t* __restrict__ pre,
                                   uint32_t* __restrict__ inner_at) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id < T) inner_at[pre[id]] = pool[id].left != NONE ? 1u : 0u;
}

__device__ __forceinline__ uint32_t code_of(uint32_t id, const BNode* pool, const uint32_t* pre, const uint32_t* rank) {
  const uint32_t g = pre[id];
  return pool[id].left != NONE ? rank[g] : (LEAF_BIT | (g - rank[g]));
}

__global__ void emit_nodes_kernel(uint32_t T, uint32_t G, const BNode* __restrict__ pool, const uint32_t* __restrict__ size,
                                  const uint32_t* __restrict__ pre, const uint32_t* __restrict__ rank,
                                  const uint32_t* __restrict__ tree_end, DeviceBVHNode* __restrict__ forest,
                                  WideNode* __restrict__ wide, uint32_t* __restrict__ leaves,
                                  uint32_t* __restrict__ root_code) {
  const uint32_t id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= T) return;
  const BNode n = pool[id];
  const NodeBox b = box_of(n);
  const uint32_t g = pre[id];
  const bool inner = n.left != NONE;
  const uint32_t next = g + size[id];
  const uint32_t miss = next < tree_end[n.tree] ? next : INVALID_NEXT;
  DeviceBVHNode o;
  o.aabb_min[0] = b.lo.x;
  o.aabb_min[1] = b.lo.y;
  o.aabb_min[2] = b.lo.z;
  o.hit_next = inner ? g + 1 : miss;
  o.aabb_max[0] = b.hi.x;
  o.aabb_max[1] = b.hi.y;
  o.aabb_max[2] = b.hi.z;
  o.miss_next = miss;
  o.content_range[0] = n.start;
  o.content_range[1] = n.end;
  o.tail[0] = 0;
  o.tail[1] = 0;
  forest[g] = o;
  if (inner) {
    const NodeBox a = box_of(pool[n.left]), c = box_of(pool[n.left + 1]);
    WideNode w;
    const float vals[12] = {a.lo.x, a.lo.y, a.lo.z, a.hi.x, a.hi.y, a.hi.z, c.lo.x, c.lo.y, c.lo.z, c.hi.x, c.hi.y, c.hi.z};
    for (int k = 0; k < 12; k++) w.w[k] = vals[k];
    w.code[0] = code_of(n.left, pool, pre, rank);
    w.code[1] = code_of(n.left + 1, pool, pre, rank);
    w.code[2] = 0;
    w.code[3] = 0;
    wide[rank[g]] = w;
  } else {
    const uint32_t l = g - rank[g];
    leaves[2 * (size_t)l] = n.start;
    leaves[2 * (size_t)l + 1] = n.end;
  }
  if (id < G) root_code[id] = code_of(id, pool, pre, rank);
}

// indices_redirect and the 64 B triangle records in the sorted order.
// One thread per sorted triangle: its three vertices, copied (no arithmetic).
__global__ void emit_vertex_records_kernel(uint32_t N, const uint32_t* __restrict__ redirect,
                                           const uint32_t* __restrict__ idx, const float* __restrict__ vtx,
                                           VertexRecord* __restrict__ out) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
    const uint32_t p = __ldg(redirect + j);
    float v[9];
    for (int k = 0; k < 3; k++) {
      const float* q = vtx + 3 * (size_t)__ldg(idx + 3 * (size_t)p + k);
      v[3 * k] = __ldg(q);
      v[3 * k + 1] = __ldg(q + 1);
      v[3 * k + 2] = __ldg(q + 2);
    }
    float4* o = reinterpret_cast<float4*>(out + j);
    o[0] = make_float4(v[0], v[1], v[2], v[3]);
    o[1] = make_float4(v[4], v[5], v[6], v[7]);
    o[2] = make_float4(v[8], 0.0f, 0.0f, 0.0f);
  }
}

__global__ void emit_primitives_kernel(uint32_t N, const uint32_t* __restrict__ order, const uint32_t* __restrict__ idx,
                                       const float* __restrict__ vtx, uint32_t* __restrict__ redirect,
                                       TriRecord* __restrict__ tris) {
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
    const uint32_t p = order[j];
    redirect[j] = p;
    F3 v[3];
    for (int k = 0; k < 3; k++) {
      const float* q = vtx + 3 * (size_t)idx[3 * (size_t)p + k];
      v[k] = {q[0], q[1], q[2]};
    }
    const F3 e1 = {v[1].x - v[0].x, v[1].y - v[0].y, v[1].z - v[0].z};
    const F3 e2 = {v[2].x - v[0].x, v[2].y - v[0].y, v[2].z - v[0].z};
    F3 nrm = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    const float mag_sq = nrm.x * nrm.x + nrm.y * nrm.y + nrm.z * nrm.z;
    if (mag_sq > 0.0f) {
      const float inv = 1.0f / sqrtf(mag_sq);
      nrm = {nrm.x * inv, nrm.y * inv, nrm.z * inv};
    }
    const float uu = e1.x * e1.x + e1.y * e1.y + e1.z * e1.z;
    const float uv = e1.x * e2.x + e1.y * e2.y + e1.z * e2.z;
    const float vv = e2.x * e2.x + e2.y * e2.y + e2.z * e2.z;
    const float inv_d = 1.0f / (uv * uv - uu * vv);
    float4* o = reinterpret_cast<float4*>(tris + j);
    o[0] = make_float4(v[0].x, v[0].y, v[0].z, nrm.x);
    o[1] = make_float4(e1.x, e1.y, e1.z, nrm.y);
    o[2] = make_float4(e2.x, e2.y, e2.z, nrm.z);
    o[3] = make_float4(uu, uv, vv, inv_d);
  }
}

// True when box s is flat on some axis and lies on a face plane of box a,
// which is not flat there (the host build's flat_on_boundary: a ray with a
// zero direction component and its origin in that plane fails a's slab test
// but passes s's, so the four-child walk, which skips the boxes of opened
// nodes, must not open a node above such a child).
__device__ __forceinline__ bool flat_on_boundary(const NodeBox& s, const NodeBox& a) {
  const float sl[3] = {s.lo.x, s.lo.y, s.lo.z}, sh[3] = {s.hi.x, s.hi.y, s.hi.z};
  const float al[3] = {a.lo.x, a.lo.y, a.lo.z}, ah[3] = {a.hi.x, a.hi.y, a.hi.z};
  for (int k = 0; k < 3; k++)
    if (sl[k] == sh[k] && al[k] != ah[k] && (al[k] == sl[k] || ah[k] == sl[k])) return true;
  return false;
}

__device__ __forceinline__ bool openable(uint32_t x, const uint32_t anc[2], const BNode* pool) {
  const NodeBox bx = box_of(pool[x]);
  for (uint32_t c = pool[x].left; c <= pool[x].left + 1; c++) {
    const NodeBox bc = box_of(pool[c]);
    if (flat_on_boundary(bc, bx)) return false;
    for (int a = 0; a < 2; a++)
      if (anc[a] != NONE && flat_on_boundary(bc, box_of(pool[anc[a]]))) return false;
  }
  return true;
}

// Four-child collapse of binary inner node b: open the inner slot with the
// largest surface area (first of equals) until 4 slots are used, skipping
// nodes that openable() refuses (the host build's emit_wide4).
__device__ __forceinline__ int collapse_slots(uint32_t b, const BNode* pool, uint32_t slot[4]) {
  uint32_t anc[4][2];
  int n = 0;
  slot[n++] = pool[b].left;
  slot[n++] = pool[b].left + 1;
  for (int k = 0; k < 4; k++) anc[k][0] = anc[k][1] = NONE;
  while (n < 4) {
    int best = -1;
    float best_area = -1.0f;
    for (int k = 0; k < n; k++) {
      if (pool[slot[k]].left == NONE || !openable(slot[k], anc[k], pool)) continue;
      const float a = half_area(box_of(pool[slot[k]]));
      if (best < 0 || a > best_area) {
        best = k;
        best_area = a;
      }
    }
    if (best < 0) break;
    const uint32_t open = slot[best];
    const uint32_t up0 = open, up1 = anc[best][0];
    for (int k = n; k > best + 1; k--) {
      slot[k] = slot[k - 1];
      anc[k][0] = anc[k - 1][0];
      anc[k][1] = anc[k - 1][1];
    }
    slot[best] = pool[open].left;
    slot[best + 1] = pool[open].left + 1;
    for (int k = best; k <= best + 1; k++) {
      anc[k][0] = up0;
      anc[k][1] = up1;
    }
    n++;
  }
  return n;
}

// Four-child layout without a host round trip per level: the binary nodes
// that root a four-child node ("collapse roots") are marked top-down, one
// binary level per launch (a root's slots lie one to three levels below it,
// so they are marked before their level runs); one scan numbers the roots in
// pool order and one launch emits every node.
__global__ void wide4_roots_kernel(uint32_t G, const BNode* __restrict__ pool, uint32_t* __restrict__ croot,
                                   uint32_t* __restrict__ level4, uint32_t* __restrict__ max_level4) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= G || pool[g].left == NONE) return;
  croot[g] = 1u;
  level4[g] = 1u;
  atomicMax(max_level4, 1u);
}

__global__ void wide4_mark_kernel(uint32_t lb, uint32_t W, const BNode* __restrict__ pool,
                                  uint32_t* __restrict__ croot, uint32_t* __restrict__ level4,
                                  uint32_t* __restrict__ max_level4) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= W || !croot[lb + i]) return;
  uint32_t slot[4];
  const int n = collapse_slots(lb + i, pool, slot);
  const uint32_t lv = level4[lb + i] + 1u;
  for (int k = 0; k < n; k++)
    if (pool[slot[k]].left != NONE) {
      croot[slot[k]] = 1u;
      level4[slot[k]] = lv;
      atomicMax(max_level4, lv);
    }
}

__global__ void wide4_emit_kernel(uint32_t T, const BNode* __restrict__ pool, const uint32_t* __restrict__ croot,
                                  const uint32_t* __restrict__ index4, const uint32_t* __restrict__ pre,
                                  const uint32_t* __restrict__ rank, Wide4Node* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T || !croot[i]) return;
  uint32_t slot[4];
  const int n = collapse_slots(i, pool, slot);
  Wide4Node w;
  for (int k = 0; k < 4; k++) {
    const bool used = k < n;
    const NodeBox b = used ? box_of(pool[slot[k]]) : NodeBox{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    w.lo_x[k] = b.lo.x;
    w.lo_y[k] = b.lo.y;
    w.lo_z[k] = b.lo.z;
    w.hi_x[k] = b.hi.x;
    w.hi_y[k] = b.hi.y;
    w.hi_z[k] = b.hi.z;
    w.pad[k] = 0;
    if (!used) {
      w.code[k] = EMPTY_SLOT;
    } else if (pool[slot[k]].left != NONE) {
      w.code[k] = index4[slot[k]];
    } else {
      const uint32_t g = pre[slot[k]];
      w.code[k] = LEAF_BIT | (g - rank[g]);
    }
  }
  out[index4[i]] = w;
}

// ---- host side -------------------------------------------------------------

// Stream-ordered scratch: allocated from the context's pool on the build
// stream and returned to it (also stream-ordered) when the build returns, so
// that a rebuild takes no driver allocation and no implicit synchronisation.
struct Scratch {
  cudaMemPool_t pool;
  cudaStream_t st;
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <class T>
  cudaError_t alloc(T** out, size_t count) {
    void* p = nullptr;
    const size_t bytes = (count ? count : 1) * sizeof(T);
    cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, st) : cudaMallocAsync(&p, bytes, st);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
};

// Device array owned by DeviceBuilt: at least one element, zeroed when empty
// (the reference uploads one zeroed element for an empty array).
template <class T>
cudaError_t alloc_out(DevBuf<T>& b, size_t count, uint64_t& bytes, cudaStream_t s) {
  const size_t n = count ? count : 1;
  cudaError_t e = cudaMalloc(&b.ptr, n * sizeof(T));
  if (e != cudaSuccess) return e;
  b.count = count;
  bytes += n * sizeof(T);
  if (!count) return cudaMemsetAsync(b.ptr, 0, sizeof(T), s);
  return cudaSuccess;
}

inline uint32_t blocks_for(uint64_t n, uint32_t per = kBlock) {
  const uint64_t b = (n + per - 1) / per;
  return (uint32_t)(b ? b : 1);
}

}  // namespace

std::string build_blas_device(const std::vector<DeviceGeometry>& geoms, uint32_t bin_size, uint32_t max_depth,
                              int sm_count, cudaMemPool_t mem_pool, DeviceBuilt& d, DeviceBlasOut& out) {
  const uint32_t G = (uint32_t)geoms.size();
  uint64_t N64 = 0, V64 = 0;
  for (const auto& g : geoms) {
    N64 += g.triangle_count;
    V64 += g.vertex_count;
  }
  if (N64 >= (1ull << 31) || V64 >= (1ull << 31) / 3 || N64 * 3 >= (1ull << 32))
    return "too many triangles or vertices for one device build";
  const uint32_t N = (uint32_t)N64, V = (uint32_t)V64;
  out = DeviceBlasOut();
  out.triangles = N;
  out.vertices = V;
  cudaStream_t st = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e != cudaSuccess) return std::string("CUDA stream: ") + cudaGetErrorString(e);
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } guard{st};
  Scratch S{mem_pool, st, {}};
  uint64_t& bytes = out.bytes;
#define CK(x)                                                                                  \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess)                                                                     \
      return std::string(e_ == cudaErrorMemoryAllocation ? "CUDA OOM " : "CUDA ") + #x + ": " + \
             cudaGetErrorString(e_);                                                           \
  } while (0)

  // geometry arrays
  CK(alloc_out(d.vertices, 3 * (size_t)V, bytes, st));
  CK(alloc_out(d.indices, 3 * (size_t)N, bytes, st));
  std::vector<uint32_t> g_prim(G + 1, 0), g_vs(G), g_vc(G), g_ix(G);
  {
    uint32_t ps = 0, vs = 0;
    for (uint32_t g = 0; g < G; g++) {
      const DeviceGeometry& q = geoms[g];
      g_prim[g] = ps;
      g_vs[g] = vs;
      g_vc[g] = q.vertex_count;
      g_ix[g] = q.indices ? 1u : 0u;
      if (q.vertex_count)
        CK(cudaMemcpyAsync(d.vertices.ptr + 3 * (size_t)vs, q.positions, 12 * (size_t)q.vertex_count,
                           cudaMemcpyHostToDevice, st));
      if (q.indices && q.triangle_count)
        CK(cudaMemcpyAsync(d.indices.ptr + 3 * (size_t)ps, q.indices, 12 * (size_t)q.triangle_count,
                           cudaMemcpyHostToDevice, st));
      ps += q.triangle_count;
      vs += q.vertex_count;
    }
    g_prim[G] = ps;
  }
  d.vertex_count = V;
  uint32_t *dg_prim, *dg_vs, *dg_vc, *dg_ix;
  CK(S.alloc(&dg_prim, G + 1));
  CK(S.alloc(&dg_vs, G));
  CK(S.alloc(&dg_vc, G));
  CK(S.alloc(&dg_ix, G));
  CK(cudaMemcpyAsync(dg_prim, g_prim.data(), 4 * (size_t)(G + 1), cudaMemcpyHostToDevice, st));
  if (G) {
    CK(cudaMemcpyAsync(dg_vs, g_vs.data(), 4 * (size_t)G, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dg_vc, g_vc.data(), 4 * (size_t)G, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dg_ix, g_ix.data(), 4 * (size_t)G, cudaMemcpyHostToDevice, st));
  }

  float4* pbox;
  float* cen;
  uint32_t *order, *scratch;
  BuildCounters* bc;
  CK(S.alloc(&pbox, 2 * (size_t)N));
  CK(S.alloc(&cen, 3 * (size_t)N));
  CK(S.alloc(&order, N));
  CK(S.alloc(&scratch, N));
  CK(S.alloc(&bc, 1));
  CK(cudaMemsetAsync(bc, 0, sizeof(BuildCounters), st));
  const uint32_t persistent = (uint32_t)(sm_count > 0 ? sm_count : 1) * 8;
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  struct EventGuard {
    cudaEvent_t a, b;
    ~EventGuard() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } eg{ev0, ev1};
  CK(cudaEventRecord(ev0, st));
  if (N) {
    prepare_primitives_kernel<<<std::min(blocks_for(N), persistent * 4), kBlock, 0, st>>>(
        N, G, dg_prim, dg_vs, dg_vc, dg_ix, d.indices.ptr, d.vertices.ptr, pbox, cen, order, bc);
    CK(cudaGetLastError());
    // stop before any kernel reads a vertex through an out-of-range index
    BuildCounters pre;
    CK(cudaMemcpyAsync(&pre, bc, sizeof(pre), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (pre.bad_index) return "triangle index out of range";
  }

  // roots: one per geometry, box pending
  size_t cap = 2 * (size_t)N + 2 * (size_t)G + 64;
  BNode* pool;
  CK(S.alloc(&pool, cap));
  {
    std::vector<BNode> roots(G);
    for (uint32_t g = 0; g < G; g++) {
      BNode& r = roots[g];
      std::memset(&r, 0, sizeof(r));
      for (int k = 0; k < 3; k++) {
        r.lo[k] = key_of(INFINITY);
        r.hi[k] = key_of(-INFINITY);
      }
      r.start = g_prim[g];
      r.end = g_prim[g + 1];
      r.depth = 0;
      r.left = NONE;
      r.tree = g;
      r.flags = F_BOX_PENDING;
    }
    if (G) CK(cudaMemcpyAsync(pool, roots.data(), sizeof(BNode) * G, cudaMemcpyHostToDevice, st));
  }

  // level rounds. Every buffer is sized for the largest possible level (a
  // level holds at most N + G nodes: ranges are disjoint and only empty roots
  // are empty), so that no level waits for the host. The host queues a batch
  // of levels, then reads the level bounds back once to see whether an empty
  // level has been reached; levels queued past it do nothing.
  const uint32_t level_cap = (uint32_t)std::min<uint64_t>(max_depth, N) + 2;  // possible levels + one empty
  const size_t node_cap = (size_t)N + G + 1;
  const size_t chunk_cap = (size_t)N / kChunk + node_cap + 1;
  const uint32_t big_cap = N / (kBigChunks * kChunk) + 2;  // a big node holds > kBigChunks * kChunk primitives
  uint32_t *lvl, *acc_cnt, *chunk_node, *chunk_cnt, *chunk_prefix, *big_list;
  LevelCounters* lcs;
  int* acc_box;
  CK(S.alloc(&lvl, (size_t)level_cap + 2));
  CK(S.alloc(&lcs, level_cap));
  CK(S.alloc(&acc_cnt, 4 * node_cap));
  CK(S.alloc(&acc_box, 24 * node_cap));
  CK(S.alloc(&chunk_node, chunk_cap));
  CK(S.alloc(&chunk_cnt, 4 * chunk_cap));
  CK(S.alloc(&chunk_prefix, 4 * chunk_cap));
  CK(S.alloc(&big_list, big_cap));
  CK(cudaMemsetAsync(lcs, 0, sizeof(LevelCounters) * level_cap, st));
  const uint32_t lvl0[2] = {0, G};
  CK(cudaMemcpyAsync(lvl, lvl0, sizeof(lvl0), cudaMemcpyHostToDevice, st));
  std::vector<uint32_t> h_lvl((size_t)level_cap + 2);
  uint32_t queued = 0, levels = 0;
  bool closed = false;
  // first batch: about the depth of a balanced tree, then a few levels at a time
  uint32_t batch = 2;
  for (uint64_t m = std::max<uint32_t>(bin_size, 1); m < N; m *= 2) batch++;
  while (!closed) {
    const uint32_t stop = std::min(queued + batch, level_cap);
    batch = 4;
    for (; queued < stop; queued++) {
      const uint32_t L = queued;
      level_prepare_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, bin_size, max_depth, pool, acc_cnt, acc_box,
                                                          chunk_node, lcs);
      level_box_kernel<<<persistent, kBlock, 0, st>>>(lcs, L, pool, chunk_node, order, pbox);
      level_stats_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, N, lcs, pool, chunk_node, order, pbox, cen,
                                                        chunk_cnt, acc_cnt, acc_box);
      level_decide_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, pool, acc_cnt, acc_box,
                                                         reinterpret_cast<const uint4*>(chunk_cnt),
                                                         reinterpret_cast<uint4*>(chunk_prefix), lcs, bc, big_list,
                                                         big_cap);
      level_big_prefix_kernel<<<persistent, kBlock, 0, st>>>(lcs, L, pool, big_list, big_cap,
                                                             reinterpret_cast<const uint4*>(chunk_cnt),
                                                             reinterpret_cast<uint4*>(chunk_prefix));
      level_select_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, N, pool, cen, order);
      level_scatter_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, N, lcs, pool, chunk_node, order, cen, acc_cnt,
                                                          chunk_prefix, scratch);
      level_copyback_kernel<<<persistent, kBlock, 0, st>>>(lvl, L, lcs, pool, chunk_node, scratch, order);
    }
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(h_lvl.data(), lvl, 4 * ((size_t)queued + 2), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (uint32_t k = 0; k <= queued && !closed; k++)
      if (h_lvl[k + 1] == h_lvl[k]) {  // level k is empty: the tree has k levels
        levels = k;
        closed = true;
      }
    if (!closed && queued >= level_cap) return "device build: tree deeper than its level bound";
  }
  std::vector<uint32_t> level_begin(h_lvl.begin(), h_lvl.begin() + levels + 1);
  const uint32_t T = h_lvl[levels];
  level_begin.push_back(T);  // level l = [level_begin[l], level_begin[l+1]); the last entry repeats T
  const uint32_t L = (uint32_t)level_begin.size() - 2;  // number of levels (0 when G == 0)
  out.max_depth = L ? L - 1 : 0;
  out.nodes = T;

  // The four-child collapse reads only the finished binary tree: its marks
  // and numbering scan run on a side stream, overlapped with the subtree
  // sizes, the pre-order numbering and their host round trips below; the
  // emit waits for them.
  struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    ~SideStream() {
      // before the scratch it reads is freed (on the main stream, by S's
      // destructor, which runs after this one), also on an early error return
      if (s) cudaStreamSynchronize(s);
      if (join) cudaEventDestroy(join);
      if (fork) cudaEventDestroy(fork);
      if (s) cudaStreamDestroy(s);
    }
  } side;
  uint32_t *croot, *level4, *index4, *max_level4;
  CK(S.alloc(&croot, T));
  CK(S.alloc(&level4, T));
  CK(S.alloc(&index4, T));
  CK(S.alloc(&max_level4, 1));
  void* scan4 = nullptr;
  if (T) CK(S.alloc(reinterpret_cast<char**>(&scan4), scan_scratch_bytes(T) + 256));
  CK(cudaMemsetAsync(croot, 0, 4 * (size_t)(T ? T : 1), st));
  CK(cudaMemsetAsync(level4, 0, 4 * (size_t)(T ? T : 1), st));
  CK(cudaMemsetAsync(max_level4, 0, 4, st));
  CK(cudaStreamCreateWithFlags(&side.s, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&side.fork, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&side.join, cudaEventDisableTiming));
  CK(cudaEventRecord(side.fork, st));
  CK(cudaStreamWaitEvent(side.s, side.fork, 0));
  if (T) {
    wide4_roots_kernel<<<blocks_for(G), kBlock, 0, side.s>>>(G, pool, croot, level4, max_level4);
    for (uint32_t l = 0; l < L; l++) {
      const uint32_t a = level_begin[l], W = level_begin[l + 1] - a;
      wide4_mark_kernel<<<blocks_for(W), kBlock, 0, side.s>>>(a, W, pool, croot, level4, max_level4);
    }
    CK(scan_u32(croot, index4, T, false, 0, scan4, side.s));
    CK(cudaGetLastError());
  }
  CK(cudaEventRecord(side.join, side.s));

  // subtree sizes, bottom-up
  uint32_t *size, *pre, *inner_at, *rank, *tree_end, *bvh_start, *root_code;
  CK(S.alloc(&size, T));
  CK(S.alloc(&pre, T));
  CK(S.alloc(&inner_at, T));
  CK(S.alloc(&rank, T));
  CK(S.alloc(&tree_end, G));
  CK(S.alloc(&bvh_start, G));
  CK(S.alloc(&root_code, G));
  for (int l = (int)L - 1; l >= 0; l--) {
    const uint32_t a = level_begin[l], W = level_begin[l + 1] - a;
    subtree_size_kernel<<<blocks_for(W), kBlock, 0, st>>>(a, W, pool, size);
  }
  CK(cudaGetLastError());
  out.tree_nodes.resize(G);
  std::vector<BNode> roots(G);
  if (G) {
    CK(cudaMemcpyAsync(out.tree_nodes.data(), size, 4 * (size_t)G, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(roots.data(), pool, sizeof(BNode) * G, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
  }
  std::vector<uint32_t> h_start(G), h_end(G);
  {
    uint32_t acc = 0;
    for (uint32_t g = 0; g < G; g++) {
      h_start[g] = acc;
      acc += out.tree_nodes[g];
      h_end[g] = acc;
    }
  }
  if (G) {
    CK(cudaMemcpyAsync(bvh_start, h_start.data(), 4 * (size_t)G, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(tree_end, h_end.data(), 4 * (size_t)G, cudaMemcpyHostToDevice, st));
    preorder_roots_kernel<<<blocks_for(G), kBlock, 0, st>>>(G, bvh_start, pre);
  }
  for (uint32_t l = 0; l < L; l++) {
    const uint32_t a = level_begin[l], W = level_begin[l + 1] - a;
    preorder_level_kernel<<<blocks_for(W), kBlock, 0, st>>>(a, W, pool, size, pre);
  }
  uint32_t inner_total = 0;
  if (T) {
    inner_flags_kernel<<<blocks_for(T), kBlock, 0, st>>>(T, pool, pre, inner_at);
    void* scan_tmp;
    CK(S.alloc(reinterpret_cast<char**>(&scan_tmp), scan_scratch_bytes(T) + 256));
    CK(scan_u32(inner_at, rank, T, false, 0, scan_tmp, st));
    uint32_t last[2];
    CK(cudaMemcpyAsync(&last[0], rank + (T - 1), 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&last[1], inner_at + (T - 1), 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    inner_total = last[0] + last[1];
  }
  const uint32_t leaf_total = T - inner_total;
  CK(alloc_out(d.tri_bvh_forest, T, bytes, st));
  CK(alloc_out(d.wide_nodes, inner_total, bytes, st));
  CK(alloc_out(d.leaf_ranges, 2 * (size_t)leaf_total, bytes, st));
  CK(alloc_out(d.indices_redirect, N, bytes, st));
  CK(alloc_out(d.tri_records, N, bytes, st));
  if (T)
    emit_nodes_kernel<<<blocks_for(T), kBlock, 0, st>>>(T, G, pool, size, pre, rank, tree_end, d.tri_bvh_forest.ptr,
                                                        d.wide_nodes.ptr, d.leaf_ranges.ptr, root_code);
  if (N)
    emit_primitives_kernel<<<std::min(blocks_for(N), persistent * 4), kBlock, 0, st>>>(
        N, order, d.indices.ptr, d.vertices.ptr, d.indices_redirect.ptr, d.tri_records.ptr);
  CK(cudaGetLastError());

  // four-child layout: collapse roots marked level by level, numbered by one
  // scan in pool order (inner geometry roots first, in geometry order), one emit
  out.root_code.resize(G);
  out.root_code4.resize(G);
  CK(alloc_out(d.wide4_nodes, inner_total, bytes, st));
  std::vector<char> leaf_root(G, 0);  // their four-child code is the two-child one, read back at the end
  {
    uint32_t inner_roots = 0;
    for (uint32_t g = 0; g < G; g++) {
      if (roots[g].left == NONE) leaf_root[g] = 1;
      else out.root_code4[g] = inner_roots++;
    }
  }
  uint32_t tail4[3] = {0, 0, 0};  // index4[T-1], croot[T-1], deepest level
  CK(cudaStreamWaitEvent(st, side.join, 0));
  if (T) {
    wide4_emit_kernel<<<blocks_for(T), kBlock, 0, st>>>(T, pool, croot, index4, pre, rank, d.wide4_nodes.ptr);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&tail4[0], index4 + (T - 1), 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tail4[1], croot + (T - 1), 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tail4[2], max_level4, 4, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaEventRecord(ev1, st));

  BuildCounters hbc;
  if (G) CK(cudaMemcpyAsync(out.root_code.data(), root_code, 4 * (size_t)G, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&hbc, bc, sizeof(hbc), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  d.wide4_nodes.count = tail4[0] + tail4[1];
  out.max_wide4_depth = tail4[2];
  for (uint32_t g = 0; g < G; g++)
    if (leaf_root[g]) out.root_code4[g] = out.root_code[g];
  float ms = 0.0f;
  CK(cudaEventElapsedTime(&ms, ev0, ev1));
  out.kernel_seconds = ms / 1000.0;
  out.sah_splits = hbc.sah;
  out.median_fallbacks = hbc.fallback;
  out.root_box.resize(G);
  for (uint32_t g = 0; g < G; g++) {
    const BNode& r = roots[g];
    out.root_box[g] = Box{{val_of(r.lo[0]), val_of(r.lo[1]), val_of(r.lo[2])}, {val_of(r.hi[0]), val_of(r.hi[1]), val_of(r.hi[2])}};
  }
#undef CK
  return std::string();
}

cudaError_t emit_vertex_records(const DeviceBuilt& d, cudaStream_t st) {
  const uint32_t N = (uint32_t)d.indices_redirect.count;
  if (N == 0) return cudaSuccess;
  const uint32_t blocks = std::min<uint32_t>((N + kBlock - 1) / kBlock, 4096u);
  emit_vertex_records_kernel<<<blocks, kBlock, 0, st>>>(N, d.indices_redirect.ptr, d.indices.ptr, d.vertices.ptr,
                                                        d.vertex_records.ptr);
  return cudaGetLastError();
}

}  // namespace rdn
