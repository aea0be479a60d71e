// Oracle — TEST INFRASTRUCTURE ONLY. Nothing in the product (rendiation_gb300/,
// include/) may include, link or call this code; only tests/, the smoke check and
// bench.py's cpu_baseline / reference arm use it, and only as the checker.
//
// A C++ restatement of the reference's CPU ray-query path, function by function:
//
//   BuildPrimitive / TreeBuildOption        content/space/src/utils.rs:20-66
//   FlattenBVH::new                         content/space/src/bvh/mod.rs:55-79
//   FlattenBVHNode child offsets            content/space/src/bvh/node.rs:43-52
//   BVHBuildStrategy::build (pre-order)     content/space/src/bvh/strategy.rs:11-43
//   BalanceTree::split                      content/space/src/bvh/strategy.rs:66-87
//   SAH::new / split / cost / degenerate    content/space/src/bvh/strategy.rs:105-136,159-161,202-284
//   median_partition_at_axis                content/space/src/bvh/apply.rs:19-45
//   build_blas / build_tlas / build         shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/mod.rs:122-494
//   compute_bvh_next                        .../geometry/naive/mod.rs:611-632
//   NaiveSahBvhCpu::traverse + RayRange     .../geometry/naive/traverse_cpu.rs:52-281
//   TraverseBvhIteratorCpu::next            .../geometry/naive/traverse_cpu.rs:291-319
//   TraverseFlags                           .../geometry/naive/flag.rs:24-117
//   intersect_ray_aabb_cpu                  .../geometry/mod.rs:44-64
//   intersect_ray_triangle_cpu              .../geometry/mod.rs:104-155
//
// PARITY UNPINNED: the reference is Rust and no Rust toolchain exists here, and
// the reference's own ray-query tests dump images without assertions
// (naive/test.rs:227-444), so this restatement cannot be checked against the
// reference's outputs. It is cross-checked instead against an FP64 brute-force
// closest hit, against hand-computed cases, and the product's BVH is compared
// with this builder node by node.
//
// Deliberate extension: the reference's CPU `Hit` drops the barycentrics; this
// restatement also returns u, v, the instance slot, the custom index and the hit
// kind (the same values the reference's GPU path stores, traverse_gpu.rs:556-590).
// Counters are per thread instead of the reference's global atomics
// (traverse_cpu.rs:38-41), with the same increments.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fno-fast-math -shared -fPIC (see Makefile).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "orc_math.h"
#include "orc_select.h"
#include "orc_shade.h"
#include "orc_ao.h"
#include "orc_pt.h"

namespace orc {

static const uint32_t INVALID_NEXT = 0xFFFFFFFFu;

// ---- flags (shader/ray-tracing/src/api/ty.rs:102-159) ----
enum : uint32_t {
  TF_FORCE_OPAQUE = 0x01,
  TF_FORCE_NON_OPAQUE = 0x02,
  TF_ACCEPT_FIRST_HIT_AND_END_SEARCH = 0x04,
  TF_CULL_BACK_FACING_TRIANGLES = 0x10,
  TF_CULL_FRONT_FACING_TRIANGLES = 0x20,
  TF_CULL_OPAQUE = 0x40,
  TF_CULL_NON_OPAQUE = 0x80,
  TF_SKIP_TRIANGLES = 0x100,
  TF_TRIANGLE_FLIP_FACING = 0x400,
};
enum : uint32_t {
  GI_TRIANGLE_FACING_CULL_DISABLE = 0x1,
  GI_TRIANGLE_FLIP_FACING = 0x2,
  GI_FORCE_OPAQUE = 0x4,
  GI_FORCE_NO_OPAQUE = 0x8,
};
static const uint32_t GEOMETRY_FLAG_OPAQUE = 0x1;
static const uint32_t ANYHIT_ACCEPT = 1, ANYHIT_END_SEARCH = 2;

static uint32_t merge_geometry_instance_flag(uint32_t f, uint32_t gi) {
  if (gi & GI_TRIANGLE_FACING_CULL_DISABLE)
    f = f & ~(TF_CULL_BACK_FACING_TRIANGLES | TF_CULL_FRONT_FACING_TRIANGLES);
  if (gi & GI_TRIANGLE_FLIP_FACING) f = f ^ TF_TRIANGLE_FLIP_FACING;
  if (gi & GI_FORCE_OPAQUE) f = f | TF_FORCE_OPAQUE;
  if (gi & GI_FORCE_NO_OPAQUE) f = f | TF_FORCE_NON_OPAQUE;
  return f;
}
static void cull_geometry(uint32_t f, uint32_t gf, bool* pass, bool* is_opaque) {
  bool geometry_opaque = (gf & GEOMETRY_FLAG_OPAQUE) != 0;
  bool force_opaque = (f & TF_FORCE_OPAQUE) != 0;
  bool force_non_opaque = (f & TF_FORCE_NON_OPAQUE) != 0;
  bool cull_opaque = (f & TF_CULL_OPAQUE) != 0;
  bool cull_non_opaque = (f & TF_CULL_NON_OPAQUE) != 0;
  bool op = (geometry_opaque || force_opaque) && !force_non_opaque;
  *pass = (op && !cull_opaque) || (!op && !cull_non_opaque);
  *is_opaque = op;
}
static void cull_triangle(uint32_t f, bool* cull_enable, bool* cull_back) {
  bool flip = (f & TF_TRIANGLE_FLIP_FACING) != 0;
  bool cf = (f & TF_CULL_FRONT_FACING_TRIANGLES) != 0;
  bool cb = (f & TF_CULL_BACK_FACING_TRIANGLES) != 0;
  *cull_enable = cf || cb;
  *cull_back = (flip && cb) || (!flip && cf);
}

// ---- intersectors ----
// far_scale: 1 is the reference's test; the watertight mode passes
// 1 + 4 * 2^-23 >= 1 + 2 gamma_3 (Ize, "Robust BVH Ray Traversal", JCGT 2013)
// so that rounding never rejects a box the ray touches.
static const float WATERTIGHT_BOX_FAR_SCALE = 1.000000476837158203125f;
static inline bool intersect_ray_aabb(V3 o, V3 d, float tmin, float tmax, V3 bmin, V3 bmax, float far_scale = 1.0f) {
  V3 inv_d = v3(1.0f, 1.0f, 1.0f) / d;
  V3 t0 = (bmin - o) * inv_d;
  V3 t1 = (bmax - o) * inv_d;
  V3 tn = vmin(t0, t1);
  V3 tf = vmax(t0, t1);
  float t_near_max = max_channel(tn);
  float t_far_min = min_channel(tf) * far_scale;
  return t_near_max <= t_far_min && tmin < t_far_min && t_near_max < tmax;
}

struct TriResult { float s, t, u, v; };
static inline TriResult intersect_ray_triangle(V3 origin, V3 direction, float near_, float far_, V3 v0, V3 v1,
                                               V3 v2, bool cull_enable, bool cull_back) {
  TriResult miss{0.0f, 0.0f, 0.0f, 0.0f};
  V3 e1 = v1 - v0;
  V3 e2 = v2 - v0;
  V3 normal = normalize(cross(e1, e2));
  float b = dot(normal, direction);
  float sign = signum(b);
  if (cull_enable) {
    bool pass = cull_back != (b < 0.0f);
    if (!pass) return miss;
  }
  V3 w0 = origin - v0;
  float a = -dot(normal, w0);
  float t = a / b;
  if (t < near_ || t > far_) return miss;
  V3 p = origin + t * direction;
  float uu = dot(e1, e1);
  float uv = dot(e1, e2);
  float vv = dot(e2, e2);
  V3 w = p - v0;
  float wu = dot(w, e1);
  float wv = dot(w, e2);
  float inverse_d = 1.0f / (uv * uv - uu * vv);
  float u = (uv * wv - vv * wu) * inverse_d;
  if (u < 0.0f || u > 1.0f) return miss;
  float v = (uv * wu - uu * wv) * inverse_d;
  if (v < 0.0f || (u + v) > 1.0f) return miss;
  return TriResult{sign, t, u, v};
}

// Watertight f32 triangle test: Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013 (sheared frame with the ray
// along +z, 2D edge functions U, V, W). It is not part of the reference, which
// only has the formula above; this is the oracle twin of the product's
// optional watertight test, with the same operations in the same order:
// kz = largest |d| component (lowest axis among equals), kx / ky the next two,
// swapped when d[kz] < 0; Sz = 1/d[kz], Sx = d[kx]*Sz, Sy = d[ky]*Sz; an edge
// function that rounds to 0 makes all three be recomputed as exact-sign
// differences of products (TwoProduct by FMA) instead of the paper's double
// fallback; t, u, v from one reciprocal of det; NaN never hits. det has the
// opposite sign of the formula above's b, so culling and the facing sign
// follow b's rules.
static inline float pick3(V3 v, uint32_t k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
static inline float diff_products(float a, float b, float c, float d) {
  float p = a * b, q = c * d;
  float e = std::fma(a, b, -p), f = std::fma(c, d, -q);
  return (p - q) + (e - f);
}
static inline TriResult intersect_ray_triangle_watertight(V3 o, V3 d, float near_, float far_, V3 v0, V3 v1, V3 v2,
                                                          bool cull_enable, bool cull_back) {
  TriResult miss{0.0f, 0.0f, 0.0f, 0.0f};
  float adx = std::fabs(d.x), ady = std::fabs(d.y), adz = std::fabs(d.z);
  uint32_t kz = adx >= ady ? (adx >= adz ? 0u : 2u) : (ady >= adz ? 1u : 2u);
  uint32_t kx = kz == 2u ? 0u : kz + 1u;
  uint32_t ky = kx == 2u ? 0u : kx + 1u;
  if (pick3(d, kz) < 0.0f) std::swap(kx, ky);
  V3 inv_d = v3(1.0f, 1.0f, 1.0f) / d;
  float sz = pick3(inv_d, kz), sx = pick3(d, kx) * sz, sy = pick3(d, ky) * sz;
  V3 A = v0 - o, B = v1 - o, C = v2 - o;
  float akz = pick3(A, kz), bkz = pick3(B, kz), ckz = pick3(C, kz);
  float ax = pick3(A, kx) - sx * akz, ay = pick3(A, ky) - sy * akz;
  float bx = pick3(B, kx) - sx * bkz, by = pick3(B, ky) - sy * bkz;
  float cx = pick3(C, kx) - sx * ckz, cy = pick3(C, ky) - sy * ckz;
  float U = cx * by - cy * bx, V = ax * cy - ay * cx, W = bx * ay - by * ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = diff_products(cx, by, cy, bx);
    V = diff_products(ax, cy, ay, cx);
    W = diff_products(bx, ay, by, ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return miss;
  float det = (U + V) + W;
  if (!(std::fabs(det) > 0.0f)) return miss;
  if (cull_enable) {
    bool pass = cull_back != (det > 0.0f);
    if (!pass) return miss;
  }
  float T = (U * (sz * akz) + V * (sz * bkz)) + W * (sz * ckz);
  float rcp = 1.0f / det;
  float t = T * rcp;
  if (!(t >= near_ && t <= far_)) return miss;
  return TriResult{det > 0.0f ? -1.0f : 1.0f, t, V * rcp, W * rcp};
}

// ---- BVH builder ----
struct BuildPrimitive {
  Box3 bounding;
  V3 center;
};
struct FlatNode {
  Box3 bounding;
  size_t start, end;
  size_t self_index;
  bool has_child;
  size_t left_count;
  int split_axis;
};
struct BuildOption {
  size_t max_tree_depth;
  size_t bin_size;
  bool should_continue(size_t count, size_t depth) const { return depth < max_tree_depth && count > bin_size; }
};
struct BuildStats {
  uint64_t sah_splits = 0, median_fallbacks = 0;
};

static Box3 bounding_from_build_source(const std::vector<size_t>& idx, const std::vector<BuildPrimitive>& prims,
                                       size_t s, size_t e) {
  Box3 b = box_empty();
  for (size_t i = s; i < e; i++) box_union(b, prims[idx[i]].bounding);
  return b;
}

struct SahBuilder {
  const std::vector<BuildPrimitive>& prims;
  std::vector<size_t>& idx;
  std::vector<FlatNode>& nodes;
  BuildOption opt;
  BuildStats stats;
  // pre_partition caches: bounding + bucket (SAH::new(4))
  static const size_t PARTITIONS = 4;
  Box3 pre_box[PARTITIONS];
  std::vector<size_t> pre_bucket[PARTITIONS];

  struct Split {
    Box3 lb;
    size_t ls, le;
    int axis;
    Box3 rb;
    size_t rs, re;
  };

  Split balance_split(const FlatNode& parent) {
    int axis = box_longest_axis(parent.bounding);
    size_t s = parent.start, e = parent.end;
    size_t middle = (e + s) / 2;
    size_t range_middle = (e - s) / 2;
    if (range_middle != 0) {
      auto less = [this, axis](const size_t& a, const size_t& b) {
        float ca = axis_of(prims[a].center, axis), cb = axis_of(prims[b].center, axis);
        // partial_cmp(..).unwrap_or(Less) == Less
        if (std::isnan(ca) || std::isnan(cb)) return true;
        return ca < cb;
      };
      RustSelect<size_t, decltype(less)> sel{less};
      sel.select_nth(idx.data() + s, e - s, range_middle);
    }
    Split r;
    r.lb = bounding_from_build_source(idx, prims, s, middle);
    r.ls = s;
    r.le = middle;
    r.axis = axis;
    r.rb = bounding_from_build_source(idx, prims, middle, e);
    r.rs = middle;
    r.re = e;
    return r;
  }

  Split sah_split(const FlatNode& parent) {
    size_t s = parent.start, e = parent.end;
    for (size_t p = 0; p < PARTITIONS; p++) {
      pre_bucket[p].clear();
      pre_box[p] = box_empty();
    }
    int axis = box_longest_axis(parent.bounding);
    float a0 = axis_of(parent.bounding.min, axis), a1 = axis_of(parent.bounding.max, axis);
    float step = (a1 - a0) / (float)PARTITIONS;
    for (size_t i = s; i < e; i++) {
      size_t index = idx[i];
      const BuildPrimitive& p = prims[index];
      float axis_value = axis_of(p.center, axis);
      size_t which = sat_usize(std::floor((axis_value - a0) / step));
      if (which == PARTITIONS) which -= 1;
      if (which > PARTITIONS) which = PARTITIONS - 1;  // unreachable for finite input (Rust would panic)
      box_union(pre_box[which], p.bounding);
      pre_bucket[which].push_back(index);
    }
    size_t empty_count = 0;
    for (size_t p = 0; p < PARTITIONS; p++) empty_count += pre_bucket[p].empty() ? 1 : 0;
    if (empty_count == PARTITIONS - 1) {
      stats.median_fallbacks++;
      return balance_split(parent);
    }
    stats.sah_splits++;
    Box3 lbox[PARTITIONS - 1], rbox[PARTITIONS - 1];
    size_t lcnt[PARTITIONS - 1], rcnt[PARTITIONS - 1];
    float cost[PARTITIONS - 1];
    for (size_t i = 0; i < PARTITIONS - 1; i++) {
      lbox[i] = box_empty();
      rbox[i] = box_empty();
      lcnt[i] = rcnt[i] = 0;
      for (size_t p = 0; p <= i; p++) {
        box_union(lbox[i], pre_box[p]);
        lcnt[i] += pre_bucket[p].size();
      }
      for (size_t p = i + 1; p < PARTITIONS; p++) {
        box_union(rbox[i], pre_box[p]);
        rcnt[i] += pre_bucket[p].size();
      }
      cost[i] = box_surface_area(lbox[i]) * (float)lcnt[i] + box_surface_area(rbox[i]) * (float)rcnt[i];
    }
    size_t best = 0;
    float best_cost = F_INF;
    for (size_t i = 0; i < PARTITIONS - 1; i++) {
      if (cost[i] < best_cost) {
        best_cost = cost[i];
        best = i;
      }
    }
    size_t ptr = s;
    for (size_t p = 0; p < PARTITIONS; p++)
      for (size_t v : pre_bucket[p]) idx[ptr++] = v;
    Split r;
    r.lb = lbox[best];
    r.ls = s;
    r.le = s + lcnt[best];
    r.axis = axis;
    r.rb = rbox[best];
    r.rs = s + lcnt[best];
    r.re = e;
    return r;
  }

  size_t build(size_t depth) {
    FlatNode node = nodes.back();
    if (!opt.should_continue(node.end - node.start, depth)) return 1;
    Split sp = sah_split(node);
    size_t node_index = nodes.size() - 1;
    nodes.push_back(FlatNode{sp.lb, sp.ls, sp.le, nodes.size(), false, 0, 0});
    size_t left_count = build(depth + 1);
    nodes.push_back(FlatNode{sp.rb, sp.rs, sp.re, nodes.size(), false, 0, 0});
    size_t right_count = build(depth + 1);
    nodes[node_index].has_child = true;
    nodes[node_index].left_count = left_count;
    nodes[node_index].split_axis = sp.axis;
    return left_count + right_count + 1;
  }
};

struct FlattenBVH {
  std::vector<FlatNode> nodes;
  std::vector<size_t> sorted_primitive_index;
  BuildStats stats;
};

static FlattenBVH flatten_bvh_new(const std::vector<Box3>& boxes, const BuildOption& opt) {
  FlattenBVH out;
  std::vector<BuildPrimitive> prims(boxes.size());
  std::vector<size_t> idx(boxes.size());
  for (size_t i = 0; i < boxes.size(); i++) {
    idx[i] = i;
    prims[i].bounding = boxes[i];
    prims[i].center = box_center(boxes[i]);
  }
  Box3 root = bounding_from_build_source(idx, prims, 0, idx.size());
  out.nodes.push_back(FlatNode{root, 0, idx.size(), 0, false, 0, 0});
  SahBuilder b{prims, idx, out.nodes, opt, {}, {}, {}};
  b.build(0);
  out.sorted_primitive_index = std::move(idx);
  out.stats = b.stats;
  return out;
}

static std::vector<std::pair<uint32_t, uint32_t>> compute_bvh_next(const std::vector<FlatNode>& nodes) {
  std::vector<std::pair<uint32_t, uint32_t>> result;
  result.reserve(nodes.size());
  std::vector<uint32_t> next_stack;
  for (const FlatNode& n : nodes) {
    if (!next_stack.empty() && next_stack.back() == (uint32_t)n.self_index) next_stack.pop_back();
    uint32_t miss = next_stack.empty() ? INVALID_NEXT : next_stack.back();
    if (n.has_child) {
      uint32_t hit = (uint32_t)(n.self_index + 1);
      next_stack.push_back((uint32_t)(n.self_index + n.left_count + 1));
      result.emplace_back(hit, miss);
    } else {
      result.emplace_back(miss, miss);
    }
  }
  return result;
}

// ---- flattened device layout (naive/mod.rs:22-71) ----
struct DeviceBVHNode {
  float aabb_min[3];
  uint32_t hit_next;
  float aabb_max[3];
  uint32_t miss_next;
  uint32_t content_range[2];
  uint32_t tail[2];
};
static_assert(sizeof(DeviceBVHNode) == 48, "DeviceBVHNode is 48 B");
struct DeviceInstance {
  float transform[16];
  float transform_inv[16];
  uint32_t instance_custom_index;
  uint32_t sbt_offset;
  uint32_t flags;
  uint32_t acceleration_structure_handle;
};
static_assert(sizeof(DeviceInstance) == 144, "instance is 144 B");
struct TlasBounding {
  float world_min[3];
  uint32_t mask;
  float world_max[3];
  uint32_t flags;
};
struct BlasMetaInfo {
  uint32_t tri_root_range[2];
};
struct GeometryMetaInfo {
  uint32_t bvh_root_idx, geometry_idx, primitive_start, geometry_flags;
};

struct GeometrySource {
  uint32_t type;  // 0 triangles, 1 AABBs (accepted and ignored, as the reference does)
  std::vector<float> positions;
  bool indexed;
  std::vector<uint32_t> indices;
  uint32_t flags;
};
struct InstanceSource {
  M4 transform;
  uint32_t custom_index, mask, sbt_offset, flags, blas_handle;
};

static DeviceBVHNode flatten_node(const FlatNode& n, uint32_t hit, uint32_t miss, uint32_t next_offset,
                                  uint32_t primitive_offset) {
  DeviceBVHNode d{};
  d.aabb_min[0] = n.bounding.min.x;
  d.aabb_min[1] = n.bounding.min.y;
  d.aabb_min[2] = n.bounding.min.z;
  d.aabb_max[0] = n.bounding.max.x;
  d.aabb_max[1] = n.bounding.max.y;
  d.aabb_max[2] = n.bounding.max.z;
  d.hit_next = hit != INVALID_NEXT ? hit + next_offset : INVALID_NEXT;
  d.miss_next = miss != INVALID_NEXT ? miss + next_offset : INVALID_NEXT;
  d.content_range[0] = (uint32_t)n.start + primitive_offset;
  d.content_range[1] = (uint32_t)n.end + primitive_offset;
  return d;
}

struct Built {
  std::vector<uint32_t> tlas_binding;
  std::vector<uint32_t> tlas_bvh_root;
  std::vector<DeviceBVHNode> tlas_bvh_forest;
  std::vector<DeviceInstance> tlas_data;
  std::vector<TlasBounding> tlas_bounding;
  std::vector<BlasMetaInfo> blas_meta_info;
  std::vector<GeometryMetaInfo> tri_bvh_root;
  std::vector<DeviceBVHNode> tri_bvh_forest;
  std::vector<uint32_t> indices_redirect;
  std::vector<uint32_t> indices;
  std::vector<float> vertices;
  uint64_t sah_splits = 0, median_fallbacks = 0;
};

struct Ctx {
  std::vector<std::unique_ptr<std::vector<GeometrySource>>> blas;
  std::vector<std::unique_ptr<std::vector<InstanceSource>>> tlas;
  std::vector<uint32_t> binding;
  std::unique_ptr<Built> built;
  BuildOption blas_opt{50, 2}, tlas_opt{50, 10};
  std::string err;
};

static int build_all(Ctx& c) {
  auto B = std::make_unique<Built>();
  std::vector<bool> blas_box_some;
  std::vector<Box3> blas_box;
  struct TriBvh {
    FlattenBVH bvh;
    std::vector<std::pair<uint32_t, uint32_t>> next;
    uint32_t primitive_start, geometry_idx, geometry_flags;
  };
  std::vector<TriBvh> tri_bvh;
  for (auto& bp : c.blas) {
    if (!bp) {
      B->blas_meta_info.push_back(BlasMetaInfo{{0, 0}});
      blas_box_some.push_back(false);
      blas_box.push_back(box_empty());
      continue;
    }
    uint32_t tri_start = (uint32_t)tri_bvh.size();
    uint32_t geometry_idx = 0;
    for (const GeometrySource& g : *bp) {
      Box3 root_box = box_empty();
      if (g.type == 0) {
        uint32_t primitive_start = (uint32_t)(B->indices.size() / 3);
        uint32_t vertex_start = (uint32_t)(B->vertices.size() / 3);
        size_t vcount = g.positions.size() / 3;
        std::vector<uint32_t> iota;
        const std::vector<uint32_t>* ind = &g.indices;
        if (!g.indexed) {
          iota.resize(vcount);
          for (size_t i = 0; i < vcount; i++) iota[i] = (uint32_t)i;
          ind = &iota;
        }
        B->vertices.insert(B->vertices.end(), g.positions.begin(), g.positions.end());
        size_t ntri = ind->size() / 3;
        std::vector<Box3> boxes(ntri);
        for (size_t t = 0; t < ntri; t++) {
          Box3 b = box_empty();
          for (int k = 0; k < 3; k++) {
            uint32_t vi = (*ind)[t * 3 + k];
            if (vi >= vcount) {
              c.err = "index out of range";
              return -1;
            }
            box_expand_point(b, v3(g.positions[vi * 3], g.positions[vi * 3 + 1], g.positions[vi * 3 + 2]));
          }
          boxes[t] = b;
        }
        TriBvh tb;
        tb.bvh = flatten_bvh_new(boxes, c.blas_opt);
        B->sah_splits += tb.bvh.stats.sah_splits;
        B->median_fallbacks += tb.bvh.stats.median_fallbacks;
        box_union(root_box, tb.bvh.nodes[0].bounding);
        tb.next = compute_bvh_next(tb.bvh.nodes);
        uint32_t raw_primitive_start = (uint32_t)(B->indices.size() / 3);
        for (size_t p : tb.bvh.sorted_primitive_index) B->indices_redirect.push_back(raw_primitive_start + (uint32_t)p);
        for (size_t t = 0; t < ntri; t++)
          for (int k = 0; k < 3; k++) B->indices.push_back(vertex_start + (*ind)[t * 3 + k]);
        tb.primitive_start = primitive_start;
        tb.geometry_idx = geometry_idx;
        tb.geometry_flags = g.flags;
        tri_bvh.push_back(std::move(tb));
      }
      // reference quirk (naive/mod.rs:239): one blas_box entry per geometry
      blas_box_some.push_back(true);
      blas_box.push_back(root_box);
      geometry_idx++;
    }
    B->blas_meta_info.push_back(BlasMetaInfo{{tri_start, (uint32_t)tri_bvh.size()}});
  }
  for (TriBvh& tb : tri_bvh) {
    uint32_t bvh_start = (uint32_t)B->tri_bvh_forest.size();
    B->tri_bvh_root.push_back(GeometryMetaInfo{bvh_start, tb.geometry_idx, tb.primitive_start, tb.geometry_flags});
    for (size_t i = 0; i < tb.bvh.nodes.size(); i++)
      B->tri_bvh_forest.push_back(
          flatten_node(tb.bvh.nodes[i], tb.next[i].first, tb.next[i].second, bvh_start, tb.primitive_start));
  }
  for (auto& tp : c.tlas) {
    if (!tp) {
      B->tlas_bvh_root.push_back(INVALID_NEXT);
      continue;
    }
    uint32_t bvh_start = (uint32_t)B->tlas_bvh_forest.size();
    uint32_t primitive_start = (uint32_t)B->tlas_data.size();
    std::vector<Box3> aabbs;
    for (const InstanceSource& s : *tp) {
      if (s.blas_handle >= blas_box.size() || !blas_box_some[s.blas_handle]) {
        c.err = "instance references a missing BLAS box";
        return -2;
      }
      aabbs.push_back(box_apply_matrix(blas_box[s.blas_handle], s.transform));
    }
    FlattenBVH bvh = flatten_bvh_new(aabbs, c.tlas_opt);
    auto next = compute_bvh_next(bvh.nodes);
    for (size_t box_idx : bvh.sorted_primitive_index) {
      const InstanceSource& s = (*tp)[box_idx];
      uint32_t flags = s.flags;
      if (m3_det(s.transform) < 0.0f) flags ^= GI_TRIANGLE_FLIP_FACING;
      DeviceInstance di{};
      memcpy(di.transform, s.transform.m, 64);
      M4 inv = m4_inverse_or_identity(s.transform);
      memcpy(di.transform_inv, inv.m, 64);
      di.instance_custom_index = s.custom_index;
      di.sbt_offset = s.sbt_offset;
      di.flags = flags;
      di.acceleration_structure_handle = s.blas_handle;
      TlasBounding tb{};
      const Box3& a = aabbs[box_idx];
      tb.world_min[0] = a.min.x;
      tb.world_min[1] = a.min.y;
      tb.world_min[2] = a.min.z;
      tb.world_max[0] = a.max.x;
      tb.world_max[1] = a.max.y;
      tb.world_max[2] = a.max.z;
      tb.mask = s.mask;
      tb.flags = flags;
      B->tlas_data.push_back(di);
      B->tlas_bounding.push_back(tb);
    }
    for (size_t i = 0; i < bvh.nodes.size(); i++)
      B->tlas_bvh_forest.push_back(flatten_node(bvh.nodes[i], next[i].first, next[i].second, bvh_start, primitive_start));
    B->tlas_bvh_root.push_back(bvh_start);
    B->sah_splits += bvh.stats.sah_splits;
    B->median_fallbacks += bvh.stats.median_fallbacks;
  }
  B->tlas_binding = c.binding;
  c.built = std::move(B);
  return 0;
}

// ---- traversal ----
struct Counters {
  uint64_t tri_visit = 0, tri_hit = 0, bvh_visit = 0, bvh_hit = 0, far_assert = 0, bad_tlas = 0;
};

struct RayIn {
  float org[3], tmin, dir[3], tmax;
};
struct HitOut {
  float t, u, v;
  uint32_t prim;
  uint32_t geometry, instance, custom, hit_kind;
};

// RayRange: `near`, shared `far`, per-level scaling (traverse_cpu.rs:251-281).
struct RayRange {
  float near_;
  float* far_;
  float scaling;
  float get_near() const { return near_ * scaling; }
  float get_far() const { return *far_ * scaling; }
};

static inline V3 ld3(const float* p) { return v3(p[0], p[1], p[2]); }

// TraverseBvhIteratorCpu::next
struct BvhIter {
  const DeviceBVHNode* bvh;
  V3 o, d;
  RayRange range;
  uint32_t curr;
  float far_scale;
  uint32_t next(Counters& cn, uint32_t* node_visits) {
    while (curr != INVALID_NEXT) {
      cn.bvh_visit++;
      (*node_visits)++;
      const DeviceBVHNode& n = bvh[curr];
      if (intersect_ray_aabb(o, d, range.get_near(), range.get_far(), ld3(n.aabb_min), ld3(n.aabb_max), far_scale)) {
        uint32_t c0 = curr;
        curr = n.hit_next;
        if (n.hit_next == n.miss_next) {
          cn.bvh_hit++;
          return c0;
        }
      } else {
        curr = n.miss_next;
      }
    }
    return INVALID_NEXT;
  }
};

// anyhit_mode: the any-hit policies offered at the C ABI in place of a user
// EDSL any-hit shader. 0 = accept; 1 = accept and end search; 2 = accept only
// even primitive ids; 3 = accept when bit `tri_idx` (the built triangle index)
// of `mask` is set (a data-driven alpha test).
static inline uint32_t any_hit_policy(uint32_t mode, uint32_t primitive_idx, uint32_t tri_idx, const uint32_t* mask) {
  if (mode == 1) return ANYHIT_ACCEPT | ANYHIT_END_SEARCH;
  if (mode == 2) return (primitive_idx & 1u) ? 0u : ANYHIT_ACCEPT;
  if (mode == 3) return (mask[tri_idx >> 5] >> (tri_idx & 31u)) & 1u ? ANYHIT_ACCEPT : 0u;
  return ANYHIT_ACCEPT;
}

// intersector: 0 the reference's triangle test, 1 the watertight test.
static void traverse(const Built& B, const RayIn& ray, uint32_t tlas_idx, uint32_t ray_flags, uint32_t cull_mask,
                     uint32_t anyhit_mode, HitOut& out, Counters& cn, uint32_t* ray_counts,
                     uint32_t* tri_out = nullptr, const uint32_t* anyhit_mask = nullptr, int intersector = 0) {
  out = HitOut{ray.tmax, 0.0f, 0.0f, INVALID_NEXT, INVALID_NEXT, INVALID_NEXT, INVALID_NEXT, 0};
  uint32_t node_visits = 0, tri_tests = 0;
  bool have = false;
  uint32_t flags = ray_flags;
  float far_cell = ray.tmax;
  RayRange ray_range{ray.tmin, &far_cell, 1.0f};
  V3 ro = ld3(ray.org), rd = ld3(ray.dir);
  const float fs = intersector ? WATERTIGHT_BOX_FAR_SCALE : 1.0f;
  if (tlas_idx >= B.tlas_binding.size() || B.tlas_binding[tlas_idx] >= B.tlas_bvh_root.size()) {
    cn.bad_tlas++;
    if (ray_counts) ray_counts[0] = ray_counts[1] = 0;
    return;
  }
  uint32_t root = B.tlas_bvh_root[B.tlas_binding[tlas_idx]];
  BvhIter tlas_iter{B.tlas_bvh_forest.data(), ro, rd, ray_range, root, fs};
  for (;;) {
    uint32_t hit_idx = tlas_iter.next(cn, &node_visits);
    if (hit_idx == INVALID_NEXT) break;
    const DeviceBVHNode& node = B.tlas_bvh_forest[hit_idx];
    for (uint32_t ti = node.content_range[0]; ti < node.content_range[1]; ti++) {
      const TlasBounding& tb = B.tlas_bounding[ti];
      if (!intersect_ray_aabb(ro, rd, ray.tmin, ray.tmax, ld3(tb.world_min), ld3(tb.world_max), fs)) continue;
      if ((cull_mask & tb.mask) == 0) continue;
      const DeviceInstance& inst = B.tlas_data[ti];
      uint32_t blas_idx = inst.acceleration_structure_handle;
      uint32_t iflags = merge_geometry_instance_flag(flags, inst.flags);
      M4 inv;
      memcpy(inv.m, inst.transform_inv, 64);
      V4 o4 = m4_mul_v4(inv, V4{ro.x, ro.y, ro.z, 1.0f});
      V3 bo = v3(o4.x, o4.y, o4.z) / o4.w;
      V3 bd = m3_mul_v3(inv, rd);
      float distance_scaling = length(bd);
      RayRange blas_range{ray_range.near_, &far_cell, distance_scaling};
      bd = normalize(bd);
      const BlasMetaInfo& bm = B.blas_meta_info[blas_idx];
      if ((iflags & TF_SKIP_TRIANGLES) == 0) {
        for (uint32_t gi = bm.tri_root_range[0]; gi < bm.tri_root_range[1]; gi++) {
          const GeometryMetaInfo& g = B.tri_bvh_root[gi];
          bool pass, is_opaque;
          cull_geometry(iflags, g.geometry_flags, &pass, &is_opaque);
          if (!pass) continue;
          bool cull_enable, cull_back;
          cull_triangle(iflags, &cull_enable, &cull_back);
          BvhIter it{B.tri_bvh_forest.data(), bo, bd, blas_range, g.bvh_root_idx, fs};
          for (;;) {
            uint32_t leaf = it.next(cn, &node_visits);
            if (leaf == INVALID_NEXT) break;
            const DeviceBVHNode& ln = B.tri_bvh_forest[leaf];
            for (uint32_t k = ln.content_range[0]; k < ln.content_range[1]; k++) {
              uint32_t tri_idx = B.indices_redirect[k];
              uint32_t i0 = B.indices[tri_idx * 3], i1 = B.indices[tri_idx * 3 + 1], i2 = B.indices[tri_idx * 3 + 2];
              V3 v0 = ld3(&B.vertices[i0 * 3]), v1 = ld3(&B.vertices[i1 * 3]), v2 = ld3(&B.vertices[i2 * 3]);
              cn.tri_visit++;
              tri_tests++;
              TriResult r = intersector ? intersect_ray_triangle_watertight(bo, bd, blas_range.get_near(),
                                                                            blas_range.get_far(), v0, v1, v2,
                                                                            cull_enable, cull_back)
                                        : intersect_ray_triangle(bo, bd, blas_range.get_near(), blas_range.get_far(),
                                                                 v0, v1, v2, cull_enable, cull_back);
              if (r.s != 0.0f) {
                float distance = r.t / distance_scaling;
                uint32_t primitive_idx = tri_idx - g.primitive_start;
                cn.tri_hit++;
                uint32_t behavior =
                    is_opaque ? ANYHIT_ACCEPT : any_hit_policy(anyhit_mode, primitive_idx, tri_idx, anyhit_mask);
                if (behavior & ANYHIT_ACCEPT) {
                  // RayRange::update_far asserts near <= far <= current far (traverse_cpu.rs:272-276);
                  // the reference aborts when they fail, the oracle counts it and goes on.
                  if (!(ray_range.near_ <= distance) || !(distance <= far_cell)) cn.far_assert++;
                  far_cell = distance;
                  have = true;
                  out.t = distance;
                  out.u = r.u;
                  out.v = r.v;
                  out.prim = primitive_idx;
                  out.geometry = g.geometry_idx;
                  out.instance = ti;
                  out.custom = inst.instance_custom_index;
                  out.hit_kind = (r.s < 0.0f) ? 0xFFu : 0xFEu;
                  if (tri_out) *tri_out = tri_idx;
                  if (iflags & TF_ACCEPT_FIRST_HIT_AND_END_SEARCH) behavior |= ANYHIT_END_SEARCH;
                }
                if (behavior & ANYHIT_END_SEARCH) goto done;
              }
            }
          }
        }
      }
    }
  }
done:
  (void)have;
  if (ray_counts) {
    ray_counts[0] = node_visits;
    ray_counts[1] = tri_tests;
  }
}

// Test infrastructure: does the ray meet a NaN distance anywhere its boxes let
// it reach? The same walk as traverse() with the far held at the ray's tmax
// (every node any walk order could visit) and nothing committed; true when a
// triangle that passes the culling tests gives t = NaN (a zero-area triangle,
// or a ray lying in the triangle's plane). Once such a NaN is committed, every
// later range test of the ray passes, so the reference's own result depends on
// the order in which it meets the triangles.
static bool nan_exposure(const Built& B, const RayIn& ray, uint32_t tlas_idx, uint32_t ray_flags,
                         uint32_t cull_mask) {
  if (tlas_idx >= B.tlas_binding.size() || B.tlas_binding[tlas_idx] >= B.tlas_bvh_root.size()) return false;
  Counters cn;
  uint32_t visits = 0;
  float far_cell = ray.tmax;
  RayRange ray_range{ray.tmin, &far_cell, 1.0f};
  V3 ro = ld3(ray.org), rd = ld3(ray.dir);
  BvhIter tlas_iter{B.tlas_bvh_forest.data(), ro, rd, ray_range, B.tlas_bvh_root[B.tlas_binding[tlas_idx]], 1.0f};
  for (;;) {
    uint32_t hit_idx = tlas_iter.next(cn, &visits);
    if (hit_idx == INVALID_NEXT) break;
    const DeviceBVHNode& node = B.tlas_bvh_forest[hit_idx];
    for (uint32_t ti = node.content_range[0]; ti < node.content_range[1]; ti++) {
      const TlasBounding& tb = B.tlas_bounding[ti];
      if (!intersect_ray_aabb(ro, rd, ray.tmin, ray.tmax, ld3(tb.world_min), ld3(tb.world_max))) continue;
      if ((cull_mask & tb.mask) == 0) continue;
      const DeviceInstance& inst = B.tlas_data[ti];
      uint32_t iflags = merge_geometry_instance_flag(ray_flags, inst.flags);
      if (iflags & TF_SKIP_TRIANGLES) continue;
      M4 inv;
      memcpy(inv.m, inst.transform_inv, 64);
      V4 o4 = m4_mul_v4(inv, V4{ro.x, ro.y, ro.z, 1.0f});
      V3 bo = v3(o4.x, o4.y, o4.z) / o4.w;
      V3 bd = m3_mul_v3(inv, rd);
      RayRange blas_range{ray_range.near_, &far_cell, length(bd)};
      bd = normalize(bd);
      const BlasMetaInfo& bm = B.blas_meta_info[inst.acceleration_structure_handle];
      for (uint32_t gi = bm.tri_root_range[0]; gi < bm.tri_root_range[1]; gi++) {
        const GeometryMetaInfo& g = B.tri_bvh_root[gi];
        bool pass, is_opaque, cull_enable, cull_back;
        cull_geometry(iflags, g.geometry_flags, &pass, &is_opaque);
        if (!pass) continue;
        cull_triangle(iflags, &cull_enable, &cull_back);
        BvhIter it{B.tri_bvh_forest.data(), bo, bd, blas_range, g.bvh_root_idx, 1.0f};
        for (;;) {
          uint32_t leaf = it.next(cn, &visits);
          if (leaf == INVALID_NEXT) break;
          const DeviceBVHNode& ln = B.tri_bvh_forest[leaf];
          for (uint32_t k = ln.content_range[0]; k < ln.content_range[1]; k++) {
            uint32_t tri_idx = B.indices_redirect[k];
            uint32_t i0 = B.indices[tri_idx * 3], i1 = B.indices[tri_idx * 3 + 1], i2 = B.indices[tri_idx * 3 + 2];
            TriResult r = intersect_ray_triangle(bo, bd, blas_range.get_near(), blas_range.get_far(),
                                                 ld3(&B.vertices[i0 * 3]), ld3(&B.vertices[i1 * 3]),
                                                 ld3(&B.vertices[i2 * 3]), cull_enable, cull_back);
            if (r.s != 0.0f && std::isnan(r.t)) return true;
          }
        }
      }
    }
  }
  return false;
}

// FP64 re-evaluation of a reported hit: the same formula in double on the same
// (object-space) triangle, to state the FP32 result's error.
static void eval_fp64(const Built& B, const RayIn& ray, const HitOut& h, double* out3) {
  out3[0] = out3[1] = out3[2] = NAN;
  if (h.prim == INVALID_NEXT || h.instance >= B.tlas_data.size()) return;
  const DeviceInstance& inst = B.tlas_data[h.instance];
  uint32_t blas_idx = inst.acceleration_structure_handle;
  const BlasMetaInfo& bm = B.blas_meta_info[blas_idx];
  const GeometryMetaInfo* g = nullptr;
  for (uint32_t gi = bm.tri_root_range[0]; gi < bm.tri_root_range[1]; gi++)
    if (B.tri_bvh_root[gi].geometry_idx == h.geometry) g = &B.tri_bvh_root[gi];
  if (!g) return;
  uint32_t tri_idx = h.prim + g->primitive_start;
  if ((size_t)tri_idx * 3 + 2 >= B.indices.size()) return;
  double M[16];
  for (int i = 0; i < 16; i++) M[i] = inst.transform_inv[i];
  double o[3] = {ray.org[0], ray.org[1], ray.org[2]}, d[3] = {ray.dir[0], ray.dir[1], ray.dir[2]};
  double bo[4], bd[3];
  for (int r = 0; r < 4; r++) bo[r] = o[0] * M[r] + o[1] * M[4 + r] + o[2] * M[8 + r] + M[12 + r];
  for (int r = 0; r < 3; r++) bo[r] /= bo[3];
  for (int r = 0; r < 3; r++) bd[r] = d[0] * M[r] + d[1] * M[4 + r] + d[2] * M[8 + r];
  double sc = std::sqrt(bd[0] * bd[0] + bd[1] * bd[1] + bd[2] * bd[2]);
  for (int r = 0; r < 3; r++) bd[r] /= sc;
  double v[3][3];
  for (int k = 0; k < 3; k++) {
    uint32_t vi = B.indices[tri_idx * 3 + k];
    for (int r = 0; r < 3; r++) v[k][r] = B.vertices[vi * 3 + r];
  }
  double e1[3], e2[3], n[3];
  for (int r = 0; r < 3; r++) {
    e1[r] = v[1][r] - v[0][r];
    e2[r] = v[2][r] - v[0][r];
  }
  n[0] = e1[1] * e2[2] - e1[2] * e2[1];
  n[1] = e1[2] * e2[0] - e1[0] * e2[2];
  n[2] = e1[0] * e2[1] - e1[1] * e2[0];
  double b = n[0] * bd[0] + n[1] * bd[1] + n[2] * bd[2];
  double a = -(n[0] * (bo[0] - v[0][0]) + n[1] * (bo[1] - v[0][1]) + n[2] * (bo[2] - v[0][2]));
  double t = a / b;
  double w[3];
  for (int r = 0; r < 3; r++) w[r] = bo[r] + t * bd[r] - v[0][r];
  double uu = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  double uv = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
  double vv = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
  double wu = w[0] * e1[0] + w[1] * e1[1] + w[2] * e1[2];
  double wv = w[0] * e2[0] + w[1] * e2[1] + w[2] * e2[2];
  double den = uv * uv - uu * vv;
  out3[0] = t / sc;
  out3[1] = (uv * wv - vv * wu) / den;
  out3[2] = (uv * wu - uu * wv) / den;
}

// ---- wavefront workload: primary -> closest hit -> shadow + diffuse bounce ----
// One pixel of the fixed-function pipeline that the product's wavefront kernels
// run (the first bounce of DeviceReferencePathTracingRenderer,
// scene/rendering/gpu-ray-tracing/src/feature/path_tracing/{ray_gen.rs,ray_hit.rs}):
// pinhole primary ray, closest hit, geometric normal facing the ray, offset
// origin, one any-hit shadow ray to a point light and one cosine-weighted
// diffuse bounce ray.
struct PixelOut {
  uint32_t primary_prim;
  float primary_t;
  uint32_t bounce_prim;
  float bounce_t;
  uint32_t primary_flags;  // bit 0: primary hit
  uint32_t light;          // 0 no shadow ray, 1 light visible, 2 occluded
  float direct;            // max(0, n.l) / |L|^2 when visible, else 0
  uint32_t primary_instance;
};
static_assert(sizeof(PixelOut) == 32, "32 B pixel");

struct Camera {
  V3 origin, forward, right, up;
  float tan_half, aspect;
};

static inline V3 camera_dir(const Camera& c, uint32_t px, uint32_t py, uint32_t W, uint32_t H) {
  float sx = (((float)px + 0.5f) / (float)W * 2.0f - 1.0f) * c.tan_half * c.aspect;
  float sy = (1.0f - ((float)py + 0.5f) / (float)H * 2.0f) * c.tan_half;
  V3 d = v3((c.forward.x + sx * c.right.x) + sy * c.up.x, (c.forward.y + sx * c.right.y) + sy * c.up.y,
            (c.forward.z + sx * c.right.z) + sy * c.up.z);
  return normalize(d);
}

// geometric normal of a hit, in world space: normalize(cross(e1, e2)) of the
// object-space triangle, then normalize(transpose(transform_inv) * n).
static inline V3 world_normal(const Built& B, uint32_t tri_idx, uint32_t inst) {
  uint32_t i0 = B.indices[tri_idx * 3], i1 = B.indices[tri_idx * 3 + 1], i2 = B.indices[tri_idx * 3 + 2];
  V3 v0 = ld3(&B.vertices[i0 * 3]), v1 = ld3(&B.vertices[i1 * 3]), v2 = ld3(&B.vertices[i2 * 3]);
  V3 n = normalize(cross(v1 - v0, v2 - v0));
  const float* m = B.tlas_data[inst].transform_inv;
  V3 w = v3(n.x * m[0] + n.y * m[1] + n.z * m[2], n.x * m[4] + n.y * m[5] + n.z * m[6],
            n.x * m[8] + n.y * m[9] + n.z * m[10]);
  return normalize(w);
}

static const float F32_EPSILON = 1.1920929e-7f;
static const float F32_MAX = 3.40282347e+38f;
static const uint32_t RAY_FLAG_END_SEARCH = 0x04;

static void wavefront_pixel(const Built& B, const Camera& cam, uint32_t W, uint32_t H, uint32_t px, uint32_t py,
                            V3 light, uint32_t sample_index, uint32_t tlas, PixelOut& o, Counters& cn,
                            uint64_t* rays, int intersector = 0, RayIn* rays_out = nullptr) {
  V3 d = camera_dir(cam, px, py, W, H);
  RayIn r{{cam.origin.x, cam.origin.y, cam.origin.z}, 0.0f, {d.x, d.y, d.z}, F_INF};
  HitOut h;
  uint32_t tri = 0;
  if (rays_out) rays_out[0] = r;
  traverse(B, r, tlas, 0, 0xFFu, 0, h, cn, nullptr, &tri, nullptr, intersector);
  rays[0]++;
  o = PixelOut{h.prim, h.t, INVALID_NEXT, F32_MAX, 0u, 0u, 0.0f, h.instance};
  if (h.prim == INVALID_NEXT) return;
  o.primary_flags = 1u;
  V3 p = cam.origin + d * h.t;
  V3 n = world_normal(B, tri, h.instance);
  V3 nf = dot(n, d) < 0.0f ? n : v3(-n.x, -n.y, -n.z);
  V3 org = offset_ray_hit(p, nf);
  // shadow ray to the point light
  V3 L = light - org;
  float dist2 = dot(L, L);
  float dist = std::sqrt(dist2);
  V3 ldir = normalize(L);
  float direct = rmax(0.0f, dot(nf, ldir)) / dist2;
  RayIn sr{{org.x, org.y, org.z}, F32_EPSILON, {ldir.x, ldir.y, ldir.z}, dist};
  HitOut sh;
  if (rays_out) rays_out[1] = sr;
  traverse(B, sr, tlas, RAY_FLAG_END_SEARCH, 0xFFu, 0, sh, cn, nullptr, nullptr, nullptr, intersector);
  rays[1]++;
  o.light = sh.prim == INVALID_NEXT ? 1u : 2u;
  o.direct = sh.prim == INVALID_NEXT ? direct : 0.0f;
  // cosine-weighted diffuse bounce
  uint32_t state = xxhash32(px, py, sample_index * 3u);
  float s0 = sample_next(state);
  float s1 = sample_next(state);
  V3 bdir = cosine_sample_in_dir(nf, s0, s1);
  RayIn br{{org.x, org.y, org.z}, F32_EPSILON, {bdir.x, bdir.y, bdir.z}, F32_MAX};
  HitOut bh;
  if (rays_out) rays_out[2] = br;
  traverse(B, br, tlas, 0, 0xFFu, 0, bh, cn, nullptr, nullptr, nullptr, intersector);
  rays[2]++;
  o.bounce_prim = bh.prim;
  o.bounce_t = bh.t;
}

// ---- batched paths: closest hit, diffuse bounce, Russian roulette ----
// The per-path loop of the reference's path tracer (feature/path_tracing/
// ray_gen.rs:89-211 with the closest-hit BRDF sampling of ray_hit.rs:57-103),
// reduced to a constant-albedo diffuse surface under a sky of radiance 1:
// a miss at bounce k ends the path with radiance = throughput; a hit at
// k == max_bounces ends it with 0; otherwise the sampler xxhash32(id, k, seed)
// gives (s0, s1) for a cosine bounce around the facing geometric normal and s2
// for Russian roulette from bounce rr_start on.
static const uint32_t PATH_ESCAPED = 0x80000000u, PATH_ROULETTE = 0x40000000u;

static void path_one(const Built& B, RayIn r, uint32_t id, uint32_t tlas, uint32_t max_bounces, uint32_t rr_start,
                     float albedo, float rr_survive, uint32_t seed, float* out2, uint64_t* seg, Counters& cn) {
  float throughput = 1.0f;
  for (uint32_t k = 0;; k++) {
    HitOut h;
    uint32_t tri = 0;
    traverse(B, r, tlas, 0, 0xFFu, 0, h, cn, nullptr, &tri);
    seg[k]++;
    uint32_t flags;
    if (h.prim == INVALID_NEXT) {
      out2[0] = throughput;
      flags = k | PATH_ESCAPED;
      memcpy(&out2[1], &flags, 4);
      return;
    }
    if (k == max_bounces) {
      out2[0] = 0.0f;
      flags = k;
      memcpy(&out2[1], &flags, 4);
      return;
    }
    uint32_t st = xxhash32(id, k, seed);
    float s0 = sample_next(st);
    float s1 = sample_next(st);
    float s2 = sample_next(st);
    float t_next = throughput * albedo;
    bool survive = true;
    if (k + 1 >= rr_start) {
      survive = s2 < rr_survive;
      t_next = t_next / rr_survive;
    }
    if (!survive) {
      out2[0] = 0.0f;
      flags = k | PATH_ROULETTE;
      memcpy(&out2[1], &flags, 4);
      return;
    }
    V3 d = ld3(r.dir);
    V3 hp = ld3(r.org) + d * h.t;
    V3 n = world_normal(B, tri, h.instance);
    V3 nf = dot(n, d) < 0.0f ? n : v3(-n.x, -n.y, -n.z);
    V3 org = offset_ray_hit(hp, nf);
    V3 dir = cosine_sample_in_dir(nf, s0, s1);
    r = RayIn{{org.x, org.y, org.z}, F32_EPSILON, {dir.x, dir.y, dir.z}, F32_MAX};
    throughput = t_next;
  }
}

}  // namespace orc

using namespace orc;

extern "C" {

struct orc_geometry {
  const float* positions;
  uint32_t vertex_count;
  const uint32_t* indices;
  uint32_t index_count;
  uint32_t flags;
  uint32_t type;
};
struct orc_instance {
  float transform[16];
  uint32_t custom_index, mask, sbt_offset, flags, blas_handle;
};

void* orc_create() { return new Ctx(); }
void orc_destroy(void* c) { delete (Ctx*)c; }
const char* orc_last_error(void* c) { return ((Ctx*)c)->err.c_str(); }

int orc_blas_create(void* cp, const orc_geometry* g, uint32_t n, uint32_t* out) {
  Ctx& c = *(Ctx*)cp;
  auto v = std::make_unique<std::vector<GeometrySource>>();
  for (uint32_t i = 0; i < n; i++) {
    GeometrySource s;
    s.type = g[i].type;
    s.positions.assign(g[i].positions, g[i].positions + (size_t)g[i].vertex_count * 3);
    s.indexed = g[i].indices != nullptr;
    if (s.indexed) s.indices.assign(g[i].indices, g[i].indices + g[i].index_count);
    s.flags = g[i].flags;
    v->push_back(std::move(s));
  }
  c.blas.push_back(std::move(v));
  c.built.reset();
  *out = (uint32_t)(c.blas.size() - 1);
  return 0;
}
int orc_blas_delete(void* cp, uint32_t h) {
  Ctx& c = *(Ctx*)cp;
  if (h >= c.blas.size()) return -1;
  c.blas[h].reset();
  c.built.reset();
  return 0;
}
int orc_tlas_create(void* cp, const orc_instance* inst, uint32_t n, uint32_t* out) {
  Ctx& c = *(Ctx*)cp;
  auto v = std::make_unique<std::vector<InstanceSource>>();
  for (uint32_t i = 0; i < n; i++) {
    InstanceSource s;
    memcpy(s.transform.m, inst[i].transform, 64);
    s.custom_index = inst[i].custom_index;
    s.mask = inst[i].mask;
    s.sbt_offset = inst[i].sbt_offset;
    s.flags = inst[i].flags;
    s.blas_handle = inst[i].blas_handle;
    v->push_back(s);
  }
  c.tlas.push_back(std::move(v));
  c.built.reset();
  *out = (uint32_t)(c.tlas.size() - 1);
  return 0;
}
int orc_tlas_delete(void* cp, uint32_t h) {
  Ctx& c = *(Ctx*)cp;
  if (h >= c.tlas.size()) return -1;
  c.tlas[h].reset();
  c.built.reset();
  return 0;
}
int orc_bind_tlas(void* cp, const uint32_t* h, uint32_t n) {
  Ctx& c = *(Ctx*)cp;
  std::vector<uint32_t> nb(h, h + n);
  if (nb != c.binding) {
    c.binding = nb;
    c.built.reset();
  }
  return 0;
}
int orc_build(void* cp, uint32_t blas_bin, uint32_t blas_depth, uint32_t tlas_bin, uint32_t tlas_depth) {
  Ctx& c = *(Ctx*)cp;
  c.blas_opt = BuildOption{blas_depth, blas_bin};
  c.tlas_opt = BuildOption{tlas_depth, tlas_bin};
  return build_all(c);
}
// stats[0] = SAH splits, stats[1] = median fallbacks
int orc_build_stats(void* cp, uint64_t* stats) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) return -1;
  stats[0] = c.built->sah_splits;
  stats[1] = c.built->median_fallbacks;
  return 0;
}

// which: 0 tlas_binding, 1 tlas_bvh_root, 2 tlas_bvh_forest, 3 tlas_data, 4 tlas_bounding,
// 5 blas_meta_info, 6 tri_bvh_root, 7 tri_bvh_forest, 8 indices_redirect, 9 indices, 10 vertices
size_t orc_get_buffer(void* cp, int which, void* dst, size_t cap) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) return 0;
  const Built& B = *c.built;
  const void* src = nullptr;
  size_t bytes = 0;
#define CASE(i, v)                               \
  case i:                                        \
    src = B.v.data();                            \
    bytes = B.v.size() * sizeof(B.v[0]);         \
    break;
  switch (which) {
    CASE(0, tlas_binding)
    CASE(1, tlas_bvh_root)
    CASE(2, tlas_bvh_forest)
    CASE(3, tlas_data)
    CASE(4, tlas_bounding)
    CASE(5, blas_meta_info)
    CASE(6, tri_bvh_root)
    CASE(7, tri_bvh_forest)
    CASE(8, indices_redirect)
    CASE(9, indices)
    CASE(10, vertices)
    default:
      return 0;
  }
#undef CASE
  if (dst && cap >= bytes && bytes) memcpy(dst, src, bytes);
  return bytes;
}

// Trace `n` rays with `threads` host threads. `tlas_idx` may be null (then
// `tlas_uniform` is used for every ray). `ray_counts` (nullable) receives
// [node visits, triangle tests] per ray; `totals` receives tri_visit, tri_hit,
// bvh_visit, bvh_hit, far_assert, bad_tlas. Returns elapsed seconds of the
// traversal loop in *seconds (nullable). intersector: 0 the reference's
// triangle test, 1 the watertight test.
int orc_trace(void* cp, const RayIn* rays, uint32_t n, const uint32_t* tlas_idx, uint32_t tlas_uniform,
              uint32_t ray_flags, uint32_t cull_mask, uint32_t anyhit_mode, const uint32_t* anyhit_mask, HitOut* out,
              uint32_t* ray_counts, uint64_t* totals, int threads, double* seconds, int intersector) {
  if (anyhit_mode == 3 && !anyhit_mask) return -1;
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  if (threads < 1) threads = 1;
  std::vector<Counters> cn(threads);
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    uint32_t s = (uint32_t)((uint64_t)n * w / threads), e = (uint32_t)((uint64_t)n * (w + 1) / threads);
    for (uint32_t i = s; i < e; i++)
      traverse(B, rays[i], tlas_idx ? tlas_idx[i] : tlas_uniform, ray_flags, cull_mask, anyhit_mode, out[i], cn[w],
               ray_counts ? ray_counts + 2 * (size_t)i : nullptr, nullptr, anyhit_mask, intersector);
  };
  if (threads == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int w = 0; w < threads; w++) th.emplace_back(work, w);
    for (auto& t : th) t.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (totals) {
    for (int k = 0; k < 6; k++) totals[k] = 0;
    for (auto& x : cn) {
      totals[0] += x.tri_visit;
      totals[1] += x.tri_hit;
      totals[2] += x.bvh_visit;
      totals[3] += x.bvh_hit;
      totals[4] += x.far_assert;
      totals[5] += x.bad_tlas;
    }
  }
  return 0;
}

// out[i] = 1 when ray i can meet a NaN distance (nan_exposure).
int orc_nan_exposure(void* cp, const RayIn* rays, uint32_t n, const uint32_t* tlas_idx, uint32_t tlas_uniform,
                     uint32_t ray_flags, uint32_t cull_mask, uint8_t* out, int threads) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  if (threads < 1) threads = 1;
  auto work = [&](int w) {
    uint32_t s = (uint32_t)((uint64_t)n * w / threads), e = (uint32_t)((uint64_t)n * (w + 1) / threads);
    for (uint32_t i = s; i < e; i++)
      out[i] = nan_exposure(B, rays[i], tlas_idx ? tlas_idx[i] : tlas_uniform, ray_flags, cull_mask) ? 1 : 0;
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  return 0;
}

// Test infrastructure: how far a reported hit lies from its triangle's edges,
// against how far the reference's f32 formula can misplace the hit point.
// out2 = [d, b] per ray: d = FP64 distance (object space) from the ray's
// intersection with the triangle's plane to the nearest edge line of the
// triangle, negative when the point lies outside it; b = 32 * 2^-24 *
// max(t, |o - v0|) / |cos theta| + 1e-4 * (smallest altitude), the f32 position
// error bound of the plane-distance formula (its t is a quotient whose
// relative error grows as 1/|cos theta| for grazing rays) plus a floor of
// 1e-4 in barycentric terms. NaN for misses.
static void edge_margin(const Built& B, const RayIn& ray, const HitOut& h, double* out2) {
  out2[0] = out2[1] = NAN;
  if (h.prim == INVALID_NEXT || h.instance >= B.tlas_data.size()) return;
  const DeviceInstance& inst = B.tlas_data[h.instance];
  const BlasMetaInfo& bm = B.blas_meta_info[inst.acceleration_structure_handle];
  const GeometryMetaInfo* g = nullptr;
  for (uint32_t gi = bm.tri_root_range[0]; gi < bm.tri_root_range[1]; gi++)
    if (B.tri_bvh_root[gi].geometry_idx == h.geometry) g = &B.tri_bvh_root[gi];
  if (!g) return;
  uint32_t tri_idx = h.prim + g->primitive_start;
  if ((size_t)tri_idx * 3 + 2 >= B.indices.size()) return;
  double M[16];
  for (int i = 0; i < 16; i++) M[i] = inst.transform_inv[i];
  double bo[4], bd[3];
  for (int r = 0; r < 4; r++) bo[r] = ray.org[0] * M[r] + ray.org[1] * M[4 + r] + ray.org[2] * M[8 + r] + M[12 + r];
  for (int r = 0; r < 3; r++) bo[r] /= bo[3];
  for (int r = 0; r < 3; r++) bd[r] = ray.dir[0] * M[r] + ray.dir[1] * M[4 + r] + ray.dir[2] * M[8 + r];
  double sc = std::sqrt(bd[0] * bd[0] + bd[1] * bd[1] + bd[2] * bd[2]);
  for (int r = 0; r < 3; r++) bd[r] /= sc;
  double v[3][3];
  for (int k = 0; k < 3; k++)
    for (int r = 0; r < 3; r++) v[k][r] = B.vertices[B.indices[tri_idx * 3 + k] * 3 + r];
  auto sub = [](const double* a, const double* b, double* o) { for (int r = 0; r < 3; r++) o[r] = a[r] - b[r]; };
  auto dotd = [](const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
  auto crossd = [](const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  double e1[3], e2[3], n[3], w0[3];
  sub(v[1], v[0], e1);
  sub(v[2], v[0], e2);
  crossd(e1, e2, n);
  double nn = std::sqrt(dotd(n, n));
  if (!(nn > 0.0)) return;
  sub(bo, v[0], w0);
  double bdn = dotd(n, bd);
  double t = -dotd(n, w0) / bdn;
  double p[3];
  for (int r = 0; r < 3; r++) p[r] = bo[r] + t * bd[r];
  // signed distance to each edge line within the plane: cross(edge, p - start) . n / (|edge| |n|)
  double dist = INFINITY, min_alt = INFINITY;
  for (int k = 0; k < 3; k++) {
    const double* a = v[k];
    const double* b = v[(k + 1) % 3];
    double e[3], ap[3], c[3];
    sub(b, a, e);
    sub(p, a, ap);
    crossd(e, ap, c);
    double le = std::sqrt(dotd(e, e));
    double dk = dotd(c, n) / (le * nn);
    dist = std::min(dist, dk);
    min_alt = std::min(min_alt, nn / le);
  }
  double cos_t = std::fabs(bdn) / nn;
  double reach = std::max(std::fabs(t), std::sqrt(dotd(w0, w0)));
  out2[0] = dist;
  out2[1] = 32.0 * std::ldexp(1.0, -24) * reach / std::max(cos_t, 1e-30) + 1e-4 * min_alt;
}

int orc_edge_margin(void* cp, const RayIn* rays, uint32_t n, const HitOut* hits, double* out) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) return -1;
  for (uint32_t i = 0; i < n; i++) edge_margin(*c.built, rays[i], hits[i], out + 2 * (size_t)i);
  return 0;
}

// FP64 re-evaluation of each hit: out = [t, u, v] per ray in double (NaN for misses).
int orc_eval_fp64(void* cp, const RayIn* rays, uint32_t n, const HitOut* hits, double* out) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) return -1;
  for (uint32_t i = 0; i < n; i++) eval_fp64(*c.built, rays[i], hits[i], out + 3 * (size_t)i);
  return 0;
}

// FP64 brute-force closest hit over every triangle of every instance of the
// bound TLAS `tlas_uniform`, no culling, no BVH: the truth the FP32 results are
// measured against on small scenes. out = [t, u, v, prim, instance] per ray.
int orc_bruteforce_fp64(void* cp, const RayIn* rays, uint32_t n, uint32_t tlas_uniform, double* out, int threads) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) return -1;
  const Built& B = *c.built;
  if (tlas_uniform >= B.tlas_binding.size()) return -2;
  uint32_t handle = B.tlas_binding[tlas_uniform];
  if (handle >= c.tlas.size() || !c.tlas[handle]) return -3;
  // instance slots of this TLAS in tlas_data: contiguous, starting at the root node's content start
  uint32_t root = B.tlas_bvh_root[handle];
  uint32_t s0 = B.tlas_bvh_forest[root].content_range[0], s1 = B.tlas_bvh_forest[root].content_range[1];
  if (threads < 1) threads = 1;
  auto work = [&](int w) {
    uint32_t s = (uint32_t)((uint64_t)n * w / threads), e = (uint32_t)((uint64_t)n * (w + 1) / threads);
    for (uint32_t i = s; i < e; i++) {
      const RayIn& ray = rays[i];
      double best_t = INFINITY, bu = NAN, bv = NAN, bp = -1, bi = -1;
      for (uint32_t ti = s0; ti < s1; ti++) {
        const DeviceInstance& inst = B.tlas_data[ti];
        double M[16];
        for (int k = 0; k < 16; k++) M[k] = inst.transform_inv[k];
        double bo[4], bd[3];
        for (int r = 0; r < 4; r++)
          bo[r] = ray.org[0] * M[r] + ray.org[1] * M[4 + r] + ray.org[2] * M[8 + r] + M[12 + r];
        for (int r = 0; r < 3; r++) bo[r] /= bo[3];
        for (int r = 0; r < 3; r++) bd[r] = ray.dir[0] * M[r] + ray.dir[1] * M[4 + r] + ray.dir[2] * M[8 + r];
        double sc = std::sqrt(bd[0] * bd[0] + bd[1] * bd[1] + bd[2] * bd[2]);
        for (int r = 0; r < 3; r++) bd[r] /= sc;
        const BlasMetaInfo& bm = B.blas_meta_info[inst.acceleration_structure_handle];
        for (uint32_t gi = bm.tri_root_range[0]; gi < bm.tri_root_range[1]; gi++) {
          const GeometryMetaInfo& g = B.tri_bvh_root[gi];
          const DeviceBVHNode& rn = B.tri_bvh_forest[g.bvh_root_idx];
          for (uint32_t k = rn.content_range[0]; k < rn.content_range[1]; k++) {
            uint32_t tri_idx = B.indices_redirect[k];
            double v[3][3];
            for (int q = 0; q < 3; q++) {
              uint32_t vi = B.indices[tri_idx * 3 + q];
              for (int r = 0; r < 3; r++) v[q][r] = B.vertices[vi * 3 + r];
            }
            double e1[3], e2[3];
            for (int r = 0; r < 3; r++) {
              e1[r] = v[1][r] - v[0][r];
              e2[r] = v[2][r] - v[0][r];
            }
            double nx = e1[1] * e2[2] - e1[2] * e2[1], ny = e1[2] * e2[0] - e1[0] * e2[2],
                   nz = e1[0] * e2[1] - e1[1] * e2[0];
            double b = nx * bd[0] + ny * bd[1] + nz * bd[2];
            if (b == 0.0) continue;
            double t = -(nx * (bo[0] - v[0][0]) + ny * (bo[1] - v[0][1]) + nz * (bo[2] - v[0][2])) / b;
            double tw = t / sc;
            if (!(tw >= ray.tmin && tw <= ray.tmax)) continue;
            double w[3];
            for (int r = 0; r < 3; r++) w[r] = bo[r] + t * bd[r] - v[0][r];
            double uu = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
            double uv = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
            double vv = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
            double wu = w[0] * e1[0] + w[1] * e1[1] + w[2] * e1[2];
            double wv = w[0] * e2[0] + w[1] * e2[1] + w[2] * e2[2];
            double den = uv * uv - uu * vv;
            double u = (uv * wv - vv * wu) / den, vb = (uv * wu - uu * wv) / den;
            if (u < 0 || u > 1 || vb < 0 || u + vb > 1) continue;
            if (tw < best_t) {
              best_t = tw;
              bu = u;
              bv = vb;
              bp = tri_idx - g.primitive_start;
              bi = ti;
            }
          }
        }
      }
      double* o = out + 5 * (size_t)i;
      o[0] = best_t;
      o[1] = bu;
      o[2] = bv;
      o[3] = bp;
      o[4] = bi;
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  return 0;
}

// Direct access to the intersectors for known-answer tests.
int orc_intersect_triangle(const float* o, const float* d, float near_, float far_, const float* v0,
                           const float* v1, const float* v2, int cull_enable, int cull_back, float* out4) {
  TriResult r = intersect_ray_triangle(ld3(o), ld3(d), near_, far_, ld3(v0), ld3(v1), ld3(v2), cull_enable != 0,
                                       cull_back != 0);
  out4[0] = r.s;
  out4[1] = r.t;
  out4[2] = r.u;
  out4[3] = r.v;
  return 0;
}
int orc_intersect_aabb(const float* o, const float* d, float tmin, float tmax, const float* bmin, const float* bmax) {
  return intersect_ray_aabb(ld3(o), ld3(d), tmin, tmax, ld3(bmin), ld3(bmax)) ? 1 : 0;
}
// select_nth_unstable_by on f32 keys (is_less = partial_cmp == Less, NaN -> Less);
// permutes `idx` in place. Exposed to pin the restated Rust selection.
int orc_select_nth(const float* keys, uint64_t* idx, size_t len, size_t index) {
  auto less = [keys](const uint64_t& a, const uint64_t& b) {
    float ka = keys[a], kb = keys[b];
    if (std::isnan(ka) || std::isnan(kb)) return true;
    return ka < kb;
  };
  RustSelect<uint64_t, decltype(less)> sel{less};
  sel.select_nth(idx, len, index);
  return 0;
}


// Wavefront workload over pixel rows [row0, row1) of a W x H image. cam = 14
// floats (origin, forward, right, up, tan_half, aspect). out receives W*(row1-row0)
// 32 B pixel records; rays3 receives [primary, shadow, bounce] rays traced.
int orc_wavefront_shadow_bounce(void* cp, const float* cam, uint32_t W, uint32_t H, const float* light,
                                uint32_t sample_index, uint32_t tlas, uint32_t row0, uint32_t row1, void* out,
                                uint64_t* rays3, int threads, double* seconds, int intersector) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  Camera cm{ld3(cam), ld3(cam + 3), ld3(cam + 6), ld3(cam + 9), cam[12], cam[13]};
  V3 L = ld3(light);
  if (row1 > H) row1 = H;
  if (row0 > row1) row0 = row1;
  if (threads < 1) threads = 1;
  uint32_t rows = row1 - row0;
  PixelOut* po = (PixelOut*)out;
  std::vector<Counters> cn(threads);
  std::vector<uint64_t> rc(3 * (size_t)threads, 0);
  std::atomic<uint32_t> next_row{row0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    for (;;) {
      uint32_t y = next_row.fetch_add(1);
      if (y >= row1) break;
      for (uint32_t x = 0; x < W; x++)
        wavefront_pixel(B, cm, W, H, x, y, L, sample_index, tlas, po[(size_t)(y - row0) * W + x], cn[w],
                        &rc[3 * (size_t)w], intersector);
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (rays3) {
    rays3[0] = rays3[1] = rays3[2] = 0;
    for (int w = 0; w < threads; w++)
      for (int k = 0; k < 3; k++) rays3[k] += rc[3 * (size_t)w + k];
  }
  (void)rows;
  return 0;
}


// The rays of the given pixels of the same workload (for classifying
// differences of those rays' results): rays[3 * i] = primary, rays[3 * i + 1]
// = shadow, rays[3 * i + 2] = bounce ray of pixel pixels[i] (y * W + x);
// has[i] = 1 when the pixel's primary ray hit (the shadow and bounce rays
// exist), else 0 and those two rays zero.
int orc_wavefront_pixel_rays(void* cp, const float* cam, uint32_t W, uint32_t H, const float* light,
                                 uint32_t sample_index, uint32_t tlas, const uint32_t* pixels, uint32_t n,
                                 RayIn* rays, uint8_t* has, int threads, int intersector) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  Camera cm{ld3(cam), ld3(cam + 3), ld3(cam + 6), ld3(cam + 9), cam[12], cam[13]};
  V3 L = ld3(light);
  if (threads < 1) threads = 1;
  auto work = [&](int w) {
    Counters cn;
    uint64_t rc3[3] = {0, 0, 0};
    uint32_t s = (uint32_t)((uint64_t)n * w / threads), e = (uint32_t)((uint64_t)n * (w + 1) / threads);
    for (uint32_t i = s; i < e; i++) {
      PixelOut po;
      RayIn* r3 = rays + 3 * (size_t)i;
      std::memset(r3, 0, 3 * sizeof(RayIn));
      const uint32_t x = pixels[i] % W, y = pixels[i] / W;
      wavefront_pixel(B, cm, W, H, x, y, L, sample_index, tlas, po, cn, rc3, intersector, r3);
      has[i] = po.primary_flags & 1u;
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  return 0;
}

// One AO sample for rows [row0, row1) of a width x height frame (see
// orc_ao.h); image: width * height RGBA8 texels, updated in place. rays2
// receives the camera and occlusion rays traced.
int orc_ao_render(void* cp, const float* vp_inv, const float* cam, uint32_t W, uint32_t H, uint32_t sample_count,
                  uint32_t tlas, const float* normals, uint32_t* image, uint32_t row0, uint32_t row1, int threads,
                  uint64_t* rays2, double* seconds) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  AoView A;
  memcpy(A.vp_inv, vp_inv, sizeof(A.vp_inv));
  memcpy(A.cam, cam, sizeof(A.cam));
  A.width = W;
  A.height = H;
  A.sample_count = sample_count;
  if (row1 > H) row1 = H;
  if (row0 > row1) row0 = row1;
  if (threads < 1) threads = 1;
  std::vector<Counters> cn(threads);
  std::vector<uint64_t> rc(2 * (size_t)threads, 0);
  std::atomic<uint32_t> next_row{row0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    for (;;) {
      const uint32_t y = next_row.fetch_add(1);
      if (y >= row1) break;
      for (uint32_t x = 0; x < W; x++) {
        V3 o, d;
        ao_camera_ray(A, x, y, &o, &d);
        RayIn r{{o.x, o.y, o.z}, F32_EPSILON, {d.x, d.y, d.z}, F32_MAX};
        HitOut h;
        uint32_t tri = 0;
        traverse(B, r, tlas, 0x10u, 0xFFFFFFFFu, 0, h, cn[w], nullptr, &tri);
        rc[2 * (size_t)w]++;
        float payload = 1.0f;
        if (h.prim != INVALID_NEXT) {
          const V3 hit = o + d * h.t;
          const V3 n = ao_shading_normal(B.indices.data(), B.vertices.data(), normals,
                                         B.tlas_data[h.instance].transform_inv, tri, h.u, h.v, o, hit);
          const V3 dir = ao_direction(n, sample_count);
          RayIn sr{{hit.x, hit.y, hit.z}, 0.01f, {dir.x, dir.y, dir.z}, 100.0f};
          HitOut sh;
          traverse(B, sr, tlas, RAY_FLAG_END_SEARCH, 0xFFFFFFFFu, 0, sh, cn[w], nullptr);
          rc[2 * (size_t)w + 1]++;
          payload = sh.prim != INVALID_NEXT ? 0.0f : 1.0f;
        }
        uint32_t& texel = image[(size_t)y * W + x];
        texel = ao_accumulate(texel, sample_count, payload);
      }
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (rays2) {
    rays2[0] = rays2[1] = 0;
    for (int w = 0; w < threads; w++) {
      rays2[0] += rc[2 * (size_t)w];
      rays2[1] += rc[2 * (size_t)w + 1];
    }
  }
  return 0;
}

// One path-tracing sample for rows [row0, row1) of a width x height frame (see
// orc_pt.h); image: width * height RGBA8 texels, updated in place; radiance
// (nullable): 4 floats per pixel (HDR radiance of the sample, core rays of its
// path). rays2 receives the core and shadow rays traced.
int orc_pt_render(void* cp, const float* vp_inv, const float* cam, uint32_t W, uint32_t H, uint32_t sample_count,
                  uint32_t tlas, const float* normals, const PtScene* scene, uint32_t* image, float* radiance,
                  uint32_t row0, uint32_t row1, int intersector, int threads, uint64_t* rays2, double* seconds) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  const PtScene& S = *scene;
  AoView A;
  memcpy(A.vp_inv, vp_inv, sizeof(A.vp_inv));
  memcpy(A.cam, cam, sizeof(A.cam));
  A.width = W;
  A.height = H;
  A.sample_count = sample_count;
  if (row1 > H) row1 = H;
  if (row0 > row1) row0 = row1;
  if (threads < 1) threads = 1;
  std::vector<Counters> cn(threads);
  std::vector<uint64_t> rc(2 * (size_t)threads, 0);
  std::atomic<uint32_t> next_row{row0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    for (;;) {
      const uint32_t y = next_row.fetch_add(1);
      if (y >= row1) break;
      for (uint32_t x = 0; x < W; x++) {
        V3 o, d;
        ao_camera_ray(A, x, y, &o, &d);
        V3 throughput = v3(1.0f, 1.0f, 1.0f), rad = v3(0.0f, 0.0f, 0.0f);
        uint32_t depth = 0, core = 0;
        while (depth < S.max_depth) {
          RayIn r{{o.x, o.y, o.z}, F32_EPSILON, {d.x, d.y, d.z}, F32_MAX};
          HitOut h;
          uint32_t tri = 0;
          traverse(B, r, tlas, 0x10u, 0xFFFFFFFFu, 0, h, cn[w], nullptr, &tri, nullptr, intersector);
          rc[2 * (size_t)w]++;
          core++;
          if (h.prim == INVALID_NEXT) {
            const V3 s = pt_miss(S, d);
            rad = v3((throughput.x * s.x + 0.0f) + rad.x, (throughput.y * s.y + 0.0f) + rad.y,
                     (throughput.z * s.z + 0.0f) + rad.z);
            break;
          }
          // closest hit: light sample, shadow ray
          const V3 hit = o + d * h.t;
          const float* m = B.tlas_data[h.instance].transform_inv;
          const uint32_t i0 = B.indices[3 * (size_t)tri], i1 = B.indices[3 * (size_t)tri + 1],
                         i2 = B.indices[3 * (size_t)tri + 2];
          const float* P = B.vertices.data();
          const V3 pa = v3(P[3 * (size_t)i0], P[3 * (size_t)i0 + 1], P[3 * (size_t)i0 + 2]);
          const V3 pb = v3(P[3 * (size_t)i1], P[3 * (size_t)i1 + 1], P[3 * (size_t)i1 + 2]);
          const V3 pc = v3(P[3 * (size_t)i2], P[3 * (size_t)i2 + 1], P[3 * (size_t)i2 + 2]);
          V3 gn = normalize(normal_mat_mul(m, cross(pa - pb, pa - pc)));
          if (dot(o - hit, gn) < 0.0f) gn = v3(-gn.x, -gn.y, -gn.z);
          const V3 sn = ao_shading_normal(B.indices.data(), P, normals, m, tri, h.u, h.v, o, hit);
          uint32_t ls = xxhash32(x, y, sample_count * 2u);
          const float rnd = sample_next(ls);
          const uint32_t n_lights = S.light_count;
          uint32_t li = (uint32_t)std::floor(rnd * (float)n_lights);
          const bool light_ok = n_lights != 0u;
          if (li == n_lights && light_ok) li = li - 1u;
          const float pmf = n_lights == 0u ? 0.0f : 1.0f / (float)n_lights;
          V3 illum = v3(0.0f, 0.0f, 0.0f), dir = illum;
          if (light_ok) {
            illum = v3(S.lights[li].illuminance[0], S.lights[li].illuminance[1], S.lights[li].illuminance[2]);
            dir = v3(S.lights[li].direction[0], S.lights[li].direction[1], S.lights[li].direction[2]);
          }
          const V3 ldir = v3(-dir.x, -dir.y, -dir.z);
          const float pdf_l = 1.0f * pmf;
          V3 lrad = light_ok ? v3(illum.x / pdf_l, illum.y / pdf_l, illum.z / pdf_l) : v3(0.0f, 0.0f, 0.0f);
          const V3 origin = offset_ray_hit(hit, gn);
          if (light_ok) {
            RayIn sr{{origin.x, origin.y, origin.z}, F32_EPSILON, {ldir.x, ldir.y, ldir.z}, F32_MAX};
            HitOut sh;
            traverse(B, sr, tlas, RAY_FLAG_END_SEARCH, 0xFFFFFFFFu, 0, sh, cn[w], nullptr, nullptr, nullptr,
                     intersector);
            rc[2 * (size_t)w + 1]++;
            if (sh.prim != INVALID_NEXT) lrad = v3(0.0f, 0.0f, 0.0f);
          }
          // map: BRDF sample and the direct light through the BRDF
          const V3 view = v3(-d.x, -d.y, -d.z);
          const PtSurface su = pt_surface(S, h.custom);
          uint32_t bs = xxhash32(x, y, sample_count * 3u);
          V3 brdf;
          float pdf;
          const V3 sdir = pt_sample(su, view, sn, bs, &brdf, &pdf);
          const V3 brdf_l = pt_bsdf(su, view, ldir, sn);
          const float light_dot = std::fabs(dot(sn, ldir));
          const V3 sampled = v3((light_dot * brdf_l.x) * lrad.x, (light_dot * brdf_l.y) * lrad.y,
                                (light_dot * brdf_l.z) * lrad.z);
          // ray generation, hit branch
          if (pdf == 0.0f) depth = S.max_depth;
          depth = depth + 1u;
          const float cosv = dot(sdir, sn);
          const float pdf_c = rmax(pdf, 0.0001f);
          throughput = v3(((throughput.x * cosv) * brdf.x) / pdf_c, ((throughput.y * cosv) * brdf.y) / pdf_c,
                          ((throughput.z * cosv) * brdf.z) / pdf_c);
          rad = v3(throughput.x * sampled.x + rad.x, throughput.y * sampled.y + rad.y,
                   throughput.z * sampled.z + rad.z);
          o = origin;
          d = sdir;
        }
        const size_t pix = (size_t)y * W + x;
        image[pix] = pt_accumulate(image[pix], sample_count, pt_tone_map(S, rad));
        if (radiance) {
          radiance[4 * pix] = rad.x;
          radiance[4 * pix + 1] = rad.y;
          radiance[4 * pix + 2] = rad.z;
          radiance[4 * pix + 3] = (float)core;
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (rays2) {
    rays2[0] = rays2[1] = 0;
    for (int w = 0; w < threads; w++) {
      rays2[0] += rc[2 * (size_t)w];
      rays2[1] += rc[2 * (size_t)w + 1];
    }
  }
  return 0;
}

// One PT surface query for tests: surface of material index sm_id under the
// scene's tables, BRDF importance sample from `seed` at view v / normal n
// (out: direction, bsdf, pdf), bsdf(v, l2, n) and pdf(v, l2, n) of a second
// direction (out2: bsdf, pdf), and the surface (out3: albedo, f0, alpha, estimate).
int orc_pt_surface_query(const PtScene* scene, uint32_t sm_id, const float* v, const float* n, uint32_t seed,
                         const float* l2, float* out, float* out2, float* out3) {
  const PtSurface su = pt_surface(*scene, sm_id);
  const V3 vv = v3(v[0], v[1], v[2]), nn = v3(n[0], n[1], n[2]);
  uint32_t st = seed;
  V3 brdf;
  float pdf;
  const V3 l = pt_sample(su, vv, nn, st, &brdf, &pdf);
  out[0] = l.x, out[1] = l.y, out[2] = l.z, out[3] = brdf.x, out[4] = brdf.y, out[5] = brdf.z, out[6] = pdf;
  const V3 ll = v3(l2[0], l2[1], l2[2]);
  const V3 b2 = pt_bsdf(su, vv, ll, nn);
  out2[0] = b2.x, out2[1] = b2.y, out2[2] = b2.z, out2[3] = pt_pdf(su, vv, ll, nn);
  out3[0] = su.albedo.x, out3[1] = su.albedo.y, out3[2] = su.albedo.z, out3[3] = su.f0.x, out3[4] = su.f0.y,
  out3[5] = su.f0.z, out3[6] = su.alpha, out3[7] = su.estimate;
  return 0;
}

// Elementwise fixed-polynomial functions for tests: op 0 atan, 1 log2, 2 exp2,
// 3 pow(x, 2.2), 4 tone map of (x, x, x) with tone map `arg` and exposure 1 (x channel).
int orc_pt_math(int op, uint32_t arg, const float* x, float* y, uint64_t n) {
  PtScene S{};
  S.tone_map = arg;
  S.exposure = 1.0f;
  for (uint64_t i = 0; i < n; i++) {
    switch (op) {
      case 0: y[i] = pt_atan(x[i]); break;
      case 1: y[i] = pt_log2(x[i]); break;
      case 2: y[i] = pt_exp2(x[i]); break;
      case 3: y[i] = pt_pow(x[i], 2.2f); break;
      default: y[i] = pt_tone_map(S, v3(x[i], x[i], x[i])).x; break;
    }
  }
  return 0;
}

// Batched paths over n rays (tlas_idx per ray, or tlas_uniform when NULL).
// out = (radiance, depth|flags bits) per ray; seg receives rays traced per
// bounce (max_bounces + 1 entries).
int orc_trace_paths(void* cp, const RayIn* rays, uint32_t n, const uint32_t* tlas_idx, uint32_t tlas_uniform,
                    uint32_t max_bounces, uint32_t rr_start, float albedo, float rr_survive, uint32_t seed,
                    float* out, uint64_t* seg, int threads, double* seconds) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  if (max_bounces > 16) return -1;
  const Built& B = *c.built;
  if (threads < 1) threads = 1;
  std::vector<Counters> cn(threads);
  std::vector<uint64_t> sg((size_t)threads * 17, 0);
  std::atomic<uint32_t> next{0};
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](int w) {
    for (;;) {
      uint32_t s = next.fetch_add(256);
      if (s >= n) break;
      uint32_t e = s + 256 < n ? s + 256 : n;
      for (uint32_t i = s; i < e; i++)
        path_one(B, rays[i], i, tlas_idx ? tlas_idx[i] : tlas_uniform, max_bounces, rr_start, albedo, rr_survive,
                 seed, out + 2 * (size_t)i, &sg[17 * (size_t)w], cn[w]);
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  auto t1 = std::chrono::steady_clock::now();
  if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
  if (seg)
    for (uint32_t k = 0; k <= max_bounces; k++) {
      seg[k] = 0;
      for (int w = 0; w < threads; w++) seg[k] += sg[17 * (size_t)w + k];
    }
  return 0;
}


// Segment rays and hit triangles of differentiable paths: a primary ray per
// path followed by up to segments-1 cosine bounces (no roulette), generated as
// in path_one. seg_rays: 32 B per segment (untouched after a miss); seg_tri:
// built triangle index per segment or ~0.
int orc_path_segments(void* cp, const RayIn* rays, uint32_t n, const uint32_t* tlas_idx, uint32_t tlas_uniform,
                      uint32_t segments, uint32_t seed, RayIn* seg_rays, uint32_t* seg_tri, int threads) {
  Ctx& c = *(Ctx*)cp;
  if (!c.built) {
    int rc = build_all(c);
    if (rc) return rc;
  }
  const Built& B = *c.built;
  if (threads < 1) threads = 1;
  std::vector<Counters> cn(threads);
  std::atomic<uint32_t> next{0};
  auto work = [&](int w) {
    for (;;) {
      uint32_t i = next.fetch_add(1);
      if (i >= n) break;
      RayIn r = rays[i];
      uint32_t tlas = tlas_idx ? tlas_idx[i] : tlas_uniform;
      bool alive = true;
      for (uint32_t k = 0; k < segments; k++) {
        size_t seg = (size_t)i * segments + k;
        seg_tri[seg] = INVALID_NEXT;
        if (!alive) continue;
        seg_rays[seg] = r;
        HitOut h;
        uint32_t tri = 0;
        traverse(B, r, tlas, 0, 0xFFu, 0, h, cn[w], nullptr, &tri);
        if (h.prim == INVALID_NEXT) {
          alive = false;
          continue;
        }
        seg_tri[seg] = tri;
        if (k + 1 < segments) {
          uint32_t st = xxhash32(i, k, seed);
          float s0 = sample_next(st);
          float s1 = sample_next(st);
          V3 d = ld3(r.dir);
          V3 hp = ld3(r.org) + d * h.t;
          V3 nn = world_normal(B, tri, h.instance);
          V3 nf = dot(nn, d) < 0.0f ? nn : v3(-nn.x, -nn.y, -nn.z);
          V3 org = offset_ray_hit(hp, nf);
          V3 dir = cosine_sample_in_dir(nf, s0, s1);
          r = RayIn{{org.x, org.y, org.z}, F32_EPSILON, {dir.x, dir.y, dir.z}, F32_MAX};
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int w = 0; w < threads; w++) th.emplace_back(work, w);
  for (auto& t : th) t.join();
  return 0;
}

}  // extern "C"
