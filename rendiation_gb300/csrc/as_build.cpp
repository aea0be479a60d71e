// Host acceleration-structure build for librdn.
//
// Produces the reference's flattened arrays bit for bit (NaiveSahBvhSource::build,
// shader/ray-tracing/src/backend/wavefront_compute/geometry/naive/mod.rs:122-494)
// and, from the same trees, the GB300 layout: 64 B two-child nodes, leaf
// ranges and 64 B precomputed triangles.
//
// Tree construction follows the reference's binned SAH exactly
// (content/space/src/bvh/strategy.rs:11-43,202-284 with SAH::new(4); degenerate
// binning falls back to BalanceTree's median split, strategy.rs:66-87) so that
// node boxes, pre-order numbering and primitive order are identical. The
// implementation is our own: bucket ids are recomputed instead of kept in
// per-bucket vectors, the in-bucket order is kept by a counting scatter, and
// independent subtrees are built on separate host threads and concatenated in
// pre-order.
//
// Must be compiled with -ffp-contract=off: every float expression mirrors the
// reference's f32 operation order.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

#include "device_build.h"
#include "rdn_core.h"
#include "rust_select.h"

namespace rdn {
namespace {

inline float fmin_r(float a, float b) { return std::fmin(a, b); }  // Rust f32::min (NaN-ignoring)
inline float fmax_r(float a, float b) { return std::fmax(a, b); }
inline Box empty_box() {
  const float inf = INFINITY;
  return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}
inline void grow(Box& b, const f3& p) {
  b.lo = {fmin_r(b.lo.x, p.x), fmin_r(b.lo.y, p.y), fmin_r(b.lo.z, p.z)};
  b.hi = {fmax_r(b.hi.x, p.x), fmax_r(b.hi.y, p.y), fmax_r(b.hi.z, p.z)};
}
inline void grow(Box& b, const Box& o) {
  b.lo = {fmin_r(b.lo.x, o.lo.x), fmin_r(b.lo.y, o.lo.y), fmin_r(b.lo.z, o.lo.z)};
  b.hi = {fmax_r(b.hi.x, o.hi.x), fmax_r(b.hi.y, o.hi.y), fmax_r(b.hi.z, o.hi.z)};
}
inline float comp(const f3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
inline float area(const Box& b) {  // 2 * (w*h + w*d + h*d)
  const float w = b.hi.x - b.lo.x, h = b.hi.y - b.lo.y, d = b.hi.z - b.lo.z;
  return 2.0f * (w * h + w * d + h * d);
}
inline int split_axis(const Box& b) {  // Box3::longest_axis
  const float x = b.hi.x - b.lo.x, y = b.hi.y - b.lo.y, z = b.hi.z - b.lo.z;
  if (x > y) return x > z ? 0 : 2;
  return y > z ? 1 : 2;
}
inline size_t bucket_of(float value, float start, float step) {
  // ((value - start) / step).floor() as usize, clamped to the last bucket
  const float f = std::floor((value - start) / step);
  size_t b = (f > 0.0f) ? (f >= 4.0f ? 4 : (size_t)f) : 0;
  return b >= 4 ? 3 : b;
}

// One node of a freshly built tree, in pre-order.
struct TreeNode {
  Box box;
  uint32_t start, end;    // range in the per-tree order array
  uint32_t left_count;    // nodes in the left subtree; 0 for a leaf
  uint32_t depth;
};

struct TreeBuilder {
  const Box* boxes;
  const f3* centers;
  uint32_t* order;    // per-primitive order (the sorted_primitive_index)
  uint32_t* scratch;  // same size as order
  uint32_t bin_size, max_depth;
  std::atomic<uint64_t> sah_splits{0}, fallbacks{0};
  std::atomic<int> spare_threads{0};
  static const uint32_t kParallelMin = 1u << 15;

  Box range_box(uint32_t s, uint32_t e) const {
    Box b = empty_box();
    for (uint32_t i = s; i < e; i++) grow(b, boxes[order[i]]);
    return b;
  }

  // Returns the split position; fills the two child boxes.
  uint32_t split(const Box& nb, uint32_t s, uint32_t e, Box& lb, Box& rb) {
    const int axis = split_axis(nb);
    const float a0 = comp(nb.lo, axis), a1 = comp(nb.hi, axis);
    const float step = (a1 - a0) / 4.0f;
    Box bb[4] = {empty_box(), empty_box(), empty_box(), empty_box()};
    uint32_t cnt[4] = {0, 0, 0, 0};
    for (uint32_t i = s; i < e; i++) {
      const uint32_t p = order[i];
      const size_t b = bucket_of(comp(centers[p], axis), a0, step);
      grow(bb[b], boxes[p]);
      cnt[b]++;
    }
    const int empties = (cnt[0] == 0) + (cnt[1] == 0) + (cnt[2] == 0) + (cnt[3] == 0);
    if (empties == 3) {
      // BalanceTree: median by centre on the same axis, then boxes of both halves
      fallbacks++;
      const uint32_t mid = (e + s) / 2;
      if ((e - s) / 2 != 0) {
        auto less = [this, axis](const uint32_t& a, const uint32_t& b) {
          const float ka = comp(centers[a], axis), kb = comp(centers[b], axis);
          return std::isnan(ka) || std::isnan(kb) || ka < kb;  // partial_cmp(..).unwrap_or(Less)
        };
        RustSelectNth<uint32_t, decltype(less)> sel(less);
        sel.run(order + s, e - s, (e - s) / 2);
      }
      lb = range_box(s, mid);
      rb = range_box(mid, e);
      return mid;
    }
    sah_splits++;
    // candidate i puts buckets 0..=i left; the first strictly cheaper candidate
    // wins, candidate 0 when no cost is below +inf (NaN costs of empty sides never win)
    float best_cost = INFINITY;
    Box best_l = empty_box(), best_r = empty_box();
    uint32_t best_lc = 0;
    for (int i = 0; i < 3; i++) {
      Box l = empty_box(), r = empty_box();
      uint32_t lc = 0, rc = 0;
      for (int p = 0; p <= i; p++) {
        grow(l, bb[p]);
        lc += cnt[p];
      }
      for (int p = i + 1; p < 4; p++) {
        grow(r, bb[p]);
        rc += cnt[p];
      }
      const float cost = area(l) * (float)lc + area(r) * (float)rc;
      if (i == 0 || cost < best_cost) {
        best_l = l;
        best_r = r;
        best_lc = lc;
      }
      if (cost < best_cost) best_cost = cost;
    }
    // stable scatter of the range in bucket order
    uint32_t off[4];
    off[0] = s;
    off[1] = off[0] + cnt[0];
    off[2] = off[1] + cnt[1];
    off[3] = off[2] + cnt[2];
    for (uint32_t i = s; i < e; i++) {
      const uint32_t p = order[i];
      scratch[off[bucket_of(comp(centers[p], axis), a0, step)]++] = p;
    }
    std::memcpy(order + s, scratch + s, (size_t)(e - s) * sizeof(uint32_t));
    lb = best_l;
    rb = best_r;
    return s + best_lc;
  }

  // Appends the subtree rooted at (box, s, e) to `out` in pre-order.
  void build(const Box& box, uint32_t s, uint32_t e, uint32_t depth, std::vector<TreeNode>& out) {
    const size_t me = out.size();
    out.push_back(TreeNode{box, s, e, 0, depth});
    if (!(depth < max_depth && (e - s) > bin_size)) return;
    Box lb, rb;
    const uint32_t m = split(box, s, e, lb, rb);
    const size_t left_begin = out.size();
    bool forked = false;
    std::vector<TreeNode> right;
    std::future<void> fut;
    if ((e - s) >= kParallelMin && spare_threads.fetch_sub(1) > 0) {
      forked = true;
      fut = std::async(std::launch::async, [&]() {
        build(rb, m, e, depth + 1, right);
        spare_threads.fetch_add(1);
      });
    } else if ((e - s) >= kParallelMin) {
      spare_threads.fetch_add(1);
    }
    build(lb, s, m, depth + 1, out);
    const uint32_t left_count = (uint32_t)(out.size() - left_begin);
    if (forked) {
      fut.get();
      out.insert(out.end(), right.begin(), right.end());
    } else {
      build(rb, m, e, depth + 1, out);
    }
    out[me].left_count = left_count;
  }
};

struct Tree {
  std::vector<TreeNode> nodes;
  std::vector<uint32_t> order;
  uint64_t sah_splits = 0, fallbacks = 0;
  uint32_t max_depth = 0;
};

// FlattenBVH::new with the given TreeBuildOption (content/space/src/bvh/mod.rs:55-79).
Tree build_tree(const std::vector<Box>& boxes, uint32_t bin_size, uint32_t max_depth, int threads) {
  Tree t;
  const uint32_t n = (uint32_t)boxes.size();
  std::vector<f3> centers(n);
  for (uint32_t i = 0; i < n; i++) {
    const Box& b = boxes[i];
    centers[i] = {(b.lo.x + b.hi.x) * 0.5f, (b.lo.y + b.hi.y) * 0.5f, (b.lo.z + b.hi.z) * 0.5f};
  }
  t.order.resize(n);
  for (uint32_t i = 0; i < n; i++) t.order[i] = i;
  std::vector<uint32_t> scratch(n);
  TreeBuilder tb;
  tb.boxes = boxes.data();
  tb.centers = centers.data();
  tb.order = t.order.data();
  tb.scratch = scratch.data();
  tb.bin_size = bin_size;
  tb.max_depth = max_depth;
  tb.spare_threads = std::max(0, threads - 1);
  Box root = empty_box();
  for (uint32_t i = 0; i < n; i++) grow(root, boxes[i]);
  t.nodes.reserve(n > 0 ? 2 * ((size_t)n / std::max<uint32_t>(1, bin_size)) + 1 : 1);
  tb.build(root, 0, n, 0, t.nodes);
  t.sah_splits = tb.sah_splits;
  t.fallbacks = tb.fallbacks;
  for (const TreeNode& nd : t.nodes) t.max_depth = std::max(t.max_depth, nd.depth);
  return t;
}

// compute_bvh_next (naive/mod.rs:611-632): threaded hit/miss links, pre-order.
std::vector<std::pair<uint32_t, uint32_t>> threaded_links(const std::vector<TreeNode>& nodes) {
  std::vector<std::pair<uint32_t, uint32_t>> links(nodes.size());
  std::vector<uint32_t> pending;
  for (uint32_t i = 0; i < (uint32_t)nodes.size(); i++) {
    if (!pending.empty() && pending.back() == i) pending.pop_back();
    const uint32_t miss = pending.empty() ? INVALID_NEXT : pending.back();
    if (nodes[i].left_count) {
      pending.push_back(i + nodes[i].left_count + 1);
      links[i] = {i + 1, miss};
    } else {
      links[i] = {miss, miss};
    }
  }
  return links;
}

DeviceBVHNode to_device_node(const TreeNode& n, std::pair<uint32_t, uint32_t> link, uint32_t node_offset,
                             uint32_t prim_offset) {
  DeviceBVHNode d;
  std::memset(&d, 0, sizeof(d));
  d.aabb_min[0] = n.box.lo.x;
  d.aabb_min[1] = n.box.lo.y;
  d.aabb_min[2] = n.box.lo.z;
  d.aabb_max[0] = n.box.hi.x;
  d.aabb_max[1] = n.box.hi.y;
  d.aabb_max[2] = n.box.hi.z;
  d.hit_next = link.first == INVALID_NEXT ? INVALID_NEXT : link.first + node_offset;
  d.miss_next = link.second == INVALID_NEXT ? INVALID_NEXT : link.second + node_offset;
  d.content_range[0] = n.start + prim_offset;
  d.content_range[1] = n.end + prim_offset;
  return d;
}

// Two-child nodes for one tree; returns the root's child code and fills
// `code` (per binary node: wide index or LEAF_BIT | leaf id).
uint32_t emit_wide(const Tree& t, uint32_t prim_offset, HostBuilt& hb, std::vector<uint32_t>& code) {
  const uint32_t nn = (uint32_t)t.nodes.size();
  code.assign(nn, 0);
  uint32_t next_inner = (uint32_t)hb.wide_nodes.size();
  uint32_t next_leaf = (uint32_t)(hb.leaf_ranges.size() / 2);
  for (uint32_t i = 0; i < nn; i++) code[i] = t.nodes[i].left_count ? next_inner++ : (LEAF_BIT | next_leaf++);
  hb.wide_nodes.resize(next_inner);
  hb.leaf_ranges.resize((size_t)next_leaf * 2);
  for (uint32_t i = 0; i < nn; i++) {
    const TreeNode& n = t.nodes[i];
    if (!n.left_count) {
      const uint32_t l = code[i] & ~LEAF_BIT;
      hb.leaf_ranges[2 * (size_t)l] = n.start + prim_offset;
      hb.leaf_ranges[2 * (size_t)l + 1] = n.end + prim_offset;
      continue;
    }
    const uint32_t li = i + 1, ri = i + n.left_count + 1;
    const Box& a = t.nodes[li].box;
    const Box& b = t.nodes[ri].box;
    WideNode& w = hb.wide_nodes[code[i]];
    const float vals[12] = {a.lo.x, a.lo.y, a.lo.z, a.hi.x, a.hi.y, a.hi.z, b.lo.x, b.lo.y, b.lo.z, b.hi.x, b.hi.y, b.hi.z};
    std::memcpy(w.w, vals, sizeof(vals));
    w.code[0] = code[li];
    w.code[1] = code[ri];
    w.code[2] = 0;
    w.code[3] = 0;
  }
  return nn ? code[0] : (LEAF_BIT | 0);
}

// True when box s is flat on some axis and lies on a face plane of box a,
// which is not flat there. The four-child walk tests a node's slots but not
// the two-child nodes it opened to reach them, which is exact only while the
// slab test is monotone (a box inside another never passes when the outer one
// fails). A ray with a zero direction component breaks that exactly here: with
// its origin in that plane it fails a's slab test (0 * inf = NaN beside
// +-inf) but passes the flat box's (NaN on both planes, dropped by fmin/fmax).
// The collapse therefore never opens a node whose children are flat on its
// faces or on the faces of the nodes opened above it.
bool flat_on_boundary(const Box& s, const Box& a) {
  const float sl[3] = {s.lo.x, s.lo.y, s.lo.z}, sh[3] = {s.hi.x, s.hi.y, s.hi.z};
  const float al[3] = {a.lo.x, a.lo.y, a.lo.z}, ah[3] = {a.hi.x, a.hi.y, a.hi.z};
  for (int k = 0; k < 3; k++)
    if (sl[k] == sh[k] && al[k] != ah[k] && (al[k] == sl[k] || ah[k] == sl[k])) return true;
  return false;
}

// Whether binary node x (opened ancestors anc, EMPTY_SLOT when absent) may be
// opened in a four-child node: no child of x is flat on a face of x or of anc.
bool openable(const Tree& t, uint32_t x, const uint32_t anc[2]) {
  const uint32_t kids[2] = {x + 1, x + t.nodes[x].left_count + 1};
  for (uint32_t c : kids) {
    if (flat_on_boundary(t.nodes[c].box, t.nodes[x].box)) return false;
    for (int a = 0; a < 2; a++)
      if (anc[a] != EMPTY_SLOT && flat_on_boundary(t.nodes[c].box, t.nodes[anc[a]].box)) return false;
  }
  return true;
}

float node_area(const Box& b) {
  const float w = b.hi.x - b.lo.x, h = b.hi.y - b.lo.y, d = b.hi.z - b.lo.z;
  return w * h + w * d + h * d;
}

// Four-child node rooted at binary inner node `bi`; returns its index and
// raises *depth to the deepest four-child level below.
uint32_t emit_wide4(const Tree& t, uint32_t bi, const std::vector<uint32_t>& code2, HostBuilt& hb, uint32_t level,
                    uint32_t* depth) {
  uint32_t slot[4];
  uint32_t anc[4][2];  // per slot, the binary nodes opened above it in this node (never tested by the walk)
  int n = 0;
  slot[n++] = bi + 1;
  slot[n++] = bi + t.nodes[bi].left_count + 1;
  for (auto& a : anc) a[0] = a[1] = EMPTY_SLOT;
  while (n < 4) {
    int best = -1;
    float best_area = -1.0f;
    for (int k = 0; k < n; k++) {
      const TreeNode& c = t.nodes[slot[k]];
      if (!c.left_count || !openable(t, slot[k], anc[k])) continue;
      const float a = node_area(c.box);
      if (best < 0 || a > best_area) {
        best = k;
        best_area = a;
      }
    }
    if (best < 0) break;
    const uint32_t open = slot[best];
    const uint32_t up[2] = {open, anc[best][0]};
    for (int k = n; k > best + 1; k--) {
      slot[k] = slot[k - 1];
      anc[k][0] = anc[k - 1][0];
      anc[k][1] = anc[k - 1][1];
    }
    slot[best] = open + 1;
    slot[best + 1] = open + t.nodes[open].left_count + 1;
    for (int k = best; k <= best + 1; k++) {
      anc[k][0] = up[0];
      anc[k][1] = up[1];
    }
    n++;
  }
  const uint32_t me = (uint32_t)hb.wide4_nodes.size();
  hb.wide4_nodes.emplace_back();
  if (level + 1 > *depth) *depth = level + 1;
  uint32_t codes[4] = {EMPTY_SLOT, EMPTY_SLOT, EMPTY_SLOT, EMPTY_SLOT};
  for (int k = 0; k < n; k++) {
    const TreeNode& c = t.nodes[slot[k]];
    codes[k] = c.left_count ? emit_wide4(t, slot[k], code2, hb, level + 1, depth) : code2[slot[k]];
  }
  Wide4Node& w = hb.wide4_nodes[me];
  for (int k = 0; k < 4; k++) {
    const bool used = k < n;
    const Box b = used ? t.nodes[slot[k]].box : Box{{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    w.lo_x[k] = b.lo.x;
    w.lo_y[k] = b.lo.y;
    w.lo_z[k] = b.lo.z;
    w.hi_x[k] = b.hi.x;
    w.hi_y[k] = b.hi.y;
    w.hi_z[k] = b.hi.z;
    w.code[k] = codes[k];
    w.pad[k] = 0;
  }
  return me;
}

TriRecord make_tri(const f3& v0, const f3& v1, const f3& v2) {
  const f3 e1 = {v1.x - v0.x, v1.y - v0.y, v1.z - v0.z};
  const f3 e2 = {v2.x - v0.x, v2.y - v0.y, v2.z - v0.z};
  f3 n = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
  const float mag_sq = n.x * n.x + n.y * n.y + n.z * n.z;
  if (mag_sq > 0.0f) {
    const float inv = 1.0f / std::sqrt(mag_sq);
    n = {n.x * inv, n.y * inv, n.z * inv};
  }
  const float uu = e1.x * e1.x + e1.y * e1.y + e1.z * e1.z;
  const float uv = e1.x * e2.x + e1.y * e2.y + e1.z * e2.z;
  const float vv = e2.x * e2.x + e2.y * e2.y + e2.z * e2.z;
  const float inv_d = 1.0f / (uv * uv - uu * vv);
  TriRecord r;
  const float q[16] = {v0.x, v0.y, v0.z, n.x, e1.x, e1.y, e1.z, n.y, e2.x, e2.y, e2.z, n.z, uu, uv, vv, inv_d};
  std::memcpy(r.q, q, sizeof(q));
  return r;
}

// Mat4 helpers in the reference's element order (math/algebra/src/mat/mat4.rs).
struct M4 {
  float a1, a2, a3, a4, b1, b2, b3, b4, c1, c2, c3, c4, d1, d2, d3, d4;
};
f3 m4_point(const M4& m, const f3& p) {  // Mat4 * Vec3: (m * (p, 1)).xyz / w
  const float x = p.x * m.a1 + p.y * m.b1 + p.z * m.c1 + 1.0f * m.d1;
  const float y = p.x * m.a2 + p.y * m.b2 + p.z * m.c2 + 1.0f * m.d2;
  const float z = p.x * m.a3 + p.y * m.b3 + p.z * m.c3 + 1.0f * m.d3;
  const float w = p.x * m.a4 + p.y * m.b4 + p.z * m.c4 + 1.0f * m.d4;
  return {x / w, y / w, z / w};
}
float m3_det(const M4& m) {  // Mat3::det of to_mat3()
  const float t11 = m.c3 * m.b2 - m.b3 * m.c2;
  const float t12 = m.b3 * m.c1 - m.c3 * m.b1;
  const float t13 = m.c2 * m.b1 - m.b2 * m.c1;
  return m.a1 * t11 + m.a2 * t12 + m.a3 * t13;
}
float m4_det(const M4& m) {
  return m.a1 * m.b2 * m.c3 * m.d4 - m.a1 * m.b2 * m.c4 * m.d3 + m.a1 * m.b3 * m.c4 * m.d2 -
         m.a1 * m.b3 * m.c2 * m.d4 + m.a1 * m.b4 * m.c2 * m.d3 - m.a1 * m.b4 * m.c3 * m.d2 -
         m.a2 * m.b3 * m.c4 * m.d1 + m.a2 * m.b3 * m.c1 * m.d4 - m.a2 * m.b4 * m.c1 * m.d3 +
         m.a2 * m.b4 * m.c3 * m.d1 - m.a2 * m.b1 * m.c3 * m.d4 + m.a2 * m.b1 * m.c4 * m.d3 +
         m.a3 * m.b4 * m.c1 * m.d2 - m.a3 * m.b4 * m.c2 * m.d1 + m.a3 * m.b1 * m.c2 * m.d4 -
         m.a3 * m.b1 * m.c4 * m.d2 + m.a3 * m.b2 * m.c4 * m.d1 - m.a3 * m.b2 * m.c1 * m.d4 -
         m.a4 * m.b1 * m.c2 * m.d3 + m.a4 * m.b1 * m.c3 * m.d2 - m.a4 * m.b2 * m.c3 * m.d1 +
         m.a4 * m.b2 * m.c1 * m.d3 - m.a4 * m.b3 * m.c1 * m.d2 + m.a4 * m.b3 * m.c2 * m.d1;
}
M4 m4_inverse_or_identity(const M4& m) {
  const float det = m4_det(m);
  if (det == 0.0f) return M4{1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  const float p = 1.0f / det, q = -p;
  M4 r;
  r.a1 = p * (m.b2 * (m.c3 * m.d4 - m.c4 * m.d3) + m.b3 * (m.c4 * m.d2 - m.c2 * m.d4) + m.b4 * (m.c2 * m.d3 - m.c3 * m.d2));
  r.a2 = q * (m.a2 * (m.c3 * m.d4 - m.c4 * m.d3) + m.a3 * (m.c4 * m.d2 - m.c2 * m.d4) + m.a4 * (m.c2 * m.d3 - m.c3 * m.d2));
  r.a3 = p * (m.a2 * (m.b3 * m.d4 - m.b4 * m.d3) + m.a3 * (m.b4 * m.d2 - m.b2 * m.d4) + m.a4 * (m.b2 * m.d3 - m.b3 * m.d2));
  r.a4 = q * (m.a2 * (m.b3 * m.c4 - m.b4 * m.c3) + m.a3 * (m.b4 * m.c2 - m.b2 * m.c4) + m.a4 * (m.b2 * m.c3 - m.b3 * m.c2));
  r.b1 = q * (m.b1 * (m.c3 * m.d4 - m.c4 * m.d3) + m.b3 * (m.c4 * m.d1 - m.c1 * m.d4) + m.b4 * (m.c1 * m.d3 - m.c3 * m.d1));
  r.b2 = p * (m.a1 * (m.c3 * m.d4 - m.c4 * m.d3) + m.a3 * (m.c4 * m.d1 - m.c1 * m.d4) + m.a4 * (m.c1 * m.d3 - m.c3 * m.d1));
  r.b3 = q * (m.a1 * (m.b3 * m.d4 - m.b4 * m.d3) + m.a3 * (m.b4 * m.d1 - m.b1 * m.d4) + m.a4 * (m.b1 * m.d3 - m.b3 * m.d1));
  r.b4 = p * (m.a1 * (m.b3 * m.c4 - m.b4 * m.c3) + m.a3 * (m.b4 * m.c1 - m.b1 * m.c4) + m.a4 * (m.b1 * m.c3 - m.b3 * m.c1));
  r.c1 = p * (m.b1 * (m.c2 * m.d4 - m.c4 * m.d2) + m.b2 * (m.c4 * m.d1 - m.c1 * m.d4) + m.b4 * (m.c1 * m.d2 - m.c2 * m.d1));
  r.c2 = q * (m.a1 * (m.c2 * m.d4 - m.c4 * m.d2) + m.a2 * (m.c4 * m.d1 - m.c1 * m.d4) + m.a4 * (m.c1 * m.d2 - m.c2 * m.d1));
  r.c3 = p * (m.a1 * (m.b2 * m.d4 - m.b4 * m.d2) + m.a2 * (m.b4 * m.d1 - m.b1 * m.d4) + m.a4 * (m.b1 * m.d2 - m.b2 * m.d1));
  r.c4 = q * (m.a1 * (m.b2 * m.c4 - m.b4 * m.c2) + m.a2 * (m.b4 * m.c1 - m.b1 * m.c4) + m.a4 * (m.b1 * m.c2 - m.b2 * m.c1));
  r.d1 = q * (m.b1 * (m.c2 * m.d3 - m.c3 * m.d2) + m.b2 * (m.c3 * m.d1 - m.c1 * m.d3) + m.b3 * (m.c1 * m.d2 - m.c2 * m.d1));
  r.d2 = p * (m.a1 * (m.c2 * m.d3 - m.c3 * m.d2) + m.a2 * (m.c3 * m.d1 - m.c1 * m.d3) + m.a3 * (m.c1 * m.d2 - m.c2 * m.d1));
  r.d3 = q * (m.a1 * (m.b2 * m.d3 - m.b3 * m.d2) + m.a2 * (m.b3 * m.d1 - m.b1 * m.d3) + m.a3 * (m.b1 * m.d2 - m.b2 * m.d1));
  r.d4 = p * (m.a1 * (m.b2 * m.c3 - m.b3 * m.c2) + m.a2 * (m.b3 * m.c1 - m.b1 * m.c3) + m.a3 * (m.b1 * m.c2 - m.b2 * m.c1));
  return r;
}
Box transform_box(const Box& b, const M4& m) {  // Box3::apply_matrix
  if (b.hi.x < b.lo.x || b.hi.y < b.lo.y || b.hi.z < b.lo.z) return b;
  Box r = empty_box();
  for (int k = 0; k < 8; k++) {
    const f3 p = {(k & 4) ? b.hi.x : b.lo.x, (k & 2) ? b.hi.y : b.lo.y, (k & 1) ? b.hi.z : b.lo.z};
    grow(r, m4_point(m, p));
  }
  return r;
}

// TLAS forest (build_tlas, naive/mod.rs:262-320, and the loop at :435-454).
// blas_box holds one entry per geometry, as naive/mod.rs:239 pushes it.
std::string build_tlas_phase(const std::vector<std::unique_ptr<std::vector<InstanceSource>>>& tlas,
                             const std::vector<Box>& blas_box, const std::vector<char>& blas_box_some,
                             const BuildOptions& opt, HostBuilt& hb) {
  for (const auto& tp : tlas) {
    if (!tp) {
      hb.tlas_bvh_root.push_back(INVALID_NEXT);
      continue;
    }
    const uint32_t bvh_start = (uint32_t)hb.tlas_bvh_forest.size();
    const uint32_t prim_start = (uint32_t)hb.tlas_data.size();
    std::vector<Box> aabbs;
    aabbs.reserve(tp->size());
    for (const InstanceSource& s : *tp) {
      if (s.blas_handle >= blas_box.size() || !blas_box_some[s.blas_handle])
        return "instance references a deleted or missing BLAS";
      M4 m;
      std::memcpy(&m, s.transform, 64);
      aabbs.push_back(transform_box(blas_box[s.blas_handle], m));
    }
    Tree t = build_tree(aabbs, opt.tlas_bin_size, opt.tlas_max_depth, 1);
    for (uint32_t idx : t.order) {
      const InstanceSource& s = (*tp)[idx];
      M4 m;
      std::memcpy(&m, s.transform, 64);
      uint32_t flags = s.flags;
      if (m3_det(m) < 0.0f) flags ^= RDN_INSTANCE_TRIANGLE_FLIP_FACING;
      DeviceInstance di;
      std::memset(&di, 0, sizeof(di));
      std::memcpy(di.transform, s.transform, 64);
      const M4 inv = m4_inverse_or_identity(m);
      std::memcpy(di.transform_inv, &inv, 64);
      di.instance_custom_index = s.custom_index;
      di.sbt_offset = s.sbt_offset;
      di.flags = flags;
      di.acceleration_structure_handle = s.blas_handle;
      TlasBounding tb;
      std::memset(&tb, 0, sizeof(tb));
      const Box& a = aabbs[idx];
      tb.world_min[0] = a.lo.x;
      tb.world_min[1] = a.lo.y;
      tb.world_min[2] = a.lo.z;
      tb.world_max[0] = a.hi.x;
      tb.world_max[1] = a.hi.y;
      tb.world_max[2] = a.hi.z;
      tb.mask = s.mask;
      tb.flags = flags;
      hb.tlas_data.push_back(di);
      hb.tlas_bounding.push_back(tb);
    }
    const auto links = threaded_links(t.nodes);
    for (size_t i = 0; i < t.nodes.size(); i++)
      hb.tlas_bvh_forest.push_back(to_device_node(t.nodes[i], links[i], bvh_start, prim_start));
    hb.tlas_bvh_root.push_back(bvh_start);
    hb.sah_splits += t.sah_splits;
    hb.median_fallbacks += t.fallbacks;
  }
  return std::string();
}

}  // namespace

std::string build_host(const std::vector<std::unique_ptr<std::vector<GeometrySource>>>& blas,
                       const std::vector<std::unique_ptr<std::vector<InstanceSource>>>& tlas,
                       const std::vector<uint32_t>& binding, const BuildOptions& opt, HostBuilt& hb) {
  const int threads = opt.host_threads ? (int)opt.host_threads : std::max(1u, std::thread::hardware_concurrency());
  // one entry per geometry, as naive/mod.rs:239 pushes it inside the geometry loop
  std::vector<Box> blas_box;
  std::vector<char> blas_box_some;

  struct Pending {
    Tree tree;
    uint32_t primitive_start, geometry_idx, flags;
  };
  std::vector<Pending> trees;

  for (const auto& bp : blas) {
    if (!bp) {
      hb.blas_meta_info.push_back(BlasMetaInfo{{0, 0}});
      blas_box.push_back(empty_box());
      blas_box_some.push_back(0);
      continue;
    }
    const uint32_t first = (uint32_t)trees.size();
    uint32_t gidx = 0;
    for (const GeometrySource& g : *bp) {
      Box root_box = empty_box();
      if (g.type == 0) {
        const uint32_t prim_start = (uint32_t)(hb.indices.size() / 3);
        const uint32_t vertex_start = (uint32_t)(hb.vertices.size() / 3);
        const size_t vcount = g.positions.size() / 3;
        const size_t ntri = (g.indexed ? g.indices.size() : vcount) / 3;
        std::vector<Box> boxes(ntri);
        for (size_t t = 0; t < ntri; t++) {
          Box b = empty_box();
          for (int k = 0; k < 3; k++) {
            const uint32_t vi = g.indexed ? g.indices[t * 3 + k] : (uint32_t)(t * 3 + k);
            if (vi >= vcount) return "triangle index out of range";
            grow(b, f3{g.positions[3 * (size_t)vi], g.positions[3 * (size_t)vi + 1], g.positions[3 * (size_t)vi + 2]});
          }
          boxes[t] = b;
        }
        hb.vertices.insert(hb.vertices.end(), g.positions.begin(), g.positions.end());
        Pending pd;
        pd.tree = build_tree(boxes, opt.blas_bin_size, opt.blas_max_depth, threads);
        grow(root_box, pd.tree.nodes[0].box);
        for (uint32_t p : pd.tree.order) hb.indices_redirect.push_back(prim_start + p);
        for (size_t t = 0; t < ntri; t++)
          for (int k = 0; k < 3; k++)
            hb.indices.push_back(vertex_start + (g.indexed ? g.indices[t * 3 + k] : (uint32_t)(t * 3 + k)));
        pd.primitive_start = prim_start;
        pd.geometry_idx = gidx;
        pd.flags = g.flags;
        hb.sah_splits += pd.tree.sah_splits;
        hb.median_fallbacks += pd.tree.fallbacks;
        hb.max_blas_depth = std::max(hb.max_blas_depth, pd.tree.max_depth);
        trees.push_back(std::move(pd));
      }
      blas_box.push_back(root_box);
      blas_box_some.push_back(1);
      gidx++;
    }
    hb.blas_meta_info.push_back(BlasMetaInfo{{first, (uint32_t)trees.size()}});
  }

  // flatten the triangle forest, both layouts
  hb.tri_records.resize(hb.indices_redirect.size());
  for (const Pending& pd : trees) {
    const uint32_t bvh_start = (uint32_t)hb.tri_bvh_forest.size();
    hb.tri_bvh_root.push_back(GeometryMetaInfo{bvh_start, pd.geometry_idx, pd.primitive_start, pd.flags});
    const auto links = threaded_links(pd.tree.nodes);
    for (size_t i = 0; i < pd.tree.nodes.size(); i++)
      hb.tri_bvh_forest.push_back(to_device_node(pd.tree.nodes[i], links[i], bvh_start, pd.primitive_start));
    std::vector<uint32_t> code2;
    hb.geom_root_code.push_back(emit_wide(pd.tree, pd.primitive_start, hb, code2));
    uint32_t d4 = 0;
    hb.geom_root_code4.push_back(pd.tree.nodes[0].left_count ? emit_wide4(pd.tree, 0, code2, hb, 0, &d4) : code2[0]);
    hb.max_wide4_depth = std::max(hb.max_wide4_depth, d4);
    const size_t cnt = pd.tree.order.size();
    for (size_t j = 0; j < cnt; j++) {
      const uint32_t tri = hb.indices_redirect[pd.primitive_start + j];
      const uint32_t* ix = &hb.indices[3 * (size_t)tri];
      const float* V = hb.vertices.data();
      const f3 v0 = {V[3 * (size_t)ix[0]], V[3 * (size_t)ix[0] + 1], V[3 * (size_t)ix[0] + 2]};
      const f3 v1 = {V[3 * (size_t)ix[1]], V[3 * (size_t)ix[1] + 1], V[3 * (size_t)ix[1] + 2]};
      const f3 v2 = {V[3 * (size_t)ix[2]], V[3 * (size_t)ix[2] + 1], V[3 * (size_t)ix[2] + 2]};
      hb.tri_records[pd.primitive_start + j] = make_tri(v0, v1, v2);
    }
  }

  std::string err = build_tlas_phase(tlas, blas_box, blas_box_some, opt, hb);
  if (!err.empty()) return err;
  hb.tlas_binding = binding;
  hb.n_triangles = hb.indices_redirect.size();
  hb.n_nodes = hb.tri_bvh_forest.size();
  hb.n_indices = hb.indices.size();
  hb.n_vertices = hb.vertices.size() / 3;
  return std::string();
}

}  // namespace rdn

namespace rdn {

std::string build_with_device_blas(const std::vector<std::unique_ptr<std::vector<GeometrySource>>>& blas,
                                   const std::vector<std::unique_ptr<std::vector<InstanceSource>>>& tlas,
                                   const std::vector<uint32_t>& binding, const BuildOptions& opt, int sm_count,
                                   cudaMemPool_t pool, HostBuilt& hb, DeviceBuilt& d, double* device_seconds) {
  // the same geometry walk as build_host: one tree per triangle geometry in
  // BLAS-slot order, one root-box entry per geometry (naive/mod.rs:239)
  std::vector<DeviceGeometry> geoms;
  struct TreeMeta {
    uint32_t geometry_idx, flags;
  };
  std::vector<TreeMeta> meta;
  std::vector<int64_t> box_entry;  // per geometry entry: tree index, -1 = non-triangle, -2 = deleted slot
  for (const auto& bp : blas) {
    if (!bp) {
      hb.blas_meta_info.push_back(BlasMetaInfo{{0, 0}});
      box_entry.push_back(-2);
      continue;
    }
    const uint32_t first = (uint32_t)geoms.size();
    uint32_t gidx = 0;
    for (const GeometrySource& g : *bp) {
      if (g.type == 0) {
        const size_t vcount = g.positions.size() / 3;
        const size_t ntri = (g.indexed ? g.indices.size() : vcount) / 3;
        if (vcount >= (1ull << 32) || ntri >= (1ull << 32)) return "geometry too large";
        box_entry.push_back((int64_t)geoms.size());
        geoms.push_back(DeviceGeometry{g.positions.data(), (uint32_t)vcount, g.indexed ? g.indices.data() : nullptr,
                                       (uint32_t)ntri});
        meta.push_back(TreeMeta{gidx, g.flags});
      } else {
        box_entry.push_back(-1);
      }
      gidx++;
    }
    hb.blas_meta_info.push_back(BlasMetaInfo{{first, (uint32_t)geoms.size()}});
  }
  DeviceBlasOut o;
  std::string err = build_blas_device(geoms, opt.blas_bin_size, opt.blas_max_depth, sm_count, pool, d, o);
  if (!err.empty()) return err;
  *device_seconds = o.kernel_seconds;
  std::vector<Box> blas_box;
  std::vector<char> blas_box_some;
  for (int64_t e : box_entry) {
    if (e >= 0) {
      Box b = empty_box();
      grow(b, o.root_box[(size_t)e]);
      blas_box.push_back(b);
    } else {
      blas_box.push_back(empty_box());
    }
    blas_box_some.push_back(e == -2 ? 0 : 1);
  }
  uint32_t bvh_start = 0, prim_start = 0;
  for (size_t t = 0; t < geoms.size(); t++) {
    hb.tri_bvh_root.push_back(GeometryMetaInfo{bvh_start, meta[t].geometry_idx, prim_start, meta[t].flags});
    bvh_start += o.tree_nodes[t];
    prim_start += geoms[t].triangle_count;
  }
  hb.geom_root_code = o.root_code;
  hb.geom_root_code4 = o.root_code4;
  hb.max_blas_depth = o.max_depth;
  hb.max_wide4_depth = o.max_wide4_depth;
  hb.sah_splits = o.sah_splits;
  hb.median_fallbacks = o.median_fallbacks;
  hb.device_blas = true;
  hb.device_bytes = o.bytes;
  hb.n_triangles = o.triangles;
  hb.n_nodes = o.nodes;
  hb.n_indices = 3 * o.triangles;
  hb.n_vertices = o.vertices;
  err = build_tlas_phase(tlas, blas_box, blas_box_some, opt, hb);
  if (!err.empty()) return err;
  hb.tlas_binding = binding;
  return std::string();
}

}  // namespace rdn
