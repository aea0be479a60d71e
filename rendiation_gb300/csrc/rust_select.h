// Median selection used by the BVH builder's degenerate-split fallback
// (BalanceTree::split -> median_partition_at_axis, content/space/src/bvh/apply.rs:19-45),
// which calls Rust core's `slice::select_nth_unstable_by`. To produce the same
// element order as the reference's build, this header restates that library
// algorithm (Rust >= 1.81 library/core/src/slice/select.rs with the shared
// pivot choice of sort/shared/pivot.rs and the branchless cyclic Lomuto
// partition of sort/unstable/quicksort.rs). Elements with distinct keys land on
// the same side under any correct selection; only the order among exactly tied
// keys depends on these details.
//
// The library's two recursions (the recursive pseudo-median of the pivot
// choice, and median-of-medians calling itself through the ninther pivot) are
// unrolled onto fixed explicit stacks so that the same code runs on the host
// and, one selection per thread, on the device without a call stack. Each
// level of either recursion shrinks the slice at least eightfold, so 24 frames
// cover every length a size_t can hold.
#pragma once
#include <cstddef>
#include <cstdint>

#if defined(__CUDACC__)
#define RDN_HD __host__ __device__
#else
#define RDN_HD
#endif

namespace rdn {

template <class T>
RDN_HD inline void rs_swap(T& a, T& b) {
  T t = a;
  a = b;
  b = t;
}

template <class T, class Less>
class RustSelectNth {
 public:
  RDN_HD explicit RustSelectNth(Less less) : lt_(less) {}

  RDN_HD void run(T* v, size_t len, size_t index) {
    if (index >= len) return;
    if (index == len - 1) {
      rs_swap(v[arg_max(v, len)], v[index]);
    } else if (index == 0) {
      rs_swap(v[arg_min(v, len)], v[index]);
    } else {
      select_loop(v, len, index);
    }
  }

  // The library's worst-case path alone (select reaches it after 16 pivots
  // that did not shrink the slice enough); public so tests can drive it.
  RDN_HD void run_median_of_medians(T* v, size_t len, size_t index) {
    if (index < len) median_of_medians(v, len, index);
  }

 private:
  Less lt_;
  static constexpr size_t kSmall = 16;       // INSERTION_SORT_THRESHOLD
  static constexpr size_t kRecMedian = 64;   // PSEUDO_MEDIAN_REC_THRESHOLD
  static constexpr int kFrames = 24;

  RDN_HD void insertion_sort(T* v, size_t len) {
    for (size_t i = 1; i < len; i++) {
      if (!lt_(v[i], v[i - 1])) continue;
      T hole = v[i];
      size_t j = i;
      do {
        v[j] = v[j - 1];
        --j;
      } while (j > 0 && lt_(hole, v[j - 1]));
      v[j] = hole;
    }
  }
  RDN_HD size_t arg_min(const T* v, size_t len) {
    size_t best = 0;
    for (size_t i = 1; i < len; i++) best = lt_(v[i], v[best]) ? i : best;
    return best;
  }
  RDN_HD size_t arg_max(const T* v, size_t len) {
    size_t best = 0;
    for (size_t i = 1; i < len; i++) best = lt_(v[best], v[i]) ? i : best;
    return best;
  }
  RDN_HD size_t med3(const T* v, size_t a, size_t b, size_t c) {
    const bool ab = lt_(v[a], v[b]);
    const bool ac = lt_(v[a], v[c]);
    if (ab != ac) return a;
    return (lt_(v[b], v[c]) != ab) ? c : b;
  }
  // Recursive pseudo-median: for n*8 >= 64 each of a, b, c is first replaced
  // by the pseudo-median of (x, x+4s, x+7s) with s = n/8, then med3 of the three.
  RDN_HD size_t med3_rec(const T* v, size_t a, size_t b, size_t c, size_t n) {
    struct Frame {
      size_t x[3];
      size_t n;
      size_t r[3];
      int stage;
    };
    Frame st[kFrames];
    int top = 0;
    st[0] = Frame{{a, b, c}, n, {0, 0, 0}, 0};
    while (true) {
      Frame& f = st[top];
      size_t ret;
      if (f.n * 8 >= kRecMedian && f.stage < 3) {
        const size_t s = f.n / 8;
        const size_t base = f.x[f.stage];
        f.stage++;
        st[top + 1] = Frame{{base, base + 4 * s, base + 7 * s}, s, {0, 0, 0}, 0};
        ++top;
        continue;
      }
      ret = (f.n * 8 >= kRecMedian) ? med3(v, f.r[0], f.r[1], f.r[2]) : med3(v, f.x[0], f.x[1], f.x[2]);
      if (top == 0) return ret;
      --top;
      st[top].r[st[top].stage - 1] = ret;
    }
  }
  RDN_HD size_t pick_pivot(const T* v, size_t len) {
    const size_t s = len / 8;
    return len < kRecMedian ? med3(v, 0, 4 * s, 7 * s) : med3_rec(v, 0, 4 * s, 7 * s, s);
  }
  // Pivot moved to v[0]; the rest is partitioned by a cyclic Lomuto pass whose
  // last step consumes the element that started in the gap; the pivot is then
  // swapped to position `num_lt`. le=false: pred(x, p) = x < p; le=true:
  // pred(x, p) = !(p < x).
  RDN_HD size_t partition(T* v, size_t len, size_t pivot_pos, bool le) {
    if (len == 0) return 0;
    rs_swap(v[0], v[pivot_pos]);
    const T pivot = v[0];
    T* w = v + 1;
    const size_t n = len - 1;
    size_t num_lt = 0;
    if (n > 0) {
      const T saved = w[0];
      size_t gap = 0;
      for (size_t r = 1; r <= n; r++) {
        const T x = (r == n) ? saved : w[r];
        const bool is_lt = le ? !lt_(pivot, x) : lt_(x, pivot);
        w[gap] = w[num_lt];
        w[num_lt] = x;
        gap = r;
        num_lt += is_lt;
      }
    }
    rs_swap(v[0], v[num_lt]);
    return num_lt;
  }
  RDN_HD size_t med_idx(const T* v, size_t a, size_t b, size_t c) {
    if (lt_(v[c], v[a])) rs_swap(a, c);
    if (lt_(v[c], v[b])) return c;
    if (lt_(v[b], v[a])) return a;
    return b;
  }
  RDN_HD void ninther(T* v, size_t a, size_t b, size_t c, size_t d, size_t e, size_t f, size_t g, size_t h,
                      size_t i) {
    b = med_idx(v, a, b, c);
    h = med_idx(v, g, h, i);
    if (lt_(v[h], v[b])) rs_swap(b, h);
    if (lt_(v[f], v[d])) rs_swap(d, f);
    if (!lt_(v[e], v[d])) {
      if (lt_(v[f], v[e])) {
        d = f;
      } else {
        if (lt_(v[e], v[b])) rs_swap(v[e], v[b]);
        else if (lt_(v[h], v[e])) rs_swap(v[e], v[h]);
        return;
      }
    }
    if (lt_(v[d], v[b])) d = b;
    else if (lt_(v[h], v[d])) d = h;
    rs_swap(v[d], v[e]);
  }
  // median_of_medians(v, len, k): loop of ninther pivots; each pivot step runs
  // median_of_medians on the middle `frac` elements (a nested frame) and then
  // partitions the whole slice around their median.
  RDN_HD void median_of_medians(T* v, size_t len, size_t k) {
    struct Frame {
      T* v;
      size_t len, k, lo, half;
    };
    Frame st[kFrames];
    int top = 0;
    st[0] = Frame{v, len, k, 0, 0};
    bool resumed = false;
    while (true) {
      Frame& f = st[top];
      if (resumed) {
        // the nested selection over [lo, lo + frac) is done: finish the pivot step
        resumed = false;
        const size_t p = partition(f.v, f.len, f.lo + f.half, false);
        if (p == f.k) goto done;
        if (p > f.k) {
          f.len = p;
        } else {
          f.v += p + 1;
          f.len -= p + 1;
          f.k -= p + 1;
        }
      }
      if (f.len <= kSmall) {
        if (f.len >= 2) insertion_sort(f.v, f.len);
        goto done;
      }
      if (f.k == f.len - 1) {
        rs_swap(f.v[arg_max(f.v, f.len)], f.v[f.k]);
        goto done;
      }
      if (f.k == 0) {
        rs_swap(f.v[arg_min(f.v, f.len)], f.v[f.k]);
        goto done;
      }
      {
        const size_t n = f.len;
        const size_t frac = n <= 1024 ? n / 12 : (n <= 128 * 1024 ? n / 64 : n / 1024);
        const size_t half = frac / 2;
        const size_t lo = n / 2 - half;
        const size_t hi = lo + frac;
        const size_t gap = (n - 9 * frac) / 4;
        size_t a = lo - 4 * frac - gap, b = hi + gap;
        for (size_t i = lo; i < hi; i++, a += 3, b += 3)
          ninther(f.v, a, i - frac, b, a + 1, i, b + 1, a + 2, i + frac, b + 2);
        f.lo = lo;
        f.half = half;
        st[top + 1] = Frame{f.v + lo, frac, half, 0, 0};
        ++top;
        continue;
      }
    done:
      if (top == 0) return;
      --top;
      resumed = true;
    }
  }
  RDN_HD void select_loop(T* v, size_t len, size_t index) {
    int budget = 16;
    bool have_anc = false;
    T anc{};
    while (true) {
      if (len <= kSmall) {
        if (len >= 2) insertion_sort(v, len);
        return;
      }
      if (budget == 0) {
        median_of_medians(v, len, index);
        return;
      }
      --budget;
      const size_t pp = pick_pivot(v, len);
      if (have_anc && !lt_(anc, v[pp])) {
        // pivot equals its ancestor: split off everything <= pivot
        const size_t num_le = partition(v, len, pp, true);
        const size_t mid = num_le + 1;
        if (mid > index) return;
        v += mid;
        len -= mid;
        index -= mid;
        have_anc = false;
        continue;
      }
      const size_t num_lt = partition(v, len, pp, false);
      if (num_lt < index) {
        anc = v[num_lt];
        have_anc = true;
        v += num_lt + 1;
        len -= num_lt + 1;
        index -= num_lt + 1;
      } else if (num_lt > index) {
        len = num_lt;
      } else {
        return;
      }
    }
  }
};

}  // namespace rdn
