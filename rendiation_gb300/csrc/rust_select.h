// Median selection used by the BVH builder's degenerate-split fallback
// (BalanceTree::split -> median_partition_at_axis, content/space/src/bvh/apply.rs:19-45),
// which calls Rust core's `slice::select_nth_unstable_by`. To produce the same
// element order as the reference's build, this header restates that library
// algorithm (Rust >= 1.81 library/core/src/slice/select.rs with the shared
// pivot choice of sort/shared/pivot.rs and the branchless cyclic Lomuto
// partition of sort/unstable/quicksort.rs). Elements with distinct keys land on
// the same side under any correct selection; only the order among exactly tied
// keys depends on these details.
#pragma once
#include <cstddef>
#include <cstdint>
#include <utility>

namespace rdn {

template <class T, class Less>
class RustSelectNth {
 public:
  explicit RustSelectNth(Less less) : lt_(less) {}

  void run(T* v, size_t len, size_t index) {
    if (index >= len) return;
    if (index == len - 1) {
      std::swap(v[arg_max(v, len)], v[index]);
    } else if (index == 0) {
      std::swap(v[arg_min(v, len)], v[index]);
    } else {
      select_loop(v, len, index);
    }
  }

 private:
  Less lt_;
  static constexpr size_t kSmall = 16;       // INSERTION_SORT_THRESHOLD
  static constexpr size_t kRecMedian = 64;   // PSEUDO_MEDIAN_REC_THRESHOLD

  void insertion_sort(T* v, size_t len) {
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
  size_t arg_min(const T* v, size_t len) {
    size_t best = 0;
    for (size_t i = 1; i < len; i++) best = lt_(v[i], v[best]) ? i : best;
    return best;
  }
  size_t arg_max(const T* v, size_t len) {
    size_t best = 0;
    for (size_t i = 1; i < len; i++) best = lt_(v[best], v[i]) ? i : best;
    return best;
  }
  size_t med3(const T* v, size_t a, size_t b, size_t c) {
    const bool ab = lt_(v[a], v[b]);
    const bool ac = lt_(v[a], v[c]);
    if (ab != ac) return a;
    return (lt_(v[b], v[c]) != ab) ? c : b;
  }
  size_t med3_rec(const T* v, size_t a, size_t b, size_t c, size_t n) {
    if (n * 8 >= kRecMedian) {
      const size_t s = n / 8;
      a = med3_rec(v, a, a + 4 * s, a + 7 * s, s);
      b = med3_rec(v, b, b + 4 * s, b + 7 * s, s);
      c = med3_rec(v, c, c + 4 * s, c + 7 * s, s);
    }
    return med3(v, a, b, c);
  }
  size_t pick_pivot(const T* v, size_t len) {
    const size_t s = len / 8;
    return len < kRecMedian ? med3(v, 0, 4 * s, 7 * s) : med3_rec(v, 0, 4 * s, 7 * s, s);
  }
  // Pivot moved to v[0]; the rest is partitioned by a cyclic Lomuto pass whose
  // last step consumes the element that started in the gap; the pivot is then
  // swapped to position `num_lt`.
  template <class P>
  size_t partition(T* v, size_t len, size_t pivot_pos, P pred) {
    if (len == 0) return 0;
    std::swap(v[0], v[pivot_pos]);
    const T pivot = v[0];
    T* w = v + 1;
    const size_t n = len - 1;
    size_t num_lt = 0;
    if (n > 0) {
      const T saved = w[0];
      size_t gap = 0;
      for (size_t r = 1; r <= n; r++) {
        const T x = (r == n) ? saved : w[r];
        const bool is_lt = pred(x, pivot);
        w[gap] = w[num_lt];
        w[num_lt] = x;
        gap = r;
        num_lt += is_lt;
      }
    }
    std::swap(v[0], v[num_lt]);
    return num_lt;
  }
  size_t med_idx(const T* v, size_t a, size_t b, size_t c) {
    if (lt_(v[c], v[a])) std::swap(a, c);
    if (lt_(v[c], v[b])) return c;
    if (lt_(v[b], v[a])) return a;
    return b;
  }
  void ninther(T* v, size_t a, size_t b, size_t c, size_t d, size_t e, size_t f, size_t g, size_t h, size_t i) {
    b = med_idx(v, a, b, c);
    h = med_idx(v, g, h, i);
    if (lt_(v[h], v[b])) std::swap(b, h);
    if (lt_(v[f], v[d])) std::swap(d, f);
    if (!lt_(v[e], v[d])) {
      if (lt_(v[f], v[e])) {
        d = f;
      } else {
        if (lt_(v[e], v[b])) std::swap(v[e], v[b]);
        else if (lt_(v[h], v[e])) std::swap(v[e], v[h]);
        return;
      }
    }
    if (lt_(v[d], v[b])) d = b;
    else if (lt_(v[h], v[d])) d = h;
    std::swap(v[d], v[e]);
  }
  size_t ninthers_pivot(T* v, size_t len) {
    const size_t frac = len <= 1024 ? len / 12 : (len <= 128 * 1024 ? len / 64 : len / 1024);
    const size_t half = frac / 2;
    const size_t lo = len / 2 - half;
    const size_t hi = lo + frac;
    const size_t gap = (len - 9 * frac) / 4;
    size_t a = lo - 4 * frac - gap, b = hi + gap;
    for (size_t i = lo; i < hi; i++, a += 3, b += 3) ninther(v, a, i - frac, b, a + 1, i, b + 1, a + 2, i + frac, b + 2);
    median_of_medians(v + lo, frac, half);
    return partition(v, len, lo + half, lt_);
  }
  void median_of_medians(T* v, size_t len, size_t k) {
    while (true) {
      if (len <= kSmall) {
        if (len >= 2) insertion_sort(v, len);
        return;
      }
      if (k == len - 1) {
        std::swap(v[arg_max(v, len)], v[k]);
        return;
      }
      if (k == 0) {
        std::swap(v[arg_min(v, len)], v[k]);
        return;
      }
      const size_t p = ninthers_pivot(v, len);
      if (p == k) return;
      if (p > k) {
        len = p;
      } else {
        v += p + 1;
        len -= p + 1;
        k -= p + 1;
      }
    }
  }
  void select_loop(T* v, size_t len, size_t index) {
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
        const size_t num_le = partition(v, len, pp, [this](const T& a, const T& b) { return !lt_(b, a); });
        const size_t mid = num_le + 1;
        if (mid > index) return;
        v += mid;
        len -= mid;
        index -= mid;
        have_anc = false;
        continue;
      }
      const size_t num_lt = partition(v, len, pp, lt_);
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
