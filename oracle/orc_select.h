// Oracle — TEST INFRASTRUCTURE ONLY (see orc_math.h).
//
// Restatement of Rust core's `slice::select_nth_unstable_by`, which the
// reference's median fallback calls (content/space/src/bvh/apply.rs:19-45).
// The function lives in the Rust standard library, not in the reference tree;
// the reference pins toolchain `nightly-2026-08-08` (rust-toolchain.toml). The
// algorithm restated here is the published one of Rust >= 1.81
// (library/core/src/slice/select.rs: partition_at_index, partition_at_index_loop,
// median_of_medians, median_of_ninthers, ninther, median_idx, min_index,
// max_index; library/core/src/slice/sort/shared/pivot.rs: choose_pivot,
// median3_rec, median3; library/core/src/slice/sort/unstable/quicksort.rs:
// partition, partition_lomuto_branchless_cyclic; sort/shared/smallsort.rs:
// insertion_sort_shift_left). It cannot be run against rustc here (no Rust
// toolchain), so the element order it leaves at exact key ties is unpinned.
// Keys that differ are split the same way by any correct selection, so tree
// topology only depends on this code when the median key is tied.
#pragma once
#include <cstddef>
#include <utility>
#include <vector>

namespace orc {

template <class T, class Less>
struct RustSelect {
  Less is_less;
  static constexpr size_t INSERTION_SORT_THRESHOLD = 16;
  static constexpr size_t PSEUDO_MEDIAN_REC_THRESHOLD = 64;

  static void swap_(T* v, size_t a, size_t b) { std::swap(v[a], v[b]); }

  void insertion_sort_shift_left(T* v, size_t len, size_t offset) {
    for (size_t i = offset; i < len; i++) {
      // insert_tail(&mut v[..=i])
      if (is_less(v[i], v[i - 1])) {
        T tmp = v[i];
        size_t j = i;
        do {
          v[j] = v[j - 1];
          j--;
        } while (j > 0 && is_less(tmp, v[j - 1]));
        v[j] = tmp;
      }
    }
  }

  size_t min_index(const T* v, size_t len) {
    size_t acc = 0;
    for (size_t i = 1; i < len; i++)
      if (is_less(v[i], v[acc])) acc = i;
    return acc;
  }
  size_t max_index(const T* v, size_t len) {
    size_t acc = 0;
    for (size_t i = 1; i < len; i++)
      if (is_less(v[acc], v[i])) acc = i;
    return acc;
  }

  // pivot.rs median3: returns the index (relative to v) of the median of a, b, c.
  size_t median3(const T* v, size_t a, size_t b, size_t c) {
    bool x = is_less(v[a], v[b]);
    bool y = is_less(v[a], v[c]);
    if (x == y) {
      bool z = is_less(v[b], v[c]);
      return (z ^ x) ? c : b;
    }
    return a;
  }
  size_t median3_rec(const T* v, size_t a, size_t b, size_t c, size_t n) {
    if (n * 8 >= PSEUDO_MEDIAN_REC_THRESHOLD) {
      size_t n8 = n / 8;
      a = median3_rec(v, a, a + n8 * 4, a + n8 * 7, n8);
      b = median3_rec(v, b, b + n8 * 4, b + n8 * 7, n8);
      c = median3_rec(v, c, c + n8 * 4, c + n8 * 7, n8);
    }
    return median3(v, a, b, c);
  }
  size_t choose_pivot(const T* v, size_t len) {
    size_t len_div_8 = len / 8;
    size_t a = 0, b = len_div_8 * 4, c = len_div_8 * 7;
    if (len < PSEUDO_MEDIAN_REC_THRESHOLD) return median3(v, a, b, c);
    return median3_rec(v, a, b, c, len_div_8);
  }

  // Branchless Lomuto partition with a cyclic permutation (Bergdoll & Peters).
  // Partitions v[0..len) against `pivot` (which is not inside v); returns the
  // number of elements for which less(elem, pivot) holds.
  template <class L>
  size_t lomuto_cyclic(T* v, size_t len, const T& pivot, L&& less) {
    if (len == 0) return 0;
    T gap_value = v[0];
    size_t gap_pos = 0;
    size_t num_lt = 0;
    // The loop body is identical for the unrolled and the tail parts.
    for (size_t right = 1; right < len; right++) {
      T x = v[right];
      bool lt = less(x, pivot);
      v[gap_pos] = v[num_lt];
      v[num_lt] = x;
      gap_pos = right;
      num_lt += lt ? 1 : 0;
    }
    {
      // final step: the element at `right` is the saved gap value
      T x = gap_value;
      bool lt = less(x, pivot);
      v[gap_pos] = v[num_lt];
      v[num_lt] = x;
      num_lt += lt ? 1 : 0;
    }
    return num_lt;
  }

  template <class L>
  size_t partition(T* v, size_t len, size_t pivot, L&& less) {
    if (len == 0) return 0;
    swap_(v, 0, pivot);
    T pv = v[0];
    size_t num_lt = lomuto_cyclic(v + 1, len - 1, pv, less);
    swap_(v, 0, num_lt);
    return num_lt;
  }

  void ninther(T* v, size_t a, size_t b, size_t c, size_t d, size_t e, size_t f, size_t g, size_t h,
               size_t i) {
    b = median_idx(v, a, b, c);
    h = median_idx(v, g, h, i);
    if (is_less(v[h], v[b])) std::swap(b, h);
    if (is_less(v[f], v[d])) std::swap(d, f);
    if (is_less(v[e], v[d])) {
      // do nothing
    } else if (is_less(v[f], v[e])) {
      d = f;
    } else {
      if (is_less(v[e], v[b])) {
        swap_(v, e, b);
      } else if (is_less(v[h], v[e])) {
        swap_(v, e, h);
      }
      return;
    }
    if (is_less(v[d], v[b])) {
      d = b;
    } else if (is_less(v[h], v[d])) {
      d = h;
    }
    swap_(v, d, e);
  }
  size_t median_idx(const T* v, size_t a, size_t b, size_t c) {
    if (is_less(v[c], v[a])) std::swap(a, c);
    if (is_less(v[c], v[b])) return c;
    if (is_less(v[b], v[a])) return a;
    return b;
  }
  size_t median_of_ninthers(T* v, size_t len) {
    size_t frac;
    if (len <= 1024) frac = len / 12;
    else if (len <= (size_t)128 * 1024) frac = len / 64;
    else frac = len / 1024;
    size_t pivot = frac / 2;
    size_t lo = len / 2 - pivot;
    size_t hi = frac + lo;
    size_t gap = (len - 9 * frac) / 4;
    size_t a = lo - 4 * frac - gap;
    size_t b = hi + gap;
    for (size_t i = lo; i < hi; i++) {
      ninther(v, a, i - frac, b, a + 1, i, b + 1, a + 2, i + frac, b + 2);
      a += 3;
      b += 3;
    }
    median_of_medians(v + lo, frac, pivot);
    return partition(v, len, lo + pivot, is_less);
  }
  void median_of_medians(T* v, size_t len, size_t k) {
    for (;;) {
      if (len <= INSERTION_SORT_THRESHOLD) {
        if (len >= 2) insertion_sort_shift_left(v, len, 1);
        return;
      }
      if (k == len - 1) {
        size_t mi = max_index(v, len);
        swap_(v, mi, k);
        return;
      } else if (k == 0) {
        size_t mi = min_index(v, len);
        swap_(v, mi, k);
        return;
      }
      size_t p = median_of_ninthers(v, len);
      if (p == k) return;
      if (p > k) {
        len = p;
      } else {
        v = v + p + 1;
        len = len - p - 1;
        k -= p + 1;
      }
    }
  }

  void partition_at_index_loop(T* v, size_t len, size_t index) {
    int limit = 16;
    bool has_ancestor = false;
    T ancestor{};
    for (;;) {
      if (len <= INSERTION_SORT_THRESHOLD) {
        if (len >= 2) insertion_sort_shift_left(v, len, 1);
        return;
      }
      if (limit == 0) {
        median_of_medians(v, len, index);
        return;
      }
      limit--;
      size_t pivot_pos = choose_pivot(v, len);
      if (has_ancestor) {
        if (!is_less(ancestor, v[pivot_pos])) {
          auto ge = [this](const T& a, const T& b) { return !is_less(b, a); };
          size_t num_lt = partition(v, len, pivot_pos, ge);
          size_t mid = num_lt + 1;
          if (mid > index) return;
          v = v + mid;
          len -= mid;
          index -= mid;
          has_ancestor = false;
          continue;
        }
      }
      size_t num_lt = partition(v, len, pivot_pos, is_less);
      if (num_lt < index) {
        ancestor = v[num_lt];
        has_ancestor = true;
        v = v + num_lt + 1;
        len = len - num_lt - 1;
        index = index - num_lt - 1;
      } else if (num_lt > index) {
        len = num_lt;
      } else {
        return;
      }
    }
  }

  void select_nth(T* v, size_t len, size_t index) {
    if (index >= len) return;  // Rust panics; callers never pass this
    if (index == len - 1) {
      size_t mi = max_index(v, len);
      swap_(v, mi, index);
    } else if (index == 0) {
      size_t mi = min_index(v, len);
      swap_(v, mi, index);
    } else {
      partition_at_index_loop(v, len, index);
    }
  }
};

}  // namespace orc
