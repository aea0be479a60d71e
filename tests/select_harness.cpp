// Test harness: the product's select_nth_unstable restatement (iterative,
// host + device) against the oracle's (recursive) on the same keys.
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "../oracle/orc_select.h"
#include "../rendiation_gb300/csrc/rust_select.h"

extern "C" int compare_select(const float* keys, uint64_t n, uint64_t index, int worst_case_path) {
  auto less = [keys](const uint64_t& a, const uint64_t& b) {
    const float ka = keys[a], kb = keys[b];
    return std::isnan(ka) || std::isnan(kb) || ka < kb;
  };
  std::vector<uint64_t> a(n), b(n);
  std::iota(a.begin(), a.end(), 0);
  std::iota(b.begin(), b.end(), 0);
  rdn::RustSelectNth<uint64_t, decltype(less)> product(less);
  orc::RustSelect<uint64_t, decltype(less)> oracle{less};
  if (worst_case_path) {
    product.run_median_of_medians(a.data(), n, index);
    oracle.median_of_medians(b.data(), n, index);
  } else {
    product.run(a.data(), n, index);
    oracle.select_nth(b.data(), n, index);
  }
  return a == b ? 1 : 0;
}
