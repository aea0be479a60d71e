// Device-wide scan, stream compaction and LSD radix sort for sm_103a: the
// parallel-compute primitives the reference's wavefront executor builds on
// (shader/parallel-compute/src/prefix_scan.rs:39-114 Kogge-Stone workgroup scan,
// lib.rs:398-429 two-level segmented scan, stream_compaction.rs:3-45,
// shuffle_move.rs:4-59, radix_sort.rs:29-74).
//
// The reference scans with one Kogge-Stone pass per workgroup and a second
// level over workgroup tails, which caps its length at WG^2 elements
// (lib.rs:395-397). Here:
//   scan     reduce-then-scan over 2048-element tiles (8 per thread, warp
//            shuffles inside a tile), recursing over the tile totals, so any
//            length up to 2^32-1 works; an optional power-of-two segment length
//            restarts the sum (the reference's workgroup-scoped scan).
//   compact  exclusive scan of keep-flags, then a scatter; the tail of the
//            output is zero-filled, as the reference's test expects.
//   sort     4 passes of 8-bit digits: per-tile digit histograms (digit-major),
//            one scan over them, and a stable scatter that ranks equal digits
//            inside a tile with warp __match_any_sync and per-warp offsets.
#include <cuda_runtime.h>

#include <cstdint>

#include "parallel.h"

namespace rdn {
namespace {

constexpr uint32_t SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr uint32_t SORT_THREADS = 256, SORT_ROUNDS = 4, SORT_TILE = SORT_THREADS * SORT_ROUNDS;

__device__ __forceinline__ uint32_t warp_inclusive(uint32_t v) {
  const uint32_t lane = threadIdx.x & 31u;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (uint32_t)o) v += n;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t inc = warp_inclusive(v);
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const uint32_t nw = blockDim.x >> 5;
    uint32_t w = lane < nw ? warp_sums[lane] : 0u;
    const uint32_t wi = warp_inclusive(w);
    if (lane < nw) warp_sums[lane] = wi - w;
    if (lane == nw - 1) warp_sums[32] = wi;
  }
  __syncthreads();
  total = warp_sums[32];
  const uint32_t r = warp_sums[warp] + inc - v;
  __syncthreads();
  return r;
}

// Per-tile scan of `in` (exclusive or inclusive) into `out`; tile totals to `sums`.
// as_flags: scan (in != 0) instead of in (keep-flags of a compaction)
__global__ void __launch_bounds__(SCAN_THREADS) tile_scan(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                          uint32_t n, int inclusive, int as_flags,
                                                          uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_sums[33];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE + (size_t)threadIdx.x * SCAN_ITEMS;
  uint32_t v[SCAN_ITEMS];
  uint32_t local = 0;
#pragma unroll
  for (int k = 0; k < (int)SCAN_ITEMS; k++) {
    v[k] = (base + k < n) ? (as_flags ? (uint32_t)(in[base + k] != 0u) : in[base + k]) : 0u;
    local += v[k];
  }
  uint32_t total;
  uint32_t run = block_exclusive(local, warp_sums, total);
#pragma unroll
  for (int k = 0; k < (int)SCAN_ITEMS; k++) {
    const uint32_t x = v[k];
    if (base + k < n) out[base + k] = inclusive ? run + x : run;
    run += x;
  }
  if (threadIdx.x == 0 && sums) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) add_tile_offsets(uint32_t* __restrict__ out, uint32_t n,
                                                                 const uint32_t* __restrict__ offsets) {
  const uint32_t add = offsets[blockIdx.x];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  for (uint32_t k = threadIdx.x; k < SCAN_TILE; k += SCAN_THREADS)
    if (base + k < n) out[base + k] += add;
}

// out[i] = incl[i] - incl[segment start - 1]  (inclusive segmented scan)
__global__ void segment_rebase(const uint32_t* __restrict__ incl, uint32_t* __restrict__ out, uint32_t n,
                               uint32_t segment) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t s = (i / segment) * segment;
  out[i] = incl[i] - (s ? incl[s - 1] : 0u);
}

__global__ void compact_scatter(const uint32_t* __restrict__ values, const uint32_t* __restrict__ flags,
                                const uint32_t* __restrict__ pos, uint32_t* __restrict__ out, uint32_t n,
                                uint32_t* __restrict__ count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t f = flags[i] != 0u;
  if (f) out[pos[i]] = values[i];
  if (i == n - 1) *count = pos[i] + f;
}

__global__ void zero_tail(uint32_t* __restrict__ out, uint32_t n, const uint32_t* __restrict__ count) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && i >= *count) out[i] = 0u;
}

// digit histogram of one tile, written digit-major: hist[d * tiles + tile]
// n_dev (nullable): the element count lives on the device; n is the capacity
__device__ __forceinline__ uint32_t live_count(uint32_t n, const uint32_t* n_dev) {
  if (!n_dev) return n;
  const uint32_t d = *n_dev;
  return d < n ? d : n;
}

__global__ void __launch_bounds__(SORT_THREADS) sort_histogram(const uint32_t* __restrict__ keys, uint32_t n_cap,
                                                               const uint32_t* __restrict__ n_dev, uint32_t shift,
                                                               uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t h[256];
  const uint32_t n = live_count(n_cap, n_dev);
  h[threadIdx.x] = 0u;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * SORT_TILE;
  for (uint32_t r = 0; r < SORT_ROUNDS; r++) {
    const size_t i = base + (size_t)r * SORT_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// stable scatter of one tile using the scanned digit offsets
__global__ void __launch_bounds__(SORT_THREADS) sort_scatter(const uint32_t* __restrict__ keys_in,
                                                             const uint32_t* __restrict__ vals_in,
                                                             uint32_t* __restrict__ keys_out,
                                                             uint32_t* __restrict__ vals_out, uint32_t n_cap,
                                                             const uint32_t* __restrict__ n_dev, uint32_t shift,
                                                             const uint32_t* __restrict__ offsets, uint32_t tiles) {
  constexpr uint32_t WARPS = SORT_THREADS / 32;
  const uint32_t n = live_count(n_cap, n_dev);
  __shared__ uint32_t run[256];          // running position of each digit in this tile
  __shared__ uint32_t wcount[WARPS][256];  // per-warp digit counts of the current round
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  run[threadIdx.x] = offsets[(size_t)threadIdx.x * tiles + blockIdx.x];
  const size_t base = (size_t)blockIdx.x * SORT_TILE;
  for (uint32_t r = 0; r < SORT_ROUNDS; r++) {
    for (uint32_t w = 0; w < WARPS; w++) wcount[w][threadIdx.x] = 0u;
    __syncthreads();
    const size_t i = base + (size_t)r * SORT_THREADS + threadIdx.x;
    const bool valid = i < n;
    const uint32_t key = valid ? keys_in[i] : 0u;
    const uint32_t d = valid ? (key >> shift) & 0xFFu : 256u;  // 256: no digit
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    const uint32_t leader = 31 - __clz(peers);  // highest lane of the group writes the count
    if (valid && lane == leader) wcount[warp][d] = __popc(peers);
    __syncthreads();
    // digit thread: exclusive prefix over warps, then advance the running position
    {
      const uint32_t dd = threadIdx.x;
      uint32_t acc = 0;
      for (uint32_t w = 0; w < WARPS; w++) {
        const uint32_t c = wcount[w][dd];
        wcount[w][dd] = acc;
        acc += c;
      }
      __syncthreads();
      if (valid) {
        const uint32_t dst = run[d] + wcount[warp][d] + rank;
        keys_out[dst] = key;
        if (vals_out) vals_out[dst] = vals_in[i];
      }
      __syncthreads();
      run[dd] += acc;
    }
    __syncthreads();
  }
}

inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

size_t scan_scratch_bytes(uint32_t n) {
  size_t bytes = 0;
  uint32_t len = n;
  while (len > SCAN_TILE) {
    len = (len + SCAN_TILE - 1) / SCAN_TILE;
    bytes += up256((size_t)len * 4);
  }
  return bytes + up256((size_t)n * 4) + 256;  // + a temporary for segmented scans
}

cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, bool inclusive, uint32_t segment, void* scratch,
                     cudaStream_t stream, bool as_flags) {
  if (n == 0) return cudaSuccess;
  char* s = static_cast<char*>(scratch);
  uint32_t* target = out;
  bool incl = inclusive;
  if (segment) {
    target = reinterpret_cast<uint32_t*>(s);
    s += up256((size_t)n * 4);
    incl = true;
  }
  // level 0 and the recursion over tile totals
  const uint32_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  uint32_t* sums = tiles > 1 ? reinterpret_cast<uint32_t*>(s) : nullptr;
  tile_scan<<<tiles, SCAN_THREADS, 0, stream>>>(in, target, n, incl ? 1 : 0, as_flags ? 1 : 0, sums);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (tiles > 1) {
    e = scan_u32(sums, sums, tiles, false, 0, s + up256((size_t)tiles * 4), stream, false);
    if (e != cudaSuccess) return e;
    add_tile_offsets<<<tiles, SCAN_THREADS, 0, stream>>>(target, n, sums);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (segment) {
    segment_rebase<<<(n + 255) / 256, 256, 0, stream>>>(target, out, n, segment);
    e = cudaGetLastError();
  }
  return e;
}

size_t compact_scratch_bytes(uint32_t n) { return up256((size_t)n * 4) + scan_scratch_bytes(n); }

cudaError_t compact_u32(const uint32_t* values, const uint32_t* flags, uint32_t* out, uint32_t* count, uint32_t n,
                        void* scratch, cudaStream_t stream) {
  if (n == 0) return cudaMemsetAsync(count, 0, 4, stream);
  uint32_t* pos = static_cast<uint32_t*>(scratch);
  void* rest = static_cast<char*>(scratch) + up256((size_t)n * 4);
  cudaError_t e = scan_u32(flags, pos, n, false, 0, rest, stream, true);
  if (e != cudaSuccess) return e;
  compact_scatter<<<(n + 255) / 256, 256, 0, stream>>>(values, flags, pos, out, n, count);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  zero_tail<<<(n + 255) / 256, 256, 0, stream>>>(out, n, count);
  return cudaGetLastError();
}

size_t sort_scratch_bytes(uint32_t n) {
  const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
  const size_t hist = (size_t)tiles * 256;
  return 2 * up256((size_t)n * 4) + 2 * up256(hist * 4) + scan_scratch_bytes((uint32_t)hist);
}

cudaError_t radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t key_bits, void* scratch,
                           cudaStream_t stream, const uint32_t* n_dev) {
  if (n <= 1) return cudaSuccess;
  const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
  const uint32_t hist_n = tiles * 256;
  char* s = static_cast<char*>(scratch);
  uint32_t* k_alt = reinterpret_cast<uint32_t*>(s);
  s += up256((size_t)n * 4);
  uint32_t* v_alt = reinterpret_cast<uint32_t*>(s);
  s += up256((size_t)n * 4);
  uint32_t* hist = reinterpret_cast<uint32_t*>(s);
  s += up256((size_t)hist_n * 4);
  uint32_t* offs = reinterpret_cast<uint32_t*>(s);
  s += up256((size_t)hist_n * 4);
  uint32_t* k_src = keys;
  uint32_t* v_src = vals;
  uint32_t* k_dst = k_alt;
  uint32_t* v_dst = vals ? v_alt : nullptr;
  const uint32_t passes = (key_bits + 7) / 8;
  for (uint32_t pass = 0; pass < passes; pass++) {
    const uint32_t shift = 8 * pass;
    sort_histogram<<<tiles, SORT_THREADS, 0, stream>>>(k_src, n, n_dev, shift, hist, tiles);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_u32(hist, offs, hist_n, false, 0, s, stream, false);
    if (e != cudaSuccess) return e;
    sort_scatter<<<tiles, SORT_THREADS, 0, stream>>>(k_src, v_src, k_dst, v_dst, n, n_dev, shift, offs, tiles);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t* t = k_src;
    k_src = k_dst;
    k_dst = t;
    t = v_src;
    v_src = v_dst;
    v_dst = vals ? t : nullptr;
  }
  if (k_src != keys) {
    // with a device-side count the copy covers the capacity (entries past the count are don't-care)
    cudaError_t e = cudaMemcpyAsync(keys, k_src, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    if (e != cudaSuccess) return e;
    if (vals) e = cudaMemcpyAsync(vals, v_src, (size_t)n * 4, cudaMemcpyDeviceToDevice, stream);
    return e;
  }
  return cudaSuccess;
}

}  // namespace rdn
