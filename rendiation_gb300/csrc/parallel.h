// Device-wide scan, stream compaction and radix sort (parallel.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace rdn {

size_t scan_scratch_bytes(uint32_t n);
// segment: 0, or a power of two at which an inclusive scan restarts.
// as_flags: scan (in != 0) instead of in.
cudaError_t scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, bool inclusive, uint32_t segment, void* scratch,
                     cudaStream_t stream, bool as_flags = false);
size_t compact_scratch_bytes(uint32_t n);
cudaError_t compact_u32(const uint32_t* values, const uint32_t* flags, uint32_t* out, uint32_t* count, uint32_t n,
                        void* scratch, cudaStream_t stream);
size_t sort_scratch_bytes(uint32_t n);
// n_dev (nullable): device-resident element count (<= n, the capacity); the
// launches are sized by n and elements at or past *n_dev are left alone.
cudaError_t radix_sort_u32(uint32_t* keys, uint32_t* vals, uint32_t n, uint32_t key_bits, void* scratch,
                           cudaStream_t stream, const uint32_t* n_dev = nullptr);

}  // namespace rdn
