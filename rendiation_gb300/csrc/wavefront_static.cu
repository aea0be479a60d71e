// Allocation-free variant of the wavefront executor.
//
// rdn_wavefront_shadow_bounce needs device scratch for its shadow and bounce
// ray queues, which the caller allocates. Some callers cannot allocate device
// memory: a host whose device memory is all handed out up front by its own
// arena (a renderer that budgets every buffer at start-up and may not allocate
// inside its frame loop), or a foreign-language host that reaches librdn only
// through the C ABI and does not link the CUDA runtime allocator itself. For
// them, rdn_wavefront_shadow_bounce_static runs the same kernels with the
// queues in a fixed array compiled into the library.
//
// The array is a file-scope __device__ variable of RDN_WAVEFRONT_STATIC_SCRATCH_BYTES
// (32 MiB): every GPU that loads this library holds it until the process exits.
// Host code cannot use the array's name as a device address (on the host it is
// only a stand-in symbol), so the address is looked up with
// cudaGetSymbolAddress, with the device current: once when a context is
// created for the device (rdn_create), and again on every call whose stream is
// not capturing, so that a module reloaded after cudaDeviceReset is picked up;
// on a capturing stream the call keeps the cached address. The queue counters are cleared on the stream at the start of
// every call (by the shared launcher), the queues themselves need no clearing.
// All calls share the one array: calls that overlap on the GPU (different
// streams, or several contexts on one device) race on it and must be ordered
// by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "rdn_core.h"
#include "trace_kernels.h"
#include "wavefront.h"

namespace rdn {
namespace {

static __device__ __align__(256) unsigned char g_wavefront_scratch[RDN_WAVEFRONT_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_symbol_lock;
void* g_symbol_addr[kMaxDevices] = {};

// Looks the address up again (refresh) or returns the cached one; `device`
// must be current.
cudaError_t static_scratch_address(int device, bool refresh, void** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_symbol_lock);
  if (refresh || !g_symbol_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_wavefront_scratch);
    if (e != cudaSuccess) return e;
    g_symbol_addr[device] = p;
  }
  *out = g_symbol_addr[device];
  return cudaSuccess;
}

}  // namespace

cudaError_t wavefront_static_prepare(int device) {
  void* unused = nullptr;
  return static_scratch_address(device, true, &unused);
}

cudaError_t launch_wavefront_static(const TraceParams& p, WavefrontParams w, int mode, uint32_t block,
                                    int sm_count, uint32_t phases, int device, cudaStream_t stream) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) return e;
  void* scratch = nullptr;
  e = static_scratch_address(device, cap == cudaStreamCaptureStatusNone, &scratch);
  if (e != cudaSuccess) return e;
  wavefront_bind_scratch(w, scratch);
  return launch_wavefront(p, w, mode, block, sm_count, phases, stream);
}

}  // namespace rdn
