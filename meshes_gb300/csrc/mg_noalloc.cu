// mg_fwdprop_noalloc: forward propagation for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc or an allocator: plugin hosts that own the device heap and forbid side
// allocations, or real-time loops that must not hit the allocator's locks and possible synchronisations.
// mg_fwdprop needs a scratch workspace (coefficient tiles, layer kinds, a status word) that the caller
// normally provides; this entry point instead uses one scratch array compiled into the library.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes (8 MiB).  Every GPU that loads
// the library holds it until the process exits.  Its host-side name is only a stand-in for the symbol,
// not a device address, so the device address is looked up with cudaGetSymbolAddress once per device,
// with that device current, on the first call made on that device.
//
// Every call shares the one array: calls that overlap on the GPU (different streams, or host threads
// issuing to the same device without ordering) race on it and corrupt each other's coefficients.
// Serialise them (one stream, or events).  Each call zeroes the status word it relies on; the tiles
// and kinds are fully rewritten by every call.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;   // 8 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_addr[64] = {};

// Device address of the scratch array on the current device (looked up once per device).
cudaError_t scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int mg_fwdprop_noalloc(int N, int L, int B, const int* lens, const int* shifts, const float* p, int ldp,
                                  const float* s, int lds, const void* u_in, void* u_out, int ldu, int crossing,
                                  void* stream) {
  const size_t need = mg_workspace_bytes(MG_OP_FWD, N, L, B, crossing, MG_GEO_NN, nullptr);
  if (need == 0) return MG_E_ARG;   // the argument error is already in mg_last_error()
  if (need > kNoAllocScratchBytes)
    return mg::set_last_error(MG_E_WORKSPACE,
                              "mg_fwdprop_noalloc: N=%d, L=%d needs %zu bytes of scratch, above its fixed %zu-byte "
                              "array; use mg_fwdprop with a caller workspace",
                              N, L, need, kNoAllocScratchBytes);
  void* scratch = nullptr;
  cudaError_t e = scratch_address(&scratch);
  if (e != cudaSuccess)
    return mg::set_last_error(MG_E_CUDA, "mg_fwdprop_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
  // the status word must start at zero; everything else is rewritten by the call
  e = cudaMemsetAsync(scratch, 0, 256, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess)
    return mg::set_last_error(MG_E_CUDA, "mg_fwdprop_noalloc: clearing status: %s", cudaGetErrorString(e));
  return mg_fwdprop(N, L, B, lens, shifts, p, ldp, s, lds, u_in, u_out, ldu, crossing, scratch, kNoAllocScratchBytes,
                    stream);
}
