// Internal host-side launch plumbing shared by the instantiation units and the C ABI.
#pragma once
#include <atomic>
#include <cuda_runtime.h>

#include "mg_prop.cuh"

namespace mg {

struct LaunchCfg {
  dim3 grid, block;
  size_t smem;
  cudaStream_t stream;
};

// Raise a kernel's dynamic shared-memory limit to the device opt-in maximum, once per device.
template <typename K>
inline cudaError_t ensure_smem_attr(K kernel, std::atomic<unsigned long long>& done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  int optin = 0;
  e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (e != cudaSuccess) return e;
  // the dynamic limit is the opt-in maximum less the kernel's static shared memory
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, kernel);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();   // do not leave the failure for the next launch check to report
    return e;
  }
  done.fetch_or(bit, std::memory_order_acq_rel);
  return cudaSuccess;
}

template <int OP, int M, int V, bool REAL, int GT, int GR, bool PERM = false, bool NN = false, int MINB = 1>
inline cudaError_t launch_one(const LaunchCfg& lc, const PropArgs& a) {
  static std::atomic<unsigned long long> done{0};
  auto k = prop_kernel<OP, M, V, REAL, GT, GR, PERM, NN, MINB>;
  cudaError_t e = ensure_smem_attr(k, done);
  if (e != cudaSuccess) return e;
  k<<<lc.grid, lc.block, lc.smem, lc.stream>>>(a);
  return cudaGetLastError();
}

template <int OP, int M, int V, bool REAL, int GT, int GR, bool NN = false>
inline cudaError_t launch_split(const LaunchCfg& lc, const PropArgs& a) {
  static std::atomic<unsigned long long> done{0};
  auto k = prop_split_kernel<OP, M, V, REAL, GT, GR, NN>;
  cudaError_t e = ensure_smem_attr(k, done);
  if (e != cudaSuccess) return e;
  k<<<lc.grid, lc.block, lc.smem, lc.stream>>>(a);
  return cudaGetLastError();
}

// max threads per CTA the instantiation was compiled for
inline int prop_max_threads(int op, int M, int V) {
  return ((op == OP_FWD && M * V <= 16) || (op == OP_BWD && M * V <= 8)) ? 512 : 256;
}

// per-op dispatchers (one translation unit each, compiled in parallel)
// error message for mg_last_error(), set from any translation unit; returns `code`
int set_last_error(int code, const char* fmt, ...);

// full: a vector fills the warp (G = 32), selecting the compile-time-G instantiation;
// gr: back-propagation gradient mode (0 dJ/dT + dT/dp tiles, 1 MZI direct, 2 orth direct)
cudaError_t launch_prop(int op, bool real, int M, int V, bool full, int gr, const LaunchCfg& lc, const PropArgs& a);
// permuted meshes (a.perm set): the PERM instantiations, runtime lane-group size, the default V of each
// (op, M) and the gradient mode of each crossing (mg_prop_perm_*.cu)
bool perm_instantiated(int op, bool real, int M, int V, int gr);
cudaError_t launch_prop_perm(int op, bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
// nearest-neighbour instantiations (layer kinds 0 and odd-shift only) of the configurations in
// nn_instantiated(), uniform or split (mg_prop_nn.cu)
bool nn_instantiated(int op, bool real, int M, int V, int gr, bool full, bool split);
// the small-mesh tiles among them (complex, full warp, few modes and vectors per lane, so that a small batch
// spreads over more schedulers; forward, and back-propagation at 4 x 2; mg_prop_nn_small.cu)
bool nn_small_instantiated(int op, bool real, int M, int V, int gr, bool full);
cudaError_t launch_prop_nn_small(int op, int M, int V, const LaunchCfg& lc, const PropArgs& a);
// and the forward-mode derivative's full-warp tiles (mg_prop_nn_fwddiff.cu)
bool nn_fwddiff_instantiated(int op, bool real, int M, int V, int gr, bool full);
cudaError_t launch_prop_nn_fwddiff(bool real, int M, int V, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_prop_nn(int op, bool real, int M, int V, int gr, bool full, bool split, const LaunchCfg& lc,
                           const PropArgs& a);
// wide nearest-neighbour meshes (512 < N <= 640): kWideM modes in each of 32 lanes (mg_prop_wide.cu)
constexpr int kWideM = 20;
bool wide_instantiated(int op, bool real, int V, int gr);
cudaError_t launch_prop_wide(int op, bool real, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
// nearest-neighbour full-warp kernels compiled for two resident 256-thread CTAs per SM (at most 128 registers
// per thread): (op, M, V) in nn2_instantiated (mg_prop_nn.cu)
bool nn2_instantiated(int op, bool real, int M, int V, int gr);
cudaError_t launch_prop_nn2(int op, bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
// warp-pair back-propagation (mg_prop_pair.cu): a vector over the 64 lanes of two warps, 4 modes per lane, on
// the tiles of an M = 8, G = 32 plan; V counts vectors per pair
bool pair_instantiated(int op, bool real, int M, int V, int gr, bool full);
cudaError_t launch_prop_pair(int V, const LaunchCfg& lc, const PropArgs& a);
// split launches (two CTA kinds per SM); instantiated only for the full-warp configurations in
// split_instantiated()
bool split_instantiated(int op, bool real, int M, int V, bool full, int gr);
cudaError_t launch_prop_split(int op, bool real, int M, int V, bool full, int gr, const LaunchCfg& lc,
                              const PropArgs& a);

}  // namespace mg
