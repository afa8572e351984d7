// Persistent multi-mesh propagation: one launch drains a (mesh, batch-tile) work queue.
//
// Every CTA (256 threads, one per SM) repeatedly takes the next work item from a device counter and
// runs the same per-tile body as the one-mesh kernel (prop_body) on it: the item's mesh descriptor
// gives N, L, the coefficient tiles (built beforehand and kept resident) and the field pointers; the
// item gives the vector range.  Meshes of different N and depth share one launch; the kernel class
// of a mesh (complex M = 8, complex M = 16, real M = 8) selects the compiled body, the lane count
// G = N/M is a run-time value.  Items are taken in array order, so a host that sorts them
// longest-first gets longest-processing-time scheduling.
#include <cuda_runtime.h>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace mg {
namespace {

constexpr int kBatchWarps = 8;

__device__ __forceinline__ int cls_M(int cls) { return cls == MG_BCLS_C16 ? 16 : 8; }

// NN: every mesh of the launch is nearest-neighbour (layer kinds 0 and odd-shift), so the bodies without
// the strided and butterfly layers run (fewer registers; a mesh with another kind is refused per item).
// CLS >= 0: every item's mesh is of kernel class CLS (others are refused per item) and only that class's body
// is compiled.  GT = 32 (class MG_BCLS_C8 with MG_BATCH_FULL_WARP): every item's mesh has a vector filling
// the warp (G = 32, N in (128, 256]) and the body has a compile-time lane group.  All batched bodies keep the
// one-vector crossings: the packed forms spilled in the three-class kernel (13% slower) and, in the G = 32
// launch, raised the ALU pipe from 11% to 42% of cycles (measured on GB300: the 512-mesh fwd+bwd 285 against
// 318 G MZI-apps/s with the one-vector body).
template <int OP, bool NN, int CLS = -1, int GT = 0>
__global__ void __launch_bounds__(kBatchWarps * 32, 1)
batched_kernel(const mg_batch_mesh* __restrict__ meshes, int n_meshes, const mg_batch_item* __restrict__ items,
               int n_items, int* head, int* status) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int s_item;
  for (;;) {
    __syncthreads();                       // previous item fully done (barriers, smem reuse)
    if (threadIdx.x == 0) s_item = atomicAdd(head, 1);
    __syncthreads();
    const int i = s_item;
    if (i >= n_items) return;
    const mg_batch_item it = items[i];
    if (it.mesh < 0 || it.mesh >= n_meshes) {
      if (threadIdx.x == 0) set_status(status, ST_BAD_WORK);
      continue;
    }
    const mg_batch_mesh md = meshes[it.mesh];
    if ((CLS >= 0 && md.cls != CLS) || (GT > 0 && md.G != GT)) {
      if (threadIdx.x == 0) set_status(status, ST_BAD_WORK);
      continue;
    }
    const int M = cls_M(md.cls);
    if (md.G < 1 || md.G > 32 || (md.G & (md.G - 1)) || md.G * M < md.N || it.v0 < 0 || it.vend > md.B) {
      if (threadIdx.x == 0) set_status(status, ST_BAD_WORK);
      continue;
    }
    PropArgs a{};
    a.N = md.N; a.L = md.L; a.B = md.B; a.ldu = md.ldu;
    a.G = md.G; a.logG = 31 - __clz(md.G); a.W = kBatchWarps; a.CL = md.CL; a.S = md.S;
    a.layer_bytes = md.layer_bytes; a.dlayer_bytes = 0;
    a.tiles = static_cast<const unsigned char*>(md.tiles); a.dtiles = nullptr;
    a.kinds = md.kinds;
    a.in0 = md.in0; a.in1 = md.in1; a.out0 = md.out0; a.out1 = md.out1;
    a.partial = (OP == OP_BWD) ? static_cast<float2*>(md.partial) + (size_t)it.part * md.L * (md.G * M / 2) : nullptr;
    a.status = status;
    a.v0 = it.v0; a.vend = it.vend;
    a.target = nullptr;
    a.perm = a.pflags = a.perm_last = a.pflag_last = nullptr;   // batched meshes carry no permutations
    if constexpr (NN) {
      // the nearest-neighbour bodies know layer kinds 0 and odd-shift only: an item whose mesh has another
      // kind is refused (status, no output)
      int bad = 0;
      for (int l = threadIdx.x; l < md.L; l += blockDim.x) {
        const int k = __ldg(md.kinds + l);
        bad |= (k != 0 && k != KIND_MIS);
      }
      if (__syncthreads_or(bad)) {
        if (threadIdx.x == 0) set_status(status, ST_BAD_GEOMETRY);
        continue;
      }
    }
    if constexpr (CLS == MG_BCLS_C8) {
      prop_body<OP, 8, 4, false, GT, (OP == OP_BWD ? 1 : 0), false, NN, false>(a, smem);
    } else if constexpr (CLS == MG_BCLS_C16) {
      prop_body<OP, 16, 2, false, 0, (OP == OP_BWD ? 1 : 0), false, NN, false>(a, smem);
    } else if constexpr (CLS == MG_BCLS_R8) {
      prop_body<OP, 8, 4, true, GT, (OP == OP_BWD ? 2 : 0), false, NN>(a, smem);
    } else {
      switch (md.cls) {
        // one-vector crossings here: with three class bodies in one kernel the packed forms made
        // back-propagation spill and gained nothing going forward (measured on GB300: the batched engine
        // 13% and 3.5% slower)
        case MG_BCLS_C8:
          // nearest-neighbour forward launches: compile-time lane groups for G = 32, 16, 8 (no run-time lane
          // index arithmetic; 2% faster on the 512-mesh benchmark).  Back-propagation keeps the run-time body:
          // a second one made the 254-register kernel spill.
          if (NN && OP == OP_FWD && md.G == 32) prop_body<OP, 8, 4, false, 32, 0, false, NN, false>(a, smem);
          else if (NN && OP == OP_FWD && md.G == 16) prop_body<OP, 8, 4, false, 16, 0, false, NN, false>(a, smem);
          else if (NN && OP == OP_FWD && md.G == 8) prop_body<OP, 8, 4, false, 8, 0, false, NN, false>(a, smem);
          else prop_body<OP, 8, 4, false, 0, (OP == OP_BWD ? 1 : 0), false, NN, false>(a, smem);
          break;
        case MG_BCLS_C16: prop_body<OP, 16, 2, false, 0, (OP == OP_BWD ? 1 : 0), false, NN, false>(a, smem); break;
        case MG_BCLS_R8: prop_body<OP, 8, 4, true, 0, (OP == OP_BWD ? 2 : 0), false, NN>(a, smem); break;
        default:
          if (threadIdx.x == 0) set_status(status, ST_BAD_WORK);
      }
    }
  }
}

// dp[l][q][k] = sum over the mesh's items (in item order) of the partials.  Grid (meshes, kReduceY): the
// kReduceY CTAs of a mesh stride over its slot positions, one position per thread at a time, consecutive
// threads on consecutive positions (coalesced); each thread keeps 8 item loads in flight and adds them in item
// order, so the sums are those of a plain sequential loop.  (One CTA per mesh, one load in flight per thread,
// took 3.85 ms on the 512-mesh benchmark - 23% of its forward + backward step.)
constexpr int kReduceY = 64;
__global__ void batched_reduce_kernel(const mg_batch_mesh* __restrict__ meshes) {
  const mg_batch_mesh md = meshes[blockIdx.x];
  if (!md.dp || !md.partial || md.n_items <= 0) return;
  const int M = cls_M(md.cls), G = md.G, np2 = G * M / 2, L = md.L, N = md.N;
  const int* geo = md.kinds + L;
  const float2* part = static_cast<const float2*>(md.partial);
  const size_t stride = (size_t)L * np2;
  const int n = md.n_items;
  for (int idx = blockIdx.y * blockDim.x + threadIdx.x; idx < L * np2; idx += gridDim.y * blockDim.x) {
    const int l = idx / np2, pos = idx - l * np2;
    const int q = pos_slot(pos, M, G);
    if (q >= N / 2) continue;
    const int sh = geo[2 * l], ln = geo[2 * l + 1];
    float sx = 0.f, sy = 0.f;
    if (q >= sh / 2 && q < sh / 2 + ln) {
      const float2* p = part + (size_t)l * np2 + pos;
      int k = 0;
      for (; k + 8 <= n; k += 8) {
        float2 v[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] = p[(size_t)(k + i) * stride];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          sx += v[i].x;
          sy += v[i].y;
        }
      }
      for (; k < n; ++k) {
        const float2 v = p[(size_t)k * stride];
        sx += v.x;
        sy += v.y;
      }
    }
    float* o = md.dp + (size_t)l * md.ldp + (size_t)q * md.n_p;
    o[0] = sx;
    if (md.n_p > 1) o[1] = sy;
  }
}

}  // namespace
}  // namespace mg

using namespace mg;

namespace {
template <int OP, bool NN, int CLS, int GT>
cudaError_t launch_batched(const mg_batch_mesh* meshes, int n_meshes, const mg_batch_item* items, int n_items, int* head,
                           int grid, size_t smem, int* status, cudaStream_t st) {
  static std::atomic<unsigned long long> done{0};
  cudaError_t e = ensure_smem_attr(batched_kernel<OP, NN, CLS, GT>, done);
  if (e == cudaSuccess)
    batched_kernel<OP, NN, CLS, GT><<<grid, kBatchWarps * 32, smem, st>>>(meshes, n_meshes, items, n_items, head, status);
  return e;
}
template <int OP, int CLS, int GT = 0>
cudaError_t launch_batched_nn(bool nn, const mg_batch_mesh* meshes, int n_meshes, const mg_batch_item* items,
                              int n_items, int* head, int grid, size_t smem, int* status, cudaStream_t st) {
  return nn ? launch_batched<OP, true, CLS, GT>(meshes, n_meshes, items, n_items, head, grid, smem, status, st)
            : launch_batched<OP, false, CLS, GT>(meshes, n_meshes, items, n_items, head, grid, smem, status, st);
}
template <int OP>
cudaError_t launch_batched_cls(int cls, bool full, bool nn, const mg_batch_mesh* meshes, int n_meshes,
                               const mg_batch_item* items, int n_items, int* head, int grid, size_t smem, int* status,
                               cudaStream_t st) {
  switch (cls) {
    case MG_BCLS_C8:
      return full ? launch_batched_nn<OP, MG_BCLS_C8, 32>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st)
                  : launch_batched_nn<OP, MG_BCLS_C8>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
    case MG_BCLS_C16: return launch_batched_nn<OP, MG_BCLS_C16>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
    case MG_BCLS_R8:
      return full ? launch_batched_nn<OP, MG_BCLS_R8, 32>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st)
                  : launch_batched_nn<OP, MG_BCLS_R8>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
    default: return launch_batched_nn<OP, -1>(nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
  }
}
}  // namespace

extern "C" int mg_batched_propagate(int op, const mg_batch_mesh* meshes, int n_meshes, const mg_batch_item* items,
                                    int n_items, int* head, int grid, size_t smem, int* status, void* stream) {
  const bool nn = (op & MG_BATCH_NN) != 0;
  const bool full = (op & MG_BATCH_FULL_WARP) != 0;
  const int cls = ((op >> 8) & 0xff) - 1;   // MG_BATCH_ONLY(cls): one class per launch, -1 any
  op &= 0x0f;
  if (cls < -1 || cls > MG_BCLS_R8) return set_last_error(MG_E_ARG, "batched class %d not in {0,1,2}", cls);
  if (full && cls != MG_BCLS_C8 && cls != MG_BCLS_R8)
    return set_last_error(MG_E_ARG, "MG_BATCH_FULL_WARP needs MG_BATCH_ONLY(MG_BCLS_C8) or MG_BATCH_ONLY(MG_BCLS_R8)");
  if (op != MG_OP_FWD && op != MG_OP_BWD) return set_last_error(MG_E_ARG, "batched op must be fwd or bwd");
  if (!meshes || n_meshes < 0 || (!items && n_items > 0) || !head || grid < 1)
    return set_last_error(MG_E_ARG, "batched launch: bad arguments");
  if (n_items == 0) return MG_OK;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem + 1024 > (size_t)optin) return set_last_error(MG_E_CONFIG, "batched smem %zu above %d", smem, optin);
  (void)cudaGetLastError();   // start from a clean error state: launch errors below are this call's
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (op == MG_OP_FWD)
    e = launch_batched_cls<OP_FWD>(cls, full, nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
  else
    e = launch_batched_cls<OP_BWD>(cls, full, nn, meshes, n_meshes, items, n_items, head, grid, smem, status, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : set_last_error(MG_E_CUDA, "batched_kernel: %s", cudaGetErrorString(e));
}

extern "C" int mg_batched_reduce(const mg_batch_mesh* meshes, int n_meshes, void* stream) {
  if (!meshes || n_meshes < 0) return set_last_error(MG_E_ARG, "batched reduce: bad arguments");
  if (n_meshes == 0) return MG_OK;
  batched_reduce_kernel<<<dim3(n_meshes, kReduceY), 256, 0, static_cast<cudaStream_t>(stream)>>>(meshes);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : set_last_error(MG_E_CUDA, "batched_reduce_kernel: %s", cudaGetErrorString(e));
}
