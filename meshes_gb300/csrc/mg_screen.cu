// Output/input phase screen of a mesh: u <- diag(exp(i ph)) u, its forward-mode derivative and the
// gradient with respect to the N screen phases.
//
// The reference applies the screen inside its CPU helper (c/dot.cpp:97-143, pos = 0 before the mesh,
// 1 after it) and forbids it in its GPU API (gpu/mesh.py:65).  Here it is a separate elementwise pass
// over the (B, N) field: HBM-bound, one read and one write of the field (about 1% of a deep mesh's
// propagation time at N = 256), so it is not fused into the propagation kernels.
//
// The gradient is reduced deterministically: one CTA per 32 modes, 8 thread rows summing batch rows
// b = row, row + 8, ... in order, then the 8 row sums combined in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

constexpr int kCols = 32, kRows = 8;

// u_out = exp(i sgn ph) u_in; with du: du_out = exp(i sgn ph) du_in + i dph u_out
__global__ void __launch_bounds__(256)
screen_kernel(int N, int B, const float* __restrict__ ph, const float* __restrict__ dph, float sgn,
              const float2* u_in, float2* u_out, const float2* du_in, float2* du_out, int ldu) {
  const long long n = (long long)N * B;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(idx / N), k = (int)(idx - (long long)b * N);
    float s, c;
    sincosf(sgn * __ldg(ph + k), &s, &c);
    const size_t o = (size_t)b * ldu + k;
    const float2 u = u_in[o];
    const float2 y = make_float2(c * u.x - s * u.y, c * u.y + s * u.x);
    u_out[o] = y;
    if (du_out) {
      const float2 d = du_in ? du_in[o] : make_float2(0.f, 0.f);
      const float dp = dph ? __ldg(dph + k) : 0.f;
      du_out[o] = make_float2(c * d.x - s * d.y - dp * y.y, c * d.y + s * d.x + dp * y.x);
    }
  }
}

// dph[k] (= or +=) sum_b Re(conj(g_bk) i u_bk) = sum_b (g.y u.x - g.x u.y), the derivative of a real J
// through u_k = exp(i ph_k) v_k, with u taken after the screen and g = 2 dJ/du* there
__global__ void __launch_bounds__(kCols * kRows)
screen_grad_kernel(int N, int B, const float2* __restrict__ u, const float2* __restrict__ g, int ldu, float* dph,
                   int accumulate) {
  __shared__ float acc[kRows][kCols];
  const int col = threadIdx.x % kCols, row = threadIdx.x / kCols;
  const int k = blockIdx.x * kCols + col;
  float sum = 0.f;
  if (k < N)
    for (int b = row; b < B; b += kRows) {
      const float2 uu = u[(size_t)b * ldu + k], gg = g[(size_t)b * ldu + k];
      sum += gg.y * uu.x - gg.x * uu.y;
    }
  acc[row][col] = sum;
  __syncthreads();
  if (row != 0 || k >= N) return;
  for (int r = 1; r < kRows; ++r) sum += acc[r][col];
  dph[k] = accumulate ? dph[k] + sum : sum;
}

int field_ok(const void* p) { return p == nullptr || (reinterpret_cast<uintptr_t>(p) & 7) == 0; }

}  // namespace

extern "C" {

int mg_phase_screen(int N, int B, const float* ph, const float* dph, int sgn, const void* u_in, void* u_out,
                    const void* du_in, void* du_out, int ldu, void* stream) {
  if (N < 1 || B < 0 || ldu < N) return mg::set_last_error(MG_E_ARG, "mg_phase_screen: N=%d B=%d ldu=%d", N, B, ldu);
  if (sgn != 1 && sgn != -1) return mg::set_last_error(MG_E_ARG, "mg_phase_screen: sgn=%d not +-1", sgn);
  if (B == 0) return mg::set_last_error(MG_OK, "%s", "");
  if (!ph || !u_in || !u_out) return mg::set_last_error(MG_E_ARG, "mg_phase_screen: ph, u_in and u_out are required");
  if (!field_ok(u_in) || !field_ok(u_out) || !field_ok(du_in) || !field_ok(du_out))
    return mg::set_last_error(MG_E_ARG, "mg_phase_screen: fields must be 8-byte aligned");
  if ((dph || du_in) && !du_out) return mg::set_last_error(MG_E_ARG, "mg_phase_screen: du_out is NULL");
  const long long n = (long long)N * B;
  const int grid = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
  screen_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      N, B, ph, dph, (float)sgn, static_cast<const float2*>(u_in), static_cast<float2*>(u_out),
      static_cast<const float2*>(du_in), static_cast<float2*>(du_out), ldu);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mg::set_last_error(MG_E_CUDA, "screen_kernel launch: %s", cudaGetErrorString(e));
  return mg::set_last_error(MG_OK, "%s", "");
}

int mg_phase_screen_grad(int N, int B, const void* u, const void* g, int ldu, float* dph, int accumulate,
                         void* stream) {
  if (N < 1 || B < 0 || ldu < N) return mg::set_last_error(MG_E_ARG, "mg_phase_screen_grad: N=%d B=%d ldu=%d", N, B, ldu);
  if (!dph || (B > 0 && (!u || !g))) return mg::set_last_error(MG_E_ARG, "mg_phase_screen_grad: NULL argument");
  if (!field_ok(u) || !field_ok(g)) return mg::set_last_error(MG_E_ARG, "mg_phase_screen_grad: fields must be 8-byte aligned");
  screen_grad_kernel<<<(N + kCols - 1) / kCols, kCols * kRows, 0, static_cast<cudaStream_t>(stream)>>>(
      N, B, static_cast<const float2*>(u), static_cast<const float2*>(g), ldu, dph, accumulate);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mg::set_last_error(MG_E_CUDA, "screen_grad_kernel launch: %s", cudaGetErrorString(e));
  return mg::set_last_error(MG_OK, "%s", "");
}

}  // extern "C"
