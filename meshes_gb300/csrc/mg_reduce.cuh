// Deterministic reductions of the back-propagation kernel's per-CTA partials (one translation unit includes
// this file: the kernels are not templates).
#pragma once
#include "mg_coeffs.cuh"

namespace mg {

// dp[l][q][k] (= or +=) sum over the nC per-CTA partials, deterministic.  Partials are stored in the
// lane-major slot order pos (slot_pos).  A block of 256 threads owns 32 consecutive positions; its 8
// thread rows sum the CTAs c = row, row+8, ... (many independent loads in flight), then the 8 row
// sums are combined in a fixed order through shared memory.
constexpr int kReduceCols = 32, kReduceRows = 8;
__global__ void __launch_bounds__(kReduceCols * kReduceRows)
dp_reduce_kernel(const float2* __restrict__ partial, int nC, int L, int np2, int M, int G, int N, float* dp, int ldp,
                 int n_p, int accumulate, const int* geo) {
  __shared__ float2 acc[kReduceRows][kReduceCols];
  const int col = threadIdx.x % kReduceCols, row = threadIdx.x / kReduceCols;
  const int idx = blockIdx.x * kReduceCols + col;
  const bool valid = idx < L * np2;
  const size_t stride = (size_t)L * np2;
  float sx = 0.f, sy = 0.f;
  if (valid) {
    const float2* p = partial + idx;
    int c = row;
    for (; c + 3 * kReduceRows < nC; c += 4 * kReduceRows) {
      const float2 a0 = __ldg(p + (size_t)c * stride), a1 = __ldg(p + (size_t)(c + kReduceRows) * stride);
      const float2 a2 = __ldg(p + (size_t)(c + 2 * kReduceRows) * stride);
      const float2 a3 = __ldg(p + (size_t)(c + 3 * kReduceRows) * stride);
      sx += a0.x; sy += a0.y; sx += a1.x; sy += a1.y; sx += a2.x; sy += a2.y; sx += a3.x; sy += a3.y;
    }
    for (; c < nC; c += kReduceRows) {
      const float2 a0 = __ldg(p + (size_t)c * stride);
      sx += a0.x; sy += a0.y;
    }
  }
  acc[row][col] = make_float2(sx, sy);
  __syncthreads();
  if (row != 0 || !valid) return;
  for (int r = 1; r < kReduceRows; ++r) {
    sx += acc[r][col].x;
    sy += acc[r][col].y;
  }
  const int l = idx / np2, pos = idx - l * np2;
  const int q = pos_slot(pos, M, G);
  if (q >= N / 2) return;
  const int sh = geo[2 * l], ln = geo[2 * l + 1];
  const bool active = q >= sh / 2 && q < sh / 2 + ln;
  float* o = dp + (size_t)l * ldp + (size_t)q * n_p;
  if (!active) {
    if (!accumulate) {
      o[0] = 0.f;
      if (n_p > 1) o[1] = 0.f;
    }
    return;
  }
  if (accumulate) {
    o[0] += sx;
    if (n_p > 1) o[1] += sy;
  } else {
    o[0] = sx;
    if (n_p > 1) o[1] = sy;
  }
}

// Stored-activation back-propagation (lossy crossings): dT[l][q][k] (= or +=) the conjugate of the sum
// over the nC per-CTA raw partials [c][l][k][pos], k = (00, 01, 10, 11).  The conjugate turns the kernel's
// sum of conj(g_i) x_j into g_i conj(x_j) = 2 dJ/dT_ij*, the gradient convention of complex tensors in
// PyTorch.  Inactive slots give 0.  A CTA's partials are one contiguous block of nl*4*np2 float2, so a
// block of 32 columns x 8 rows owns 32 consecutive entries: its rows sum the CTAs c = row, row + 8, ...
// (several loads in flight), then the 8 row sums are combined in a fixed order (bit-stable).
__global__ void __launch_bounds__(kReduceCols * kReduceRows)
raw_reduce_kernel(const float2* __restrict__ partial, int nC, int L, int np2, int M, int G, int N, float2* dT,
                  int accumulate, const int* geo) {
  __shared__ float2 acc[kReduceRows][kReduceCols];
  const int col = threadIdx.x % kReduceCols, row = threadIdx.x / kReduceCols;
  const size_t n = (size_t)L * 4 * np2;
  const size_t idx = (size_t)blockIdx.x * kReduceCols + col;
  const bool valid = idx < n;
  float2 s = make_float2(0.f, 0.f);
  if (valid) {
    const float2* p = partial + idx;
    int c = row;
    for (; c + 3 * kReduceRows < nC; c += 4 * kReduceRows) {
      const float2 a0 = __ldg(p + (size_t)c * n), a1 = __ldg(p + (size_t)(c + kReduceRows) * n);
      const float2 a2 = __ldg(p + (size_t)(c + 2 * kReduceRows) * n), a3 = __ldg(p + (size_t)(c + 3 * kReduceRows) * n);
      s = cadd(s, a0); s = cadd(s, a1); s = cadd(s, a2); s = cadd(s, a3);
    }
    for (; c < nC; c += kReduceRows) s = cadd(s, __ldg(p + (size_t)c * n));
  }
  acc[row][col] = s;
  __syncthreads();
  if (row != 0 || !valid) return;
  for (int r = 1; r < kReduceRows; ++r) s = cadd(s, acc[r][col]);
  const int l = (int)(idx / (4 * (size_t)np2));
  const int rem = (int)(idx - (size_t)l * 4 * np2);
  const int k = rem / np2, pos = rem - k * np2;
  const int q = pos_slot(pos, M, G);
  if (q >= N / 2) return;
  const int sh = geo[2 * l], ln = geo[2 * l + 1];
  const bool active = q >= sh / 2 && q < sh / 2 + ln;
  float2* o = dT + ((size_t)l * (N / 2) + q) * 4 + k;
  const float2 c = active ? make_float2(s.x, -s.y) : make_float2(0.f, 0.f);
  *o = accumulate ? cadd(*o, c) : c;
}

}  // namespace mg
