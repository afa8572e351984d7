// Transfer matrices of the lossy generic MZI (reference crossing.py:444-488) and their vector-Jacobian
// product with respect to (theta, phi), one thread per slot, double precision, for the checkpointed
// lossy adjoint: replaces the dozens of elementwise tensor operations (and their autograd) that the
// same formula costs in PyTorch.
//
//   T = S(beta) D2 S(alpha) D1,  S(a) = [[cos(pi/4 + a), i sin(pi/4 + a)], [i sin(pi/4 + a), cos(pi/4 + a)]],
//   D1 = diag(exp(i(phi + e11 + x11) + g11/2), exp(i(e21 + x21) + g21/2)),
//   D2 = diag(exp(i(theta + e12 + x12) + g12/2), exp(i(e22 + x22) + g22/2)),
//   s = (alpha, beta, e11, e21, e12, e22, x11, x21, x12, x22, g11, g21, g12, g22) per slot.
// Derivatives: theta enters D2[0] and phi D1[0] through exp(i .), so with N = D2 S(alpha) D1,
//   dT/dphi = T diag(i, 0),
//   dT/dtheta = S(beta) diag(i, 0) N   (columns: d t0j = i cb n0j, d t1j = -sb n0j).
// With G = 2 dJ/dT* (PyTorch's complex gradient), dJ/dp = Re sum_ij conj(G_ij) dT_ij/dp.
#include <cuda_runtime.h>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

using mg::Z;
using mg::zmul;
using mg::zadd;

struct GenericT {
  Z t[4];     // t00, t01, t10, t11
  Z n0[2];    // first row of N = D2 S(alpha) D1
  double cb, sb;
};

__device__ __forceinline__ Z ep(double phase, double gain) {     // exp(i phase + gain / 2)
  double s, c;
  mg::sincos_d(phase, &s, &c);
  const double r = exp(0.5 * gain);
  return Z{r * c, r * s};
}

__device__ __forceinline__ GenericT generic_T(const double* p, const double* s) {
  double sv[14];
  for (int k = 0; k < 14; ++k) sv[k] = s ? s[k] : 0.0;
  const Z d1a = ep(p[1] + sv[2] + sv[6], sv[10]), d1b = ep(sv[3] + sv[7], sv[11]);
  const Z d2a = ep(p[0] + sv[4] + sv[8], sv[12]), d2b = ep(sv[5] + sv[9], sv[13]);
  double sa, ca, sbv, cbv;
  mg::sincos_d(0.78539816339744830962 + sv[0], &sa, &ca);
  mg::sincos_d(0.78539816339744830962 + sv[1], &sbv, &cbv);
  const Z isa = {0.0, sa};
  const Z n00 = zmul(d2a, mg::zscale(ca, d1a)), n01 = zmul(d2a, zmul(isa, d1b));
  const Z n10 = zmul(d2b, zmul(isa, d1a)), n11 = zmul(d2b, mg::zscale(ca, d1b));
  const Z isb = {0.0, sbv};
  GenericT g;
  g.t[0] = zadd(mg::zscale(cbv, n00), zmul(isb, n10));
  g.t[1] = zadd(mg::zscale(cbv, n01), zmul(isb, n11));
  g.t[2] = zadd(zmul(isb, n00), mg::zscale(cbv, n10));
  g.t[3] = zadd(zmul(isb, n01), mg::zscale(cbv, n11));
  g.n0[0] = n00;
  g.n0[1] = n01;
  g.cb = cbv;
  g.sb = sbv;
  return g;
}

__global__ void generic_T_kernel(int n, const double* __restrict__ p, const double* __restrict__ s, float2* T) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const GenericT g = generic_T(p + 2 * (size_t)q, s ? s + 14 * (size_t)q : nullptr);
  for (int k = 0; k < 4; ++k) T[4 * (size_t)q + k] = mg::zf(g.t[k]);
}

// Re(conj(G) * D) summed over the four entries
__device__ __forceinline__ double re_conj_dot(const float2* G, const Z* D) {
  double acc = 0.0;
  for (int k = 0; k < 4; ++k) acc += (double)G[k].x * D[k].x + (double)G[k].y * D[k].y;
  return acc;
}

__global__ void generic_T_vjp_kernel(int n, const double* __restrict__ p, const double* __restrict__ s,
                                     const float2* __restrict__ G, double* dp) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const GenericT g = generic_T(p + 2 * (size_t)q, s ? s + 14 * (size_t)q : nullptr);
  const Z i_n00 = {-g.n0[0].y, g.n0[0].x}, i_n01 = {-g.n0[1].y, g.n0[1].x};
  const Z dth[4] = {mg::zscale(g.cb, i_n00), mg::zscale(g.cb, i_n01), mg::zscale(-g.sb, g.n0[0]),
                    mg::zscale(-g.sb, g.n0[1])};
  const Z dph[4] = {{-g.t[0].y, g.t[0].x}, {0.0, 0.0}, {-g.t[2].y, g.t[2].x}, {0.0, 0.0}};
  const float2* Gq = G + 4 * (size_t)q;
  dp[2 * (size_t)q] = re_conj_dot(Gq, dth);
  dp[2 * (size_t)q + 1] = re_conj_dot(Gq, dph);
}

}  // namespace

extern "C" {

int mg_generic_mzi_T(int n, const double* p, const double* s, void* T, void* stream) {
  if (n < 0 || (n > 0 && (!p || !T))) return mg::set_last_error(MG_E_ARG, "mg_generic_mzi_T: bad arguments");
  if (n == 0) return MG_OK;
  generic_T_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(n, p, s, static_cast<float2*>(T));
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : mg::set_last_error(MG_E_CUDA, "generic_T_kernel: %s", cudaGetErrorString(e));
}

int mg_generic_mzi_T_vjp(int n, const double* p, const double* s, const void* gT, double* dp, void* stream) {
  if (n < 0 || (n > 0 && (!p || !gT || !dp))) return mg::set_last_error(MG_E_ARG, "mg_generic_mzi_T_vjp: bad arguments");
  if (n == 0) return MG_OK;
  generic_T_vjp_kernel<<<(n + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
      n, p, s, static_cast<const float2*>(gT), dp);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : mg::set_last_error(MG_E_CUDA, "generic_T_vjp_kernel: %s", cudaGetErrorString(e));
}

}  // extern "C"
