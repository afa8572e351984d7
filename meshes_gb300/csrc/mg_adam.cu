// Adam (Kingma and Ba, "Adam: A Method for Stochastic Optimization", 2015: Algorithm 1 with its bias
// correction) over a float32 parameter tensor in one launch, its step count on the device.
//
// A mesh-training step (coefficient pass, forward, loss, back-propagation, gradient reduction) is a handful of
// launches; an optimizer built from elementwise passes (lerp, mul, addcmul, sqrt, div, ...) adds a dozen more,
// each reading and writing the parameter-sized state, which for small meshes costs as much as the mesh
// kernels themselves.  Here every parameter is read and written once per step.  The step count lives on the
// device, so the update can be recorded in a CUDA graph and replayed.
//
// For t = step + 1, per parameter:  m = m + (1 - b1) (g - m);  v = b2 v + (1 - b2) g^2;
//                                   p = p - lr / (1 - b1^t) * m / (sqrt(v) / sqrt(1 - b2^t) + eps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

// state[0]: steps taken; state[1]: blocks finished in the current launch (zero between launches).  Every
// block reads state[0] before it counts itself finished, and the last block to finish advances it.
// b1, b2 and their complements c1 = 1 - b1, c2 = 1 - b2 are each rounded to float from double on the host (a
// complement formed in float from a float beta would carry the beta's rounding error: 1.3e-5 relative for
// b2 = 0.999).
__global__ void __launch_bounds__(256)
adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, int n,
            float lr, float b1, float c1, float b2, float c2, float eps, int* state) {
  const int t = state[0] + 1;
  const float step_size = lr / (1.f - powf(b1, (float)t));
  const float bc2_sqrt = sqrtf(1.f - powf(b2, (float)t));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i], m0 = m[i];
    const float mi = __fadd_rn(m0, __fmul_rn(c1, __fsub_rn(gi, m0)));
    const float vi = __fadd_rn(__fmul_rn(b2, v[i]), __fmul_rn(__fmul_rn(c2, gi), gi));
    m[i] = mi;
    v[i] = vi;
    p[i] -= step_size * mi / (sqrtf(vi) / bc2_sqrt + eps);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(state + 1, 1) == (int)gridDim.x - 1) {
      state[0] = t;
      state[1] = 0;
    }
  }
}

}  // namespace

extern "C" {

int mg_adam_step(float* p, const float* g, float* m, float* v, int n, double lr, double beta1, double beta2, double eps,
                 int* state, void* stream) {
  if (n < 0) return mg::set_last_error(MG_E_ARG, "mg_adam_step: n=%d", n);
  if (!(lr >= 0.0) || !(beta1 >= 0.0 && beta1 < 1.0) || !(beta2 >= 0.0 && beta2 < 1.0) || !(eps >= 0.0))
    return mg::set_last_error(MG_E_ARG, "mg_adam_step: lr=%g beta1=%g beta2=%g eps=%g", lr, beta1, beta2, eps);
  if (n == 0) return mg::set_last_error(MG_OK, "%s", "");
  if (!p || !g || !m || !v || !state) return mg::set_last_error(MG_E_ARG, "mg_adam_step: NULL argument");
  const int grid = std::min((n + 255) / 256, 152 * 4);
  adam_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(p, g, m, v, n, (float)lr, (float)beta1,
                                                                    (float)(1.0 - beta1), (float)beta2,
                                                                    (float)(1.0 - beta2), (float)eps, state);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return mg::set_last_error(MG_E_CUDA, "adam_kernel launch: %s", cudaGetErrorString(e));
  return mg::set_last_error(MG_OK, "%s", "");
}

}  // extern "C"
