// Dispatch of the propagation launches to their instantiation units.
#include "mg_launch.h"

namespace mg {

cudaError_t launch_fwd_g0(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_fwd_g32(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_fwddiff_g0(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_fwddiff_g32(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_bwd_g0_g(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_bwd_g0_d(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_bwd_g32_g(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_bwd_g32_d(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_fwd_stored(int M, int V, bool full, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_bwd_stored(int M, int V, bool full, const LaunchCfg& lc, const PropArgs& a);

cudaError_t launch_prop(int op, bool real, int M, int V, bool full, int gr, const LaunchCfg& lc, const PropArgs& a) {
  if (gr == 4) {   // stored activations (complex only)
    if (real) return cudaErrorInvalidConfiguration;
    if (op == 0) return launch_fwd_stored(M, V, full, lc, a);
    if (op == 2) return launch_bwd_stored(M, V, full, lc, a);
    return cudaErrorInvalidConfiguration;
  }
  if (op == 0 && full == false) return launch_fwd_g0(real, M, V, gr, lc, a);
  if (op == 0 && full == true) return launch_fwd_g32(real, M, V, gr, lc, a);
  if (op == 1 && full == false) return launch_fwddiff_g0(real, M, V, gr, lc, a);
  if (op == 1 && full == true) return launch_fwddiff_g32(real, M, V, gr, lc, a);
  if (op == 2 && full == false && gr == 0) return launch_bwd_g0_g(real, M, V, gr, lc, a);
  if (op == 2 && full == false && gr != 0) return launch_bwd_g0_d(real, M, V, gr, lc, a);
  if (op == 2 && full == true && gr == 0) return launch_bwd_g32_g(real, M, V, gr, lc, a);
  if (op == 2 && full == true && gr != 0) return launch_bwd_g32_d(real, M, V, gr, lc, a);
  return cudaErrorInvalidConfiguration;
}

}  // namespace mg
