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

cudaError_t launch_perm_fwd(int op, bool real, int M, const LaunchCfg& lc, const PropArgs& a);
cudaError_t launch_perm_bwd(bool real, int M, int gr, const LaunchCfg& lc, const PropArgs& a);

// default V per (op, M = 2, 4, 8, 16), the only V the permuted instantiations take
static int perm_v(int op, int M) {
  static const int v[3][4] = {{8, 8, 4, 2}, {4, 4, 2, 1}, {4, 4, 4, 2}};
  const int i = M == 2 ? 0 : M == 4 ? 1 : M == 8 ? 2 : M == 16 ? 3 : -1;
  return (op < 0 || op > 2 || i < 0) ? -1 : v[op][i];
}

bool perm_instantiated(int op, bool real, int M, int V, int gr) {
  if (perm_v(op, M) != V) return false;
  if (op != OP_BWD) return gr == 0;
  return real ? gr == 2 : (gr == 0 || gr == 1);
}

cudaError_t launch_prop_perm(int op, bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a) {
  if (!perm_instantiated(op, real, M, V, gr)) return cudaErrorInvalidConfiguration;
  return op == OP_BWD ? launch_perm_bwd(real, M, gr, lc, a) : launch_perm_fwd(op, real, M, lc, a);
}

cudaError_t launch_prop(int op, bool real, int M, int V, bool full, int gr, const LaunchCfg& lc, const PropArgs& a) {
  if (a.perm != nullptr) return launch_prop_perm(op, real, M, V, gr, lc, a);
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
