// Warp-pair back-propagation launches (mg_prop_pair.cuh): direct MZI gradients of nearest-neighbour complex
// meshes with an M = 8, G = 32 plan, V vectors per warp pair.
#include "mg_launch.h"
#include "mg_prop_pair.cuh"

namespace mg {

namespace {
constexpr int kPairV[] = {6, 7, 8};

template <int V>
cudaError_t launch_pair_v(const LaunchCfg& lc, const PropArgs& a) {
  static std::atomic<unsigned long long> done{0};
  auto k = prop_pair_kernel<V>;
  cudaError_t e = ensure_smem_attr(k, done);
  if (e != cudaSuccess) return e;
  k<<<lc.grid, lc.block, lc.smem, lc.stream>>>(a);
  return cudaGetLastError();
}
}  // namespace

bool pair_instantiated(int op, bool real, int M, int V, int gr, bool full) {
  if (op != OP_BWD || real || M != 8 || gr != 1 || !full) return false;
  for (int v : kPairV)
    if (v == V) return true;
  return false;
}

cudaError_t launch_prop_pair(int V, const LaunchCfg& lc, const PropArgs& a) {
  switch (V) {
    case 6: return launch_pair_v<6>(lc, a);
    case 7: return launch_pair_v<7>(lc, a);
    case 8: return launch_pair_v<8>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
