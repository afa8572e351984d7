// Nearest-neighbour forward instantiations for small meshes and batches (Clements or Reck, complex, a vector over
// the 32 lanes of a warp): 2 or 4 modes and 1 to 4 vectors per lane.  A plain forward call of a small mesh is
// latency-bound - at N=64, B=1024 the default 2-mode x 4-vector tile gives 256 warps for 608 schedulers, one
// warp per busy scheduler - so fewer vectors per lane put more warps on more schedulers.
#include "mg_launch.h"

namespace mg {

namespace {
constexpr int kSmall[][2] = {{2, 1}, {2, 2}, {2, 4}, {4, 1}, {4, 2}};
}  // namespace

bool nn_small_instantiated(int op, bool real, int M, int V, int gr, bool full) {
  if (op != OP_FWD || real || gr != 0 || !full) return false;
  for (const auto& k : kSmall)
    if (k[0] == M && k[1] == V) return true;
  return false;
}

cudaError_t launch_prop_nn_small(int M, int V, const LaunchCfg& lc, const PropArgs& a) {
  switch (M * 10 + V) {
    case 21: return launch_one<OP_FWD, 2, 1, false, 32, 0, false, true>(lc, a);
    case 22: return launch_one<OP_FWD, 2, 2, false, 32, 0, false, true>(lc, a);
    case 24: return launch_one<OP_FWD, 2, 4, false, 32, 0, false, true>(lc, a);
    case 41: return launch_one<OP_FWD, 4, 1, false, 32, 0, false, true>(lc, a);
    case 42: return launch_one<OP_FWD, 4, 2, false, 32, 0, false, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
