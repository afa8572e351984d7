// Nearest-neighbour instantiations for small meshes and batches (Clements or Reck, complex, a vector over the 32
// lanes of a warp): forward with 2 or 4 modes and 1 to 4 vectors per lane, and back-propagation with 4 modes and 2
// vectors per lane (the tile the tuner picks at N=128, B=128).  A call on a small mesh is latency-bound - at
// N=64, B=1024 the default 2-mode x 4-vector forward tile gives 256 warps for 608 schedulers, one warp per busy
// scheduler - so fewer vectors per lane put more warps on more schedulers.
#include "mg_launch.h"

namespace mg {

namespace {
// (op, gr, M, V)
constexpr int kSmall[][4] = {{OP_FWD, 0, 2, 1}, {OP_FWD, 0, 2, 2}, {OP_FWD, 0, 2, 4}, {OP_FWD, 0, 4, 1},
                             {OP_FWD, 0, 4, 2}, {OP_BWD, 1, 4, 1}, {OP_BWD, 1, 4, 2}};
}  // namespace

bool nn_small_instantiated(int op, bool real, int M, int V, int gr, bool full) {
  if (real || !full) return false;
  for (const auto& k : kSmall)
    if (k[0] == op && k[1] == gr && k[2] == M && k[3] == V) return true;
  return false;
}

cudaError_t launch_prop_nn_small(int op, int M, int V, const LaunchCfg& lc, const PropArgs& a) {
  switch (op * 10000 + M * 10 + V) {
    case 21: return launch_one<OP_FWD, 2, 1, false, 32, 0, false, true>(lc, a);
    case 22: return launch_one<OP_FWD, 2, 2, false, 32, 0, false, true>(lc, a);
    case 24: return launch_one<OP_FWD, 2, 4, false, 32, 0, false, true>(lc, a);
    case 41: return launch_one<OP_FWD, 4, 1, false, 32, 0, false, true>(lc, a);
    case 42: return launch_one<OP_FWD, 4, 2, false, 32, 0, false, true>(lc, a);
    case OP_BWD * 10000 + 41: return launch_one<OP_BWD, 4, 1, false, 32, 1, false, true>(lc, a);
    case OP_BWD * 10000 + 42: return launch_one<OP_BWD, 4, 2, false, 32, 1, false, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
