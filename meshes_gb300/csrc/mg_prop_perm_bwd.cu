// Instantiations of the back-propagation kernel for permuted meshes (PERM = true): runtime lane-group
// size, the default V of each M, gradient mode by crossing (1 mzi, 0 sym and generic, 2 orth).
#include "mg_launch.h"

namespace mg {

cudaError_t launch_perm_bwd(bool real, int M, int gr, const LaunchCfg& lc, const PropArgs& a) {
  const int key = gr * 1000 + (real ? 100 : 0) + M;
  switch (key) {
    case 1002: return launch_one<OP_BWD, 2, 4, false, 0, 1, true>(lc, a);
    case 1004: return launch_one<OP_BWD, 4, 4, false, 0, 1, true>(lc, a);
    case 1008: return launch_one<OP_BWD, 8, 4, false, 0, 1, true>(lc, a);
    case 1016: return launch_one<OP_BWD, 16, 2, false, 0, 1, true>(lc, a);
    case 2: return launch_one<OP_BWD, 2, 4, false, 0, 0, true>(lc, a);
    case 4: return launch_one<OP_BWD, 4, 4, false, 0, 0, true>(lc, a);
    case 8: return launch_one<OP_BWD, 8, 4, false, 0, 0, true>(lc, a);
    case 16: return launch_one<OP_BWD, 16, 2, false, 0, 0, true>(lc, a);
    case 2102: return launch_one<OP_BWD, 2, 4, true, 0, 2, true>(lc, a);
    case 2104: return launch_one<OP_BWD, 4, 4, true, 0, 2, true>(lc, a);
    case 2108: return launch_one<OP_BWD, 8, 4, true, 0, 2, true>(lc, a);
    case 2116: return launch_one<OP_BWD, 16, 2, true, 0, 2, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
