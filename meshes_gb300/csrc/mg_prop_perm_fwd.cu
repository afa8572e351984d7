// Instantiations of the propagation kernel for permuted meshes (PERM = true): forward and forward-mode
// derivative, runtime lane-group size, the default V of each M (the list in perm_instantiated()).
#include "mg_launch.h"

namespace mg {

cudaError_t launch_perm_fwd(int op, bool real, int M, const LaunchCfg& lc, const PropArgs& a) {
  const int key = op * 1000 + (real ? 100 : 0) + M;
  switch (key) {
    case 2: return launch_one<OP_FWD, 2, 8, false, 0, 0, true>(lc, a);
    case 4: return launch_one<OP_FWD, 4, 8, false, 0, 0, true>(lc, a);
    case 8: return launch_one<OP_FWD, 8, 4, false, 0, 0, true>(lc, a);
    case 16: return launch_one<OP_FWD, 16, 2, false, 0, 0, true>(lc, a);
    case 102: return launch_one<OP_FWD, 2, 8, true, 0, 0, true>(lc, a);
    case 104: return launch_one<OP_FWD, 4, 8, true, 0, 0, true>(lc, a);
    case 108: return launch_one<OP_FWD, 8, 4, true, 0, 0, true>(lc, a);
    case 116: return launch_one<OP_FWD, 16, 2, true, 0, 0, true>(lc, a);
    case 1002: return launch_one<OP_FWDDIFF, 2, 4, false, 0, 0, true>(lc, a);
    case 1004: return launch_one<OP_FWDDIFF, 4, 4, false, 0, 0, true>(lc, a);
    case 1008: return launch_one<OP_FWDDIFF, 8, 2, false, 0, 0, true>(lc, a);
    case 1016: return launch_one<OP_FWDDIFF, 16, 1, false, 0, 0, true>(lc, a);
    case 1102: return launch_one<OP_FWDDIFF, 2, 4, true, 0, 0, true>(lc, a);
    case 1104: return launch_one<OP_FWDDIFF, 4, 4, true, 0, 0, true>(lc, a);
    case 1108: return launch_one<OP_FWDDIFF, 8, 2, true, 0, 0, true>(lc, a);
    case 1116: return launch_one<OP_FWDDIFF, 16, 1, true, 0, 0, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
