// Explicit instantiations of the propagation kernel (generated; keep the (M, V) list in sync with
// mg_inst_table.h).
#include "mg_launch.h"

namespace mg {

cudaError_t launch_fwddiff_g32(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a) {
  const int key = gr * 10000 + (real ? 1000 : 0) + M * 10 + V;
  switch (key) {
    case 24: return launch_one<OP_FWDDIFF, 2, 4, false, 32, 0>(lc, a);
    case 42: return launch_one<OP_FWDDIFF, 4, 2, false, 32, 0>(lc, a);
    case 44: return launch_one<OP_FWDDIFF, 4, 4, false, 32, 0>(lc, a);
    case 81: return launch_one<OP_FWDDIFF, 8, 1, false, 32, 0>(lc, a);
    case 82: return launch_one<OP_FWDDIFF, 8, 2, false, 32, 0>(lc, a);
    case 84: return launch_one<OP_FWDDIFF, 8, 4, false, 32, 0>(lc, a);
    case 161: return launch_one<OP_FWDDIFF, 16, 1, false, 32, 0>(lc, a);
    case 162: return launch_one<OP_FWDDIFF, 16, 2, false, 32, 0>(lc, a);
    case 1024: return launch_one<OP_FWDDIFF, 2, 4, true, 32, 0>(lc, a);
    case 1042: return launch_one<OP_FWDDIFF, 4, 2, true, 32, 0>(lc, a);
    case 1044: return launch_one<OP_FWDDIFF, 4, 4, true, 32, 0>(lc, a);
    case 1081: return launch_one<OP_FWDDIFF, 8, 1, true, 32, 0>(lc, a);
    case 1082: return launch_one<OP_FWDDIFF, 8, 2, true, 32, 0>(lc, a);
    case 1084: return launch_one<OP_FWDDIFF, 8, 4, true, 32, 0>(lc, a);
    case 1161: return launch_one<OP_FWDDIFF, 16, 1, true, 32, 0>(lc, a);
    case 1162: return launch_one<OP_FWDDIFF, 16, 2, true, 32, 0>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
