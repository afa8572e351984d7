// Explicit instantiations of the propagation kernel (generated; keep the (M, V) list in sync with
// mg_inst_table.h).
#include "mg_launch.h"

namespace mg {

cudaError_t launch_bwd_g0_d(bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a) {
  const int key = gr * 10000 + (real ? 1000 : 0) + M * 10 + V;
  switch (key) {
    case 10024: return launch_one<OP_BWD, 2, 4, false, 0, 1>(lc, a);
    case 10042: return launch_one<OP_BWD, 4, 2, false, 0, 1>(lc, a);
    case 10044: return launch_one<OP_BWD, 4, 4, false, 0, 1>(lc, a);
    case 10081: return launch_one<OP_BWD, 8, 1, false, 0, 1>(lc, a);
    case 10082: return launch_one<OP_BWD, 8, 2, false, 0, 1>(lc, a);
    case 10084: return launch_one<OP_BWD, 8, 4, false, 0, 1>(lc, a);
    case 10161: return launch_one<OP_BWD, 16, 1, false, 0, 1>(lc, a);
    case 10162: return launch_one<OP_BWD, 16, 2, false, 0, 1>(lc, a);
    case 21024: return launch_one<OP_BWD, 2, 4, true, 0, 2>(lc, a);
    case 21042: return launch_one<OP_BWD, 4, 2, true, 0, 2>(lc, a);
    case 21044: return launch_one<OP_BWD, 4, 4, true, 0, 2>(lc, a);
    case 21081: return launch_one<OP_BWD, 8, 1, true, 0, 2>(lc, a);
    case 21082: return launch_one<OP_BWD, 8, 2, true, 0, 2>(lc, a);
    case 21084: return launch_one<OP_BWD, 8, 4, true, 0, 2>(lc, a);
    case 21161: return launch_one<OP_BWD, 16, 1, true, 0, 2>(lc, a);
    case 21162: return launch_one<OP_BWD, 16, 2, true, 0, 2>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
