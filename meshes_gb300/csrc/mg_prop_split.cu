// Instantiations of the split propagation launch (two CTA kinds per SM, V and V-1 vectors per lane
// group) for the full-warp configurations where one wave of uniform CTAs leaves SMs idle at the batch
// sizes of training steps.
#include "mg_launch.h"

namespace mg {

bool split_instantiated(int op, bool real, int M, int V, bool full, int gr) {
  if (!full) return false;
  if (op == OP_FWD) return (!real && ((M == 8 && V == 4) || (M == 16 && V == 2))) || (real && M == 8 && V == 4);
  if (op == OP_BWD)
    return (!real && gr == 1 && ((M == 8 && V == 4) || (M == 16 && V == 2))) || (real && gr == 2 && M == 8 && V == 4);
  return false;
}

cudaError_t launch_prop_split(int op, bool real, int M, int V, bool full, int gr, const LaunchCfg& lc,
                              const PropArgs& a) {
  if (!split_instantiated(op, real, M, V, full, gr)) return cudaErrorInvalidConfiguration;
  if (op == OP_FWD) {
    if (real) return launch_split<OP_FWD, 8, 4, true, 32, 0>(lc, a);
    if (M == 8) return launch_split<OP_FWD, 8, 4, false, 32, 0>(lc, a);
    return launch_split<OP_FWD, 16, 2, false, 32, 0>(lc, a);
  }
  if (real) return launch_split<OP_BWD, 8, 4, true, 32, 2>(lc, a);
  if (M == 8) return launch_split<OP_BWD, 8, 4, false, 32, 1>(lc, a);
  return launch_split<OP_BWD, 16, 2, false, 32, 1>(lc, a);
}

}  // namespace mg
