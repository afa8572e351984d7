// Instantiations of the propagation kernel in its stored-activation mode (GR 4, complex crossings):
// the forward pass writes every layer's input, back-propagation reads them back (lossy meshes).
// Keep the (M, V) list in sync with instantiated_stored() in mg_capi.cu.
#include "mg_launch.h"

namespace mg {

cudaError_t launch_bwd_stored(int M, int V, bool full, const LaunchCfg& lc, const PropArgs& a) {
  const int key = (full ? 1000 : 0) + M * 10 + V;
  switch (key) {
    case 24: return launch_one<OP_BWD, 2, 4, false, 0, 4>(lc, a);
    case 44: return launch_one<OP_BWD, 4, 4, false, 0, 4>(lc, a);
    case 84: return launch_one<OP_BWD, 8, 4, false, 0, 4>(lc, a);
    case 1084: return launch_one<OP_BWD, 8, 4, false, 32, 4>(lc, a);
    case 1162: return launch_one<OP_BWD, 16, 2, false, 32, 4>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
