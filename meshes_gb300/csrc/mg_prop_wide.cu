// Instantiations for wide nearest-neighbour meshes, 512 < N <= 640 (the reference's limit,
// gpu/mesh.py:83): 20 modes in each of the 32 lanes of a warp (a power-of-two split would pad N=640 to
// 1024 modes), layer kinds 0 and odd-shift only (the butterfly strides need a power-of-two split).  V
// keeps the fields in registers without spills: 2 vectors per lane forward, 1 (complex) or 2 (real) in
// back-propagation.
#include "mg_launch.h"

namespace mg {

bool wide_instantiated(int op, bool real, int V, int gr) {
  if (op == OP_FWD) return V == 2 && gr == 0;
  if (op == OP_FWDDIFF) return V == 1 && gr == 0;
  if (op == OP_BWD) return real ? (V == 2 && gr == 2) : (V == 1 && (gr == 0 || gr == 1));
  return false;
}

cudaError_t launch_prop_wide(int op, bool real, int V, int gr, const LaunchCfg& lc, const PropArgs& a) {
  if (!wide_instantiated(op, real, V, gr)) return cudaErrorInvalidConfiguration;
  constexpr int M = kWideM;
  if (op == OP_FWD)
    return real ? launch_one<OP_FWD, M, 2, true, 32, 0, false, true>(lc, a)
                : launch_one<OP_FWD, M, 2, false, 32, 0, false, true>(lc, a);
  if (op == OP_FWDDIFF)
    return real ? launch_one<OP_FWDDIFF, M, 1, true, 32, 0, false, true>(lc, a)
                : launch_one<OP_FWDDIFF, M, 1, false, 32, 0, false, true>(lc, a);
  if (real) return launch_one<OP_BWD, M, 2, true, 32, 2, false, true>(lc, a);
  return gr == 1 ? launch_one<OP_BWD, M, 1, false, 32, 1, false, true>(lc, a)
                 : launch_one<OP_BWD, M, 1, false, 32, 0, false, true>(lc, a);
}

}  // namespace mg
