// Nearest-neighbour instantiations of the forward-mode derivative kernel (fwddiff: (y, dy) of (x, dx) along a
// phase direction) for the full-warp tiles of Clements and Reck meshes: layer kinds 0 and odd-shift only, so
// the strided and butterfly bodies and their registers stay out of the kernel.
#include "mg_launch.h"

namespace mg {

namespace {
constexpr int kFwddiff[][3] = {{0, 8, 4}, {0, 8, 2}, {1, 8, 4}};   // (real, M, V)
}  // namespace

bool nn_fwddiff_instantiated(int op, bool real, int M, int V, int gr, bool full) {
  if (op != OP_FWDDIFF || gr != 0 || !full) return false;
  for (const auto& k : kFwddiff)
    if (k[0] == (real ? 1 : 0) && k[1] == M && k[2] == V) return true;
  return false;
}

cudaError_t launch_prop_nn_fwddiff(bool real, int M, int V, const LaunchCfg& lc, const PropArgs& a) {
  switch ((real ? 1000 : 0) + M * 10 + V) {
    case 84: return launch_one<OP_FWDDIFF, 8, 4, false, 32, 0, false, true>(lc, a);
    case 82: return launch_one<OP_FWDDIFF, 8, 2, false, 32, 0, false, true>(lc, a);
    case 1084: return launch_one<OP_FWDDIFF, 8, 4, true, 32, 0, false, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

}  // namespace mg
