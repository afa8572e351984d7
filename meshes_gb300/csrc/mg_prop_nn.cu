// Nearest-neighbour instantiations of the propagation kernel (layer kinds 0 and odd-shift only) for the
// Clements and Reck meshes: the full-warp configurations (uniform and split) and the main runtime lane-group
// ones; the small-mesh forward tiles are in mg_prop_nn_small.cu.  Without the strided and butterfly layer bodies, and with one fused pair order, the
// back-propagation kernel does not spill; measured on GB300 at N=256, L=256, B=4096 it runs 9% faster than
// the general instantiation, with identical results.
#include "mg_launch.h"

namespace mg {

namespace {
// (op, real, M, V, gr, full): the instantiated set (split: forward, full only)
constexpr int kNN[][6] = {{OP_FWD, 0, 8, 4, 0, 1}, {OP_FWD, 0, 16, 2, 0, 1}, {OP_FWD, 1, 8, 4, 0, 1},
                          {OP_BWD, 0, 8, 4, 1, 1}, {OP_BWD, 0, 16, 2, 1, 1}, {OP_BWD, 1, 8, 4, 2, 1},
                          {OP_FWD, 0, 8, 4, 0, 0}, {OP_FWD, 1, 8, 4, 0, 0}, {OP_BWD, 0, 8, 4, 1, 0},
                          {OP_BWD, 1, 8, 4, 2, 0}};
}  // namespace

bool nn_instantiated(int op, bool real, int M, int V, int gr, bool full, bool split) {
  if (split && (op != OP_FWD || !full)) return false;
  if (!split && (nn_small_instantiated(op, real, M, V, gr, full) || nn_fwddiff_instantiated(op, real, M, V, gr, full)))
    return true;
  for (const auto& k : kNN)
    if (k[0] == op && k[1] == (real ? 1 : 0) && k[2] == M && k[3] == V && k[4] == gr && k[5] == (full ? 1 : 0))
      return true;
  return false;
}

cudaError_t launch_prop_nn(int op, bool real, int M, int V, int gr, bool full, bool split, const LaunchCfg& lc,
                           const PropArgs& a) {
  if (!nn_instantiated(op, real, M, V, gr, full, split)) return cudaErrorInvalidConfiguration;
  if (!split && nn_small_instantiated(op, real, M, V, gr, full)) return launch_prop_nn_small(op, M, V, lc, a);
  if (!split && nn_fwddiff_instantiated(op, real, M, V, gr, full)) return launch_prop_nn_fwddiff(real, M, V, lc, a);
  const int key = op * 10000 + (real ? 1000 : 0) + M * 10 + V;
  if (!full) {
    switch (key) {
      case 84: return launch_one<OP_FWD, 8, 4, false, 0, 0, false, true>(lc, a);
      case 1084: return launch_one<OP_FWD, 8, 4, true, 0, 0, false, true>(lc, a);
      case 20084: return launch_one<OP_BWD, 8, 4, false, 0, 1, false, true>(lc, a);
      case 21084: return launch_one<OP_BWD, 8, 4, true, 0, 2, false, true>(lc, a);
      default: return cudaErrorInvalidConfiguration;
    }
  }
  if (split) {
    switch (key) {
      case 84: return launch_split<OP_FWD, 8, 4, false, 32, 0, true>(lc, a);
      case 162: return launch_split<OP_FWD, 16, 2, false, 32, 0, true>(lc, a);
      case 1084: return launch_split<OP_FWD, 8, 4, true, 32, 0, true>(lc, a);
      default: return cudaErrorInvalidConfiguration;
    }
  }
  switch (key) {
    case 84: return launch_one<OP_FWD, 8, 4, false, 32, 0, false, true>(lc, a);
    case 162: return launch_one<OP_FWD, 16, 2, false, 32, 0, false, true>(lc, a);
    case 1084: return launch_one<OP_FWD, 8, 4, true, 32, 0, false, true>(lc, a);
    case 20084: return launch_one<OP_BWD, 8, 4, false, 32, 1, false, true>(lc, a);
    case 20162: return launch_one<OP_BWD, 16, 2, false, 32, 1, false, true>(lc, a);
    case 21084: return launch_one<OP_BWD, 8, 4, true, 32, 2, false, true>(lc, a);
    default: return cudaErrorInvalidConfiguration;
  }
}

bool nn2_instantiated(int op, bool real, int M, int V, int gr) {
  return !real && M == 8 && V == 2 && ((op == OP_FWD && gr == 0) || (op == OP_BWD && gr == 1));
}

cudaError_t launch_prop_nn2(int op, bool real, int M, int V, int gr, const LaunchCfg& lc, const PropArgs& a) {
  if (!nn2_instantiated(op, real, M, V, gr)) return cudaErrorInvalidConfiguration;
  return op == OP_FWD ? launch_one<OP_FWD, 8, 2, false, 32, 0, false, true, 2>(lc, a)
                      : launch_one<OP_BWD, 8, 2, false, 32, 1, false, true, 2>(lc, a);
}

}  // namespace mg
