// Native autotuner of the propagation kernels' tile configuration (mg_autotune, declared in
// include/meshes_gb300.h).  It drives the library's own public entry points - mg_workspace_bytes,
// mg_build_tiles, mg_propagate - on the caller's mesh parameters and times each candidate with CUDA events
// on the caller's stream, flushing the L2 before every timed launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

bool same(const mg_config& a, const mg_config& b) {
  return a.M == b.M && a.V == b.V && a.W == b.W && a.CL == b.CL && a.S == b.S && a.split == b.split;
}

}  // namespace

extern "C" int mg_autotune(int op, int N, int L, int B, int crossing, int geometry, const int* lens,
                           const int* shifts, const int* strides, const float* p, int ldp, const float* s, int lds,
                           int reps, int record, mg_config* best, float* best_ms, mg_config* tried, float* tried_ms,
                           int max_tried, int* n_tried, void* stream) {
  if (op < 0 || op > 2) return mg::set_last_error(MG_E_ARG, "mg_autotune: op %d not in {0, 1, 2}", op);
  if (crossing == MG_GENERIC) return mg::set_last_error(MG_E_ARG, "mg_autotune: generic crossings need Tgen");
  if (reps < 1 || !best || B < 1 || L < 1 || !p)
    return mg::set_last_error(MG_E_ARG, "mg_autotune: need reps >= 1, B >= 1, L >= 1, p and best");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const bool real = crossing == MG_ORTH;
  const size_t el = real ? 4 : 8;
  const int n_p = real ? 1 : 2;

  // stage 1: register blocking and CTA width; pipeline and schedule from the heuristic, uniform CTAs
  int Np = 1;
  while (Np < N) Np <<= 1;
  std::vector<mg_config> cands;
  static const int vs[3][4] = {{1, 2, 4, 8}, {1, 2, 4, 0}, {1, 2, 4, 0}};
  for (int M : {2, 4, 8, 16}) {
    if (N > 512 || M > Np || Np / M > 32) continue;
    for (int V : vs[op]) {
      if (!V) continue;
      for (int W : {1, 2, 4, 8}) cands.push_back(mg_config{M, V, W, 0, 0, 2});
    }
  }
  if (N > 512)   // wide meshes: 20 modes per lane
    for (int V : {1, 2})
      for (int W : {2, 4, 8}) cands.push_back(mg_config{mg::kWideM, V, W, 0, 0, 2});

  // scratch (stream-ordered, freed before returning): fields x, dx / g, y, dy / g_in, dJ/dp, an L2 flush
  // buffer and the workspace of the largest candidate so far
  const size_t field = (size_t)B * N * el;
  const size_t kFlush = 256u << 20;   // larger than the 129 MB L2
  void* f[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  void* flush = nullptr;
  void* ws = nullptr;
  auto release = [&]() {
    for (void*& q : f)
      if (q) cudaFreeAsync(q, st), q = nullptr;
    if (flush) cudaFreeAsync(flush, st), flush = nullptr;
    if (ws) cudaFreeAsync(ws, st), ws = nullptr;
    return cudaStreamSynchronize(st);
  };
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaMallocAsync(&f[i], field, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&f[4], sizeof(float) * (size_t)L * (N / 2) * n_p, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&flush, kFlush, st);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaMemsetAsync(f[i], 0, field, st);
  if (e != cudaSuccess) {
    release();
    return mg::set_last_error(MG_E_CUDA, "mg_autotune: scratch: %s", cudaGetErrorString(e));
  }
  size_t ws_bytes = 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);

  std::vector<mg_config> done;
  std::vector<float> done_ms;
  auto measure = [&](const mg_config& c) {
    for (const mg_config& d : done)
      if (same(d, c)) return;
    const size_t nb = mg_workspace_bytes(op, N, L, B, crossing, geometry, &c);
    if (nb == 0) return;                       // not a valid configuration of this shape
    if (nb > ws_bytes) {
      if (ws) cudaFreeAsync(ws, st);
      ws = nullptr;
      ws_bytes = 0;
      if (cudaMallocAsync(&ws, nb, st) != cudaSuccess) {
        ws = nullptr;
        return;
      }
      ws_bytes = nb;
    }
    if (mg_workspace_init(ws, ws_bytes, stream) != MG_OK) return;
    if (mg_build_tiles(op, N, L, geometry, lens, shifts, strides, crossing, p, ldp, s, lds,
                       op == MG_OP_FWDDIFF ? p : nullptr, nullptr, nullptr, B, &c, ws, ws_bytes, stream) != MG_OK)
      return;
    auto run = [&]() {
      if (op == MG_OP_FWD)
        return mg_propagate(op, N, L, B, crossing, geometry, f[0], nullptr, f[2], nullptr, N, nullptr, 0, 0, &c, ws,
                            ws_bytes, stream);
      if (op == MG_OP_FWDDIFF)
        return mg_propagate(op, N, L, B, crossing, geometry, f[0], f[1], f[2], f[3], N, nullptr, 0, 0, &c, ws,
                            ws_bytes, stream);
      return mg_propagate(op, N, L, B, crossing, geometry, f[0], f[1], nullptr, f[3], N, static_cast<float*>(f[4]),
                          N / 2 * n_p, 0, &c, ws, ws_bytes, stream);
    };
    for (int w = 0; w < 2; ++w)
      if (run() != MG_OK) return;
    std::vector<float> ts;
    for (int r = 0; r < reps; ++r) {
      cudaMemsetAsync(flush, r & 0xff, kFlush, st);
      cudaEventRecord(e0, st);
      if (run() != MG_OK) return;
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess) return;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      ts.push_back(ms);
    }
    if (mg_read_status(ws, 1, stream) != 0) return;   // a timed-out or malformed launch does not count
    std::sort(ts.begin(), ts.end());
    done.push_back(c);
    done_ms.push_back(ts[ts.size() / 2]);
  };

  for (const mg_config& c : cands) measure(c);
  int rc = MG_OK;
  if (done.empty()) {
    rc = mg::set_last_error(MG_E_CONFIG, "mg_autotune: no configuration of this shape ran");
  } else {
    // stage 2 around the winner: layers per stage and stages; forward also the split launch
    const size_t w1 = std::min_element(done_ms.begin(), done_ms.end()) - done_ms.begin();
    const mg_config c1 = done[w1];
    for (int CL : {0, 4, 8, 16})
      for (int S : {2, 3}) measure(mg_config{c1.M, c1.V, c1.W, CL, S, 2});
    // every layer resident at once, in 1, 2 or 4 stages (no stage reused; shapes whose tiles do not fit are
    // not valid configurations and are skipped)
    for (int S : {1, 2, 4}) measure(mg_config{c1.M, c1.V, c1.W, (L + S - 1) / S, S, 2});
    if (op == MG_OP_FWD && c1.V >= 2)
      for (int CL : {0, 4, 6, 8, 12})
        for (int S : {2, 3}) measure(mg_config{c1.M, c1.V, 4, CL, S, 1});
    const size_t w = std::min_element(done_ms.begin(), done_ms.end()) - done_ms.begin();
    *best = done[w];
    if (best_ms) *best_ms = done_ms[w];
    const int n = (int)done.size();
    if (n_tried) *n_tried = n;
    for (int i = 0; i < std::min(n, max_tried); ++i) {
      if (tried) tried[i] = done[i];
      if (tried_ms) tried_ms[i] = done_ms[i];
    }
    if (record) rc = mg_set_tuned(op, crossing, geometry, N, B, B, best);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const cudaError_t es = release();
  if (rc == MG_OK && es != cudaSuccess)
    rc = mg::set_last_error(MG_E_CUDA, "mg_autotune: %s", cudaGetErrorString(es));
  return rc;
}
