// C ABI of libmeshes_gb300.so (declared in include/meshes_gb300.h).
//
// Each reference-shaped entry point checks its arguments on the host, derives a launch plan (tile
// configuration, shared-memory footprint, workspace layout), then enqueues on the caller's stream:
//   coef_kernel      p, s[, dp] -> coefficient tiles + layer kinds (+ dT/dp tiles for back-prop)
//   prop_kernel      the propagation itself
//   dp_reduce_kernel (back-prop only) deterministic sum of the per-CTA gradient partials
// Nothing is allocated: all scratch lives in the caller's workspace.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/meshes_gb300.h"
#include "mg_coeffs.cuh"
#include "mg_reduce.cuh"
#include "mg_inst_table.h"
#include "mg_launch.h"

using namespace mg;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  return fail(MG_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int pow2ceil(int x) {
  int p = 1;
  while (p < x) p <<= 1;
  return p;
}
int ilog2(int x) {
  int l = 0;
  while ((1 << l) < x) ++l;
  return l;
}
size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

struct DevInfo {
  int sms = 0;
  int smem_optin = 0;
  int smem_per_sm = 0;
};
DevInfo dev_info() {
  static std::mutex mu;
  static DevInfo cache[64];
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  DevInfo& d = cache[dev & 63];
  if (d.sms == 0) {
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&d.smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (d.sms <= 0) d.sms = 152;
    if (d.smem_optin <= 0) d.smem_optin = 227 * 1024;
    if (d.smem_per_sm <= 0) d.smem_per_sm = 228 * 1024;
  }
  return d;
}

bool instantiated(int op, int M, int V) {
  for (int i = 0; i < kInstCount[op]; ++i)
    if (kInst[op][i][0] == M && kInst[op][i][1] == V) return true;
  return false;
}

// Tuning table: configurations measured by the autotuner, used when a call passes no config.
struct Tuned {
  int op, crossing, geometry, N, Blo, Bhi;
  mg_config cfg;
};
std::mutex g_tuned_mu;
std::vector<Tuned> g_tuned;

bool lookup_tuned(int op, int crossing, int geometry, int N, int B, mg_config* out) {
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  for (const Tuned& t : g_tuned)
    if (t.op == op && t.crossing == crossing && t.geometry == geometry && t.N == N && B >= t.Blo && B <= t.Bhi) {
      *out = t.cfg;
      return true;
    }
  return false;
}

struct Plan {
  int op, N, L, B, crossing, geometry;
  bool real;
  int gr;
  int M, V, W, CL, S, G, logG, R, np2, grid;
  bool split;   // two CTA kinds per SM (V and V-1 vectors per lane group), CTAs [0, nA) the first kind
  int nA;
  bool pair;    // warp-pair launch: a vector over two warps (4 modes per lane), V vectors per pair
  bool occ2;    // kernel compiled for two resident CTAs per SM; shared memory sized for two
  unsigned lb, dlb;
  size_t smem;
  size_t off_kinds, off_tiles, off_dtiles, off_partial, total;
  bool perm;        // MG_GEO_PERM: permutation tables at off_perm, gather scratch after the smem layout
  size_t off_perm;
};

// Permutation tables in the workspace: forward rows [L+1][N], back-propagation rows [L+1][N], forward
// flags [L+1], back-propagation flags [L+1] (int32).
size_t perm_table_bytes(int N, int L) { return 4 * (2 * (size_t)(L + 1) * N + 2 * (size_t)(L + 1)); }

// Shared memory of a launch of plan P over L layers, with the permutation scratch when P has one.
size_t launch_smem(const Plan& P, int op, int gslot, int L) {
  const size_t b = prop_smem_bytes(op, gslot, P.M, P.G, P.W, P.CL, P.S, P.lb, P.dlb, L);
  return P.perm ? perm_scratch_offset(b) + perm_scratch_bytes(P.W, P.M, P.real) : b;
}

// (M, V) instantiated for the stored-activation kernels (GR 4), by op (FWD writes, BWD reads)
bool instantiated_stored(int op, int M, int V) {
  static const int fwd[][2] = {{2, 8}, {4, 8}, {8, 4}, {16, 2}};
  static const int bwd[][2] = {{2, 4}, {4, 4}, {8, 4}, {16, 2}};
  for (int i = 0; i < 4; ++i) {
    const int* t = (op == OP_FWD) ? fwd[i] : bwd[i];
    if (t[0] == M && t[1] == V) return true;
  }
  return false;
}
int stored_default_v(int op, int M) { return op == OP_FWD ? (M <= 4 ? 8 : (M == 8 ? 4 : 2)) : (M <= 8 ? 4 : 2); }

// op MG_OP_BWD_STORED plans the back-propagation kernel in its stored-activation mode (GR 4): T tiles
// only, 32-byte dJ/dT staging per slot, raw partials of 4 complex per slot.
int make_plan(int op, int N, int L, int B, int crossing, int geometry, const mg_config* cfg, Plan* P) {
  const bool stored = op == MG_OP_BWD_STORED;
  if (stored) {
    if (crossing == CR_ORTH) return fail(MG_E_ARG, "stored-activation back-propagation needs a complex crossing");
    op = OP_BWD;
  } else if (op < 0 || op > 2) {
    return fail(MG_E_ARG, "op %d not in {0,1,2,4}", op);
  }
  if (crossing < 0 || crossing > 3) return fail(MG_E_ARG, "crossing %d not in {0,1,2,3}", crossing);
  const bool perm = geometry >= 0 && (geometry & MG_GEO_PERM) != 0;
  if (perm) geometry &= ~MG_GEO_PERM;
  if (geometry < 0 || geometry > 1) return fail(MG_E_ARG, "geometry %d not in {0,1} (| MG_GEO_PERM)", geometry);
  if (N < 2 || N % 2) return fail(MG_E_ARG, "N=%d must be even and >= 2 (reference gpu/mesh.py:67)", N);
  // wide meshes (512 < N <= 640, the reference's limit, gpu/mesh.py:83): 20 modes in each of 32 lanes,
  // nearest-neighbour geometry only (kWideM)
  if (N > 640) return fail(MG_E_ARG, "N=%d above the supported maximum 640", N);
  if (N > 512 && geometry != GEO_NN) return fail(MG_E_ARG, "N=%d > 512 needs nearest-neighbour geometry", N);
  if (L < 0 || B < 0) return fail(MG_E_ARG, "L=%d, B=%d must be non-negative", L, B);
  // the permutation flags travel in the shared-memory copy of the layer kinds
  if (perm && L > kMaxSmemKinds) return fail(MG_E_ARG, "permuted meshes take at most %d layers", kMaxSmemKinds);
  const DevInfo di = dev_info();
  mg_config tuned;
  // tuned entries were measured without the permutation scratch: permuted meshes take the defaults
  if (!cfg && !perm && lookup_tuned(op, crossing, geometry, N, B, &tuned)) cfg = &tuned;
  Plan& p = *P;
  p.op = op; p.N = N; p.L = L; p.B = B; p.crossing = crossing; p.geometry = geometry;
  p.perm = perm;
  p.real = crossing == CR_ORTH;
  p.gr = stored ? 4 : (op != OP_BWD) ? 0 : (crossing == CR_MZI ? 1 : (crossing == CR_ORTH ? 2 : 0));
  const bool wide = N > 512;
  const int Np = wide ? 32 * kWideM : pow2ceil(N);
  int M = (cfg && cfg->M) ? cfg->M : (wide ? kWideM : std::max(std::min(8, Np), Np / 32));
  if (wide ? M != kWideM : (M < 2 || M > 16 || (M & (M - 1))))
    return fail(MG_E_CONFIG, "modes per lane M=%d not in %s", M, wide ? "{20} for N > 512" : "{2,4,8,16}");
  if (M > Np) M = Np;
  const int G = Np / M;
  if (G > 32) return fail(MG_E_CONFIG, "N=%d needs more than 32 lanes at M=%d", N, M);
  int V = (cfg && cfg->V) ? cfg->V : 0;
  if (!V) {
    static const int vd[3][5] = {{8, 8, 4, 2, 0}, {4, 4, 2, 1, 0}, {4, 4, 4, 2, 0}};   // by ilog2(M)-1
    static const int vw[3] = {2, 1, 1};                                                // M = kWideM
    V = wide ? ((op == OP_BWD && p.real) ? 2 : vw[op]) : stored ? stored_default_v(OP_BWD, M) : vd[op][ilog2(M) - 1];
  }
  if (perm && stored) return fail(MG_E_ARG, "stored-activation back-propagation takes no permutations");
  // warp-pair launch (split 3): back-propagation of a nearest-neighbour complex mesh with a full-warp M = 8 plan
  const int split_mode = cfg ? cfg->split : 0;
  p.pair = split_mode == 3;
  p.occ2 = split_mode == 4;
  if (p.occ2 && (stored || perm || geometry != GEO_NN || G != 32 || !nn2_instantiated(op, crossing == CR_ORTH, M, V, p.gr)))
    return fail(MG_E_CONFIG, "no two-CTA-per-SM kernel for op=%d crossing=%d geometry=%d M=%d G=%d V=%d", op, crossing,
                geometry, M, G, V);
  if (p.pair) {
    if (!(cfg && cfg->V)) V = 7;
    if (stored || perm || geometry != GEO_NN || G != 32 || !pair_instantiated(op, crossing == CR_ORTH, M, V, p.gr, true))
      return fail(MG_E_CONFIG, "no warp-pair kernel for op=%d crossing=%d geometry=%d M=%d G=%d V=%d", op, crossing,
                  geometry, M, G, V);
  } else if (p.occ2) {
  } else if (wide ? (perm || stored || !wide_instantiated(op, crossing == CR_ORTH, V, p.gr))
           : perm ? !perm_instantiated(op, crossing == CR_ORTH, M, V, p.gr)
                  : (stored ? !instantiated_stored(OP_BWD, M, V)
                            : !(instantiated(op, M, V) ||
                                (geometry == GEO_NN && nn_small_instantiated(op, p.real, M, V, p.gr, G == 32)))))
    return fail(MG_E_CONFIG, "no %skernel instantiated for op=%d M=%d V=%d",
                wide ? "wide-mesh " : perm ? "permuted-mesh " : "", stored ? MG_OP_BWD_STORED : op, M, V);
  p.M = M; p.V = V; p.G = G; p.logG = ilog2(G); p.R = 32 / G; p.np2 = G * M / 2;
  // split launch: when one wave of uniform CTAs cannot cover the SMs evenly (B between SMs x 4 warps x V
  // and SMs x 4 warps x (2V-1) vectors), run two 4-warp CTAs per SM holding V and V-1 vectors per lane
  // group.  split: 0 auto, 1 on, 2 off.  Automatic for forward propagation only: measured on GB300 at
  // N=256, B=4096 it saves 5% there, while back-propagation gets 28% slower: its two bodies (V and
  // V-1, ~25 KB of code each) overflow the instruction cache together (ncu: instruction-fetch stalls
  // 17x those of the uniform launch).
  p.split = false;
  p.nA = 0;
  if (split_mode != 2 && !p.pair && !p.occ2 && (op == OP_FWD || op == OP_BWD) && V >= 2 && !stored && !perm &&
      split_instantiated(op, crossing == CR_ORTH, M, V, G == 32, p.gr)) {
    const long ws = (cfg && cfg->W) ? cfg->W : 4;
    const long capA = ws * p.R * V, capB = ws * p.R * (V - 1);
    p.split = split_mode == 1 ||
              (op == OP_FWD && (long)di.sms * capA < B && B <= (long)di.sms * (capA + capB));
  }
  const unsigned tslot = p.real ? 16 : 32;               // bytes per slot of a T tile
  // layer tiles are copied by bulk TMA: every size and offset must be a multiple of 16 bytes
  p.lb = (unsigned)align16((size_t)p.np2 * tslot * (op == OP_FWDDIFF ? 2 : 1) + (p.gr == 1 ? (size_t)p.np2 * 8 : 0));
  p.dlb = (op == OP_BWD && p.gr == 0) ? (unsigned)(p.np2 * (p.real ? 16 : 64)) : 0;
  const int gslot = (op != OP_BWD) ? 0 : ((p.gr == 1 || p.gr == 2) ? 8 : (p.real ? 16 : 32));
  const size_t gstl = (size_t)p.np2 * gslot;
  const int maxw = p.occ2 ? 8 : prop_max_threads(op, M, V) / 32;
  int W = (cfg && cfg->W) ? cfg->W : (p.split ? 4 : (p.pair || p.occ2) ? 8 : 0);
  if (p.pair && (W & 1)) return fail(MG_E_CONFIG, "a warp-pair launch needs an even W, got %d", W);
  if (!W) {
    // enough warps to cover the batch in one wave, rounded up to a multiple of 4 so the four
    // schedulers of an SM carry equal work (measured: 8 warps on 128 SMs beat 7 warps on 147)
    const long per_warp = (long)p.R * V;
    const long warps = (B + per_warp - 1) / per_warp;
    long w = std::max<long>((warps + di.sms - 1) / di.sms, 1);
    if (w > 2) w = (w + 3) / 4 * 4;
    W = (int)std::min<long>(w, std::min(8, maxw));
  }
  if (W < 1 || W > maxw) return fail(MG_E_CONFIG, "W=%d warps outside [1, %d]", W, maxw);
  int S = (cfg && cfg->S) ? cfg->S : ((op == OP_FWD || p.split) ? 2 : 3);
  if (S < 1 || S > 8) return fail(MG_E_CONFIG, "S=%d stages outside [1, 8]", S);
  // a split launch keeps two CTAs resident per SM (each also pays the 1 KB the SM reserves per CTA)
  const size_t budget = (p.split || p.occ2) ? (size_t)di.smem_per_sm / 2 - 1024 : (size_t)di.smem_optin - 1024;
  int CL = (cfg && cfg->CL) ? cfg->CL : 0;
  const size_t per_layer = (size_t)S * p.lb + p.dlb + W * gstl;
  const size_t fixed = 8 * (size_t)(S + 1) + (L <= kMaxSmemKinds ? 4 * (size_t)L : 0) +
                       (perm ? 16 + perm_scratch_bytes(W, M, p.real) : 0);
  if (!CL) {
    // forward: deep enough to hide the copies, shallow enough to start soon (split CTAs: about 68 KB measured best)
    const size_t target = (op == OP_BWD) ? budget : std::min<size_t>(budget, (p.split ? 68 : 160) * 1024);
    CL = (int)std::max<size_t>(1, std::min<size_t>(16, (target > fixed ? target - fixed : 0) / per_layer));
    if (L > 0) CL = std::min(CL, L);
    // a uniform forward launch whose tiles all fit the target takes them in one copy and one stage: no chunk
    // boundaries (measured on GB300 at N=64, L=64, B=1024: 7.4 us against 8.3 us with 16-layer chunks in 2 stages)
    if (op == OP_FWD && !p.split && !(cfg && cfg->S) && L > 16 && fixed + (size_t)L * p.lb + W * gstl <= target) {
      S = 1;
      CL = L;
    }
  }
  if (CL < 1) return fail(MG_E_CONFIG, "CL=%d", CL);
  p.W = W; p.S = S; p.CL = CL;
  p.smem = launch_smem(p, op, gslot, L);
  if (p.smem > budget)
    return fail(MG_E_CONFIG, "shared memory %zu B above the %zu B available (M=%d W=%d CL=%d S=%d)", p.smem, budget, M,
                W, CL, S);
  if (p.lb % 16 || p.dlb % 16) return fail(MG_E_CONFIG, "tile sizes %u/%u not multiples of 16 bytes", p.lb, p.dlb);
  if ((size_t)CL * p.lb >= (1u << 20) || (size_t)CL * p.dlb >= (1u << 20))
    return fail(MG_E_CONFIG, "one pipeline stage exceeds the 1 MB bulk-copy limit");
  const long per_cta = p.pair ? (long)(W / 2) * V : (long)W * p.R * V;
  p.grid = (int)((B + per_cta - 1) / per_cta);
  if (p.split) {
    const long capB = (long)W * p.R * (V - 1);
    const long nA = std::min<long>(di.sms, (B + per_cta - 1) / per_cta);
    const long rem = std::max<long>(0, (long)B - nA * per_cta);
    p.nA = (int)nA;
    p.grid = (int)(nA + (rem + capB - 1) / capB);
  }
  p.off_kinds = 256;
  p.off_tiles = p.off_kinds + align256((size_t)std::max(L, 1) * 12);   // kinds + (shift, len)
  p.off_dtiles = p.off_tiles + align256((size_t)L * p.lb);
  p.off_perm = p.off_dtiles + align256((size_t)L * p.dlb);
  p.off_partial = p.off_perm + (perm ? align256(perm_table_bytes(N, L)) : 0);
  p.total = p.off_partial + ((op == OP_BWD) ? align256((size_t)p.grid * L * p.np2 * (p.gr == 4 ? 32 : 8)) : 0);
  return MG_OK;
}

int check_ws(const Plan& p, void* ws, size_t bytes) {
  if (!ws) return fail(MG_E_WORKSPACE, "workspace is NULL (need %zu bytes)", p.total);
  if ((reinterpret_cast<uintptr_t>(ws) & 255) != 0) return fail(MG_E_WORKSPACE, "workspace not 256-byte aligned");
  if (bytes < p.total) return fail(MG_E_WORKSPACE, "workspace has %zu bytes, needs %zu", bytes, p.total);
  return MG_OK;
}

int check_field(const void* ptr, const char* name, bool real, bool required) {
  if (!ptr) return required ? fail(MG_E_ARG, "%s is NULL", name) : MG_OK;
  const uintptr_t a = reinterpret_cast<uintptr_t>(ptr);
  if (a & (real ? 7 : 15)) return fail(MG_E_ARG, "%s not %d-byte aligned", name, real ? 8 : 16);
  return MG_OK;
}

int check_params(const Plan& p, const float* pp, int ldp, const float* s, int lds, const void* Tgen) {
  if (p.L == 0) return MG_OK;
  if (p.crossing == CR_GENERIC) {
    if (!Tgen) return fail(MG_E_ARG, "generic crossing needs Tgen");
    return MG_OK;
  }
  const int n_p = crossing_np(p.crossing), n_s = crossing_ns(p.crossing);
  if (!pp) return fail(MG_E_ARG, "p is NULL");
  if (ldp < p.N / 2 * n_p) return fail(MG_E_ARG, "ldp=%d < N/2*n_p=%d (gpu/mesh.py:155)", ldp, p.N / 2 * n_p);
  if (s && n_s == 0) return fail(MG_E_ARG, "crossing %d takes no splitter array", p.crossing);
  if (s && lds < p.N / 2 * n_s) return fail(MG_E_ARG, "lds=%d < N/2*n_s=%d", lds, p.N / 2 * n_s);
  return MG_OK;
}

CoefArgs coef_args(const Plan& P, const int* lens, const int* shifts, const int* strides, const float* p, int ldp,
                   const float* s, int lds, const float* dp, const void* Tgen, const void* Dgen, unsigned char* ws) {
  CoefArgs a;
  a.N = P.N; a.L = P.L; a.crossing = P.crossing; a.geometry = P.geometry; a.op = P.op;
  a.gr = P.gr;
  a.M = P.M; a.G = P.G;
  a.lens = lens; a.shifts = shifts; a.strides = strides;
  a.p = p; a.ldp = ldp; a.s = s; a.lds = lds; a.dp = dp;
  a.Tgen = static_cast<const float2*>(Tgen);
  a.Dgen = static_cast<const float2*>(Dgen);
  a.tiles = ws + P.off_tiles; a.layer_bytes = P.lb;
  a.dtiles = ws + P.off_dtiles; a.dlayer_bytes = P.dlb;
  a.kinds = reinterpret_cast<int*>(ws + P.off_kinds);
  a.status = reinterpret_cast<int*>(ws);
  return a;
}

// MZI crossings without derivative tiles take the float-float quad form of the coefficient pass
bool quad_coef(const Plan& P) { return P.crossing == CR_MZI && (P.op == OP_FWD || (P.op == OP_BWD && P.gr == 1)); }

int build_tiles(const Plan& P, const int* lens, const int* shifts, const int* strides, const float* p, int ldp,
                const float* s, int lds, const float* dp, const void* Tgen, const void* Dgen, unsigned char* ws,
                cudaStream_t st) {
  if (P.L == 0) return MG_OK;
  if (P.geometry == GEO_NN && (!lens || !shifts)) return fail(MG_E_ARG, "lens/shifts are NULL");
  if (P.geometry == GEO_FFT && !strides) return fail(MG_E_ARG, "strides is NULL");
  const CoefArgs a = coef_args(P, lens, shifts, strides, p, ldp, s, lds, dp, Tgen, Dgen, ws);
  // MZI crossings without derivative tiles (forward, and back-propagation with direct gradients) take the
  // float-float path with a quad of lanes per slot: the four sin/cos chains of a slot run side by side.  Measured
  // on GB300 (ncu, N=64, L=64) one thread per slot spent ~8500 cycles per warp on a 1550-instruction chain; the
  // pass is latency-bound for small meshes, so it is spread over every SM in blocks of 32 to 256 threads.
  const bool quad = quad_coef(P);
  const int n = P.L * P.np2 * (quad ? 4 : 1);
  const int sms = dev_info().sms;
  int bt = 256;
  if (n < 256 * sms) bt = std::max(32, std::min(256, ((n + sms - 1) / sms + 31) / 32 * 32));
  if (quad) coef_kernel<true><<<(n + bt - 1) / bt, bt, 0, st>>>(a);
  else coef_kernel<false><<<(n + bt - 1) / bt, bt, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "coef_kernel launch");
}

// Permutation arguments of a launch over layers [l0, l1) of plan P (the launch's layer i is layer l0 + i):
// forward kinds gather forward row l before layer l and row L after layer L-1 (only when the range
// ends there); back-propagation gathers row l (the inverse of perms[l+1]) before its step through layer
// l and row L (the inverse of perms[0]) after layer 0 (only when the range starts there).
void set_perm_args(const Plan& P, unsigned char* ws, int l0, int l1, PropArgs& a) {
  a.perm = a.pflags = a.perm_last = a.pflag_last = nullptr;
  if (!P.perm) return;
  const bool bwd = P.op == OP_BWD;
  const int* tab = reinterpret_cast<const int*>(ws + P.off_perm) + (bwd ? (size_t)(P.L + 1) * P.N : 0);
  const int* flags = reinterpret_cast<const int*>(ws + P.off_perm) + 2 * (size_t)(P.L + 1) * P.N + (bwd ? P.L + 1 : 0);
  a.perm = tab + (size_t)l0 * P.N;
  a.pflags = flags + l0;
  if (bwd ? l0 == 0 : l1 == P.L) {
    a.perm_last = tab + (size_t)P.L * P.N;
    a.pflag_last = flags + P.L;
  }
}

PropArgs prop_args(const Plan& P, const void* in0, const void* in1, void* out0, void* out1, int ldu, unsigned char* ws,
                   const void* target, void* ckpt, int ckpt_every, unsigned long long wait_ns, int unarmed) {
  PropArgs a{};
  a.wait_ns = wait_ns;
  a.unarmed = unarmed;
  a.target = target;
  a.act = nullptr;
  a.act_plane = 0;
  a.N = P.N; a.L = P.L; a.B = P.B; a.ldu = ldu;
  a.G = P.G; a.logG = P.logG; a.W = P.W; a.CL = P.CL; a.S = P.S;
  a.layer_bytes = P.lb; a.dlayer_bytes = P.dlb;
  a.tiles = ws + P.off_tiles; a.dtiles = ws + P.off_dtiles;
  a.kinds = reinterpret_cast<const int*>(ws + P.off_kinds);
  a.in0 = in0; a.in1 = in1; a.out0 = out0; a.out1 = out1;
  a.partial = reinterpret_cast<float2*>(ws + P.off_partial);
  a.status = reinterpret_cast<int*>(ws);
  a.ckpt = ckpt;
  a.ckpt_every = ckpt_every;
  a.ckpt_plane = (size_t)P.B * ldu;
  set_perm_args(P, ws, 0, P.L, a);
  a.nA = P.nA;
  return a;
}

int run_prop(const Plan& P, const void* in0, const void* in1, void* out0, void* out1, int ldu, float* dp, int ldp,
             int accumulate, unsigned char* ws, cudaStream_t st, const void* target = nullptr, void* ckpt = nullptr,
             int ckpt_every = 0, unsigned long long wait_ns = 0, int unarmed = 0) {
  if (P.B == 0) return MG_OK;
  PropArgs a = prop_args(P, in0, in1, out0, out1, ldu, ws, target, ckpt, ckpt_every, wait_ns, unarmed);
  LaunchCfg lc;
  lc.grid = dim3(P.grid);
  lc.block = dim3(32 * P.W);
  lc.smem = P.smem;
  lc.stream = st;
  cudaError_t e;
  if (P.pair)
    e = launch_prop_pair(P.V, lc, a);
  else if (P.occ2)
    e = launch_prop_nn2(P.op, P.real, P.M, P.V, P.gr, lc, a);
  else if (P.M == kWideM)
    e = launch_prop_wide(P.op, P.real, P.V, P.gr, lc, a);
  else if (!P.perm && P.geometry == GEO_NN && nn_instantiated(P.op, P.real, P.M, P.V, P.gr, P.G == 32, P.split))
    e = launch_prop_nn(P.op, P.real, P.M, P.V, P.gr, P.G == 32, P.split, lc, a);
  else
    e = P.split ? launch_prop_split(P.op, P.real, P.M, P.V, P.G == 32, P.gr, lc, a)
                : launch_prop(P.op, P.real, P.M, P.V, P.G == 32, P.gr, lc, a);
  if (e != cudaSuccess) return cuda_fail(e, "prop_kernel launch");
  if (P.op == OP_BWD && dp && P.L > 0) {
    const int n = P.L * P.np2;
    dp_reduce_kernel<<<(n + kReduceCols - 1) / kReduceCols, kReduceCols * kReduceRows, 0, st>>>(
        a.partial, P.grid, P.L, P.np2, P.M, P.G, P.N, dp, ldp,
                                                        crossing_np(P.crossing), accumulate,
                                                        reinterpret_cast<const int*>(ws + P.off_kinds) + P.L);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "dp_reduce_kernel launch");
  }
  return MG_OK;
}

int check_ldu(const Plan& P, int ldu) {
  if (ldu < P.N || (ldu & 1)) return fail(MG_E_ARG, "ldu=%d must be >= N=%d and even", ldu, P.N);
  return MG_OK;
}

#define TRY(x)                  \
  do {                          \
    int _rc = (x);              \
    if (_rc != MG_OK) return _rc; \
  } while (0)

int fwdprop_impl(int geo, int N, int L, int B, const int* lens, const int* shifts, const int* strides, const float* p,
                 int ldp, const float* s, int lds, const void* u_in, void* u_out, int ldu, int crossing, void* ws,
                 size_t wsb, void* stream) {
  g_err.clear();
  Plan P;
  TRY(make_plan(OP_FWD, N, L, B, crossing, geo, nullptr, &P));
  if (crossing == CR_GENERIC) return fail(MG_E_ARG, "use mg_build_tiles for generic crossings");
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(u_in, "u_in", P.real, B > 0));
  TRY(check_field(u_out, "u_out", P.real, B > 0));
  TRY(check_params(P, p, ldp, s, lds, nullptr));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  TRY(build_tiles(P, lens, shifts, strides, p, ldp, s, lds, nullptr, nullptr, nullptr, w, st));
  return run_prop(P, u_in, nullptr, u_out, nullptr, ldu, nullptr, 0, 0, w, st);
}

int fwddiff_impl(int geo, int N, int L, int B, const int* lens, const int* shifts, const int* strides, const float* p,
                 const float* dp, int ldp, const float* s, int lds, const void* u_in, const void* du_in, void* u_out,
                 void* du_out, int ldu, int crossing, void* ws, size_t wsb, void* stream) {
  g_err.clear();
  Plan P;
  TRY(make_plan(OP_FWDDIFF, N, L, B, crossing, geo, nullptr, &P));
  if (crossing == CR_GENERIC) return fail(MG_E_ARG, "use mg_build_tiles for generic crossings");
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(u_in, "u_in", P.real, B > 0));
  TRY(check_field(du_in, "du_in", P.real, false));
  TRY(check_field(u_out, "u_out", P.real, B > 0));
  TRY(check_field(du_out, "du_out", P.real, B > 0));
  TRY(check_params(P, p, ldp, s, lds, nullptr));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  TRY(build_tiles(P, lens, shifts, strides, p, ldp, s, lds, dp, nullptr, nullptr, w, st));
  return run_prop(P, u_in, du_in, u_out, du_out, ldu, nullptr, 0, 0, w, st);
}

int backdiff_impl(int geo, int N, int L, int B, const int* lens, const int* shifts, const int* strides, const float* p,
                  float* dp, int ldp, const float* s, int lds, const void* u_out, const void* dJdu_out, void* u_in,
                  void* dJdu_in, int ldu, int crossing, int accumulate, void* ws, size_t wsb, void* stream) {
  g_err.clear();
  Plan P;
  TRY(make_plan(OP_BWD, N, L, B, crossing, geo, nullptr, &P));
  if (crossing == CR_GENERIC) return fail(MG_E_ARG, "use mg_build_tiles for generic crossings");
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(u_out, "u_out", P.real, B > 0));
  TRY(check_field(dJdu_out, "dJdu_out", P.real, B > 0));
  TRY(check_field(u_in, "u_in", P.real, false));
  TRY(check_field(dJdu_in, "dJdu_in", P.real, B > 0));
  TRY(check_params(P, p, ldp, s, lds, nullptr));
  if (!dp && L > 0) return fail(MG_E_ARG, "dp is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  if (B == 0) {
    if (!accumulate && L > 0) {
      cudaError_t e = cudaMemsetAsync(dp, 0, sizeof(float) * ((size_t)(L - 1) * ldp + (size_t)N / 2 * crossing_np(crossing)), st);
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(dp)");
    }
    return MG_OK;
  }
  TRY(build_tiles(P, lens, shifts, strides, p, ldp, s, lds, nullptr, nullptr, nullptr, w, st));
  return run_prop(P, u_out, dJdu_out, u_in, dJdu_in, ldu, dp, ldp, accumulate, w, st);
}

// Gather tables of the reference's perms ((L+1) x N, row k gathered before layer k, row L after the
// last layer), one block per row k: forward row k = perms[k]; back-propagation row k-1 (row L for k = 0)
// = the inverse of perms[k], so that the backward step through layer l is preceded by the inverse of
// perms[l+1] and the last one is the inverse of perms[0] (mesh.py:381-390 with perms_bk = argsort(perms)).
// Flags mark rows that move something.  A row that is not a permutation of 0..N-1 becomes the identity
// and records bad geometry.
__global__ void perm_build_kernel(int N, int L, const int* __restrict__ perms, int* fwd, int* bwd, int* fflags,
                                  int* bflags, int* status) {
  __shared__ int hits[512];
  __shared__ int bad, moved;
  const int k = blockIdx.x;
  const int* row = perms + (size_t)k * N;
  if (threadIdx.x == 0) {
    bad = 0;
    moved = 0;
  }
  for (int q = threadIdx.x; q < N; q += blockDim.x) hits[q] = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    const int t = row[q];
    if ((unsigned)t < (unsigned)N) atomicAdd(&hits[t], 1);
    else atomicOr(&bad, 1);
    if (t != q) atomicOr(&moved, 1);
  }
  __syncthreads();
  for (int q = threadIdx.x; q < N; q += blockDim.x)
    if (hits[q] != 1) atomicOr(&bad, 1);
  __syncthreads();
  const int kb = (k == 0) ? L : k - 1;
  int* f = fwd + (size_t)k * N;
  int* b = bwd + (size_t)kb * N;
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    if (bad) {
      f[q] = q;
      b[q] = q;
    } else {
      const int t = row[q];
      f[q] = t;
      b[t] = q;
    }
  }
  if (threadIdx.x == 0) {
    const int fl = (!bad && moved) ? 1 : 0;
    fflags[k] = fl;
    bflags[kb] = fl;
    if (bad) set_status(status, ST_BAD_GEOMETRY);
  }
}

__global__ void fma_probe_kernel(float* sink, int iters, float m) {
  float a[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) a[k] = threadIdx.x * 1e-3f + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = fmaf(a[k], m, 0.25f);
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = fmaf(a[k], m, -0.25f);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 32; ++k) s += a[k];
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// sincos_d, sincos_c and sincos_small (the coefficient precompute's own double sin/cos: full precision,
// tile precision, small splitter angles) against the library sincos
__global__ void trig_check_kernel(const double* x, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s, c, s2, c2, s3, c3, s4, c4;
  sincos_d(x[i], &s, &c);
  sincos(x[i], &s2, &c2);
  sincos_c(x[i], &s3, &c3);
  sincos_small(x[i], &s4, &c4);
  out[6 * i] = s - s2;
  out[6 * i + 1] = c - c2;
  out[6 * i + 2] = s3 - s2;
  out[6 * i + 3] = c3 - c2;
  out[6 * i + 4] = s4 - s2;
  out[6 * i + 5] = c4 - c2;
}

// The same chains with packed FP32 pairs (one fma.rn.f32x2 = two FMAs per lane): whether the FMA pipe
// retires more FLOPs per clock through the packed form than through scalar FMAs.
__global__ void fma2_probe_kernel(float* sink, int iters, float m) {
  float2 a[32];
#pragma unroll
  for (int k = 0; k < 32; ++k) a[k] = make_float2(threadIdx.x * 1e-3f + k, threadIdx.x * 2e-3f - k);
  const float2 mm = make_float2(m, m), p = make_float2(0.25f, 0.25f), q = make_float2(-0.25f, -0.25f);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = __ffma2_rn(a[k], mm, p);
#pragma unroll
    for (int k = 0; k < 32; ++k) a[k] = __ffma2_rn(a[k], mm, q);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 32; ++k) s += a[k].x + a[k].y;
  sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

namespace mg {
// Record an error message for mg_last_error() from another translation unit of the library.
int set_last_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
}  // namespace mg

extern "C" {

const char* mg_last_error(void) { return g_err.c_str(); }

const char* mg_version(void) { return "meshes_gb300 0.1 (sm_103a)"; }

size_t mg_workspace_bytes(int op, int N, int L, int B, int crossing, int geometry, const mg_config* cfg) {
  Plan P;
  if (make_plan(op, N, L, B, crossing, geometry, cfg, &P) != MG_OK) return 0;
  return P.total;
}

int mg_workspace_init(void* ws, size_t bytes, void* stream) {
  g_err.clear();
  if (!ws || bytes < 256) return fail(MG_E_WORKSPACE, "workspace NULL or smaller than 256 bytes");
  cudaError_t e = cudaMemsetAsync(ws, 0, 256, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "cudaMemsetAsync(status)");
}

int mg_read_status(void* ws, int clear, void* stream) {
  g_err.clear();
  if (!ws) return fail(MG_E_WORKSPACE, "workspace is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, ws, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "reading status");
  if (clear && v) {
    e = cudaMemsetAsync(ws, 0, sizeof(int), st);
    if (e != cudaSuccess) return cuda_fail(e, "clearing status");
  }
  return v;
}

int mg_default_config(int op, int N, int B, int crossing, mg_config* out) {
  g_err.clear();
  Plan P;
  TRY(make_plan(op, N, 1, B, crossing, GEO_NN, nullptr, &P));
  if (out) {
    out->M = P.M; out->V = P.V; out->W = P.W; out->CL = P.CL; out->S = P.S;
  }
  return MG_OK;
}

int mg_fwdprop(int N, int L, int B, const int* lens, const int* shifts, const float* p, int ldp, const float* s,
               int lds, const void* u_in, void* u_out, int ldu, int crossing, void* ws, size_t wsb, void* stream) {
  return fwdprop_impl(GEO_NN, N, L, B, lens, shifts, nullptr, p, ldp, s, lds, u_in, u_out, ldu, crossing, ws, wsb,
                      stream);
}
int mg_fwdprop_ft(int N, int L, int B, const int* strides, const float* p, int ldp, const float* s, int lds,
                  const void* u_in, void* u_out, int ldu, int crossing, void* ws, size_t wsb, void* stream) {
  return fwdprop_impl(GEO_FFT, N, L, B, nullptr, nullptr, strides, p, ldp, s, lds, u_in, u_out, ldu, crossing, ws,
                      wsb, stream);
}
int mg_fwddiff(int N, int L, int B, const int* lens, const int* shifts, const float* p, const float* dp, int ldp,
               const float* s, int lds, const void* u_in, const void* du_in, void* u_out, void* du_out, int ldu,
               int crossing, void* ws, size_t wsb, void* stream) {
  return fwddiff_impl(GEO_NN, N, L, B, lens, shifts, nullptr, p, dp, ldp, s, lds, u_in, du_in, u_out, du_out, ldu,
                      crossing, ws, wsb, stream);
}
int mg_fwddiff_ft(int N, int L, int B, const int* strides, const float* p, const float* dp, int ldp, const float* s,
                  int lds, const void* u_in, const void* du_in, void* u_out, void* du_out, int ldu, int crossing,
                  void* ws, size_t wsb, void* stream) {
  return fwddiff_impl(GEO_FFT, N, L, B, nullptr, nullptr, strides, p, dp, ldp, s, lds, u_in, du_in, u_out, du_out,
                      ldu, crossing, ws, wsb, stream);
}
int mg_backdiff(int N, int L, int B, const int* lens, const int* shifts, const float* p, float* dp, int ldp,
                const float* s, int lds, const void* u_out, const void* dJdu_out, void* u_in, void* dJdu_in, int ldu,
                int crossing, int accumulate, void* ws, size_t wsb, void* stream) {
  return backdiff_impl(GEO_NN, N, L, B, lens, shifts, nullptr, p, dp, ldp, s, lds, u_out, dJdu_out, u_in, dJdu_in,
                       ldu, crossing, accumulate, ws, wsb, stream);
}
int mg_backdiff_ft(int N, int L, int B, const int* strides, const float* p, float* dp, int ldp, const float* s,
                   int lds, const void* u_out, const void* dJdu_out, void* u_in, void* dJdu_in, int ldu, int crossing,
                   int accumulate, void* ws, size_t wsb, void* stream) {
  return backdiff_impl(GEO_FFT, N, L, B, nullptr, nullptr, strides, p, dp, ldp, s, lds, u_out, dJdu_out, u_in,
                       dJdu_in, ldu, crossing, accumulate, ws, wsb, stream);
}

int mg_build_tiles(int op, int N, int L, int geometry, const int* lens, const int* shifts, const int* strides,
                   int crossing, const float* p, int ldp, const float* s, int lds, const float* dp, const void* Tgen,
                   const void* Dgen, int B, const mg_config* cfg, void* ws, size_t wsb, void* stream) {
  g_err.clear();
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, geometry, cfg, &P));
  TRY(check_ws(P, ws, wsb));
  TRY(check_params(P, p, ldp, s, lds, Tgen));
  if (crossing == CR_GENERIC && op == OP_BWD && !Dgen && L > 0) return fail(MG_E_ARG, "generic back-prop needs Dgen");
  if (crossing == CR_GENERIC && op == OP_FWDDIFF) return fail(MG_E_ARG, "generic crossings support fwd and bwd only");
  if (P.perm) {   // no permutation until mg_build_perms writes the tables
    cudaError_t e = cudaMemsetAsync(static_cast<unsigned char*>(ws) + P.off_perm + 8 * (size_t)(L + 1) * N, 0,
                                    8 * (size_t)(L + 1), static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(permutation flags)");
  }
  return build_tiles(P, lens, shifts, strides, p, ldp, s, lds, dp, Tgen, Dgen, static_cast<unsigned char*>(ws),
                     static_cast<cudaStream_t>(stream));
}

int mg_propagate(int op, int N, int L, int B, int crossing, int geometry, const void* in0, const void* in1, void* out0,
                 void* out1, int ldu, float* dp, int ldp, int accumulate, const mg_config* cfg, void* ws, size_t wsb,
                 void* stream) {
  g_err.clear();
  if (op == MG_OP_FWD_BWDTILES) {
    // forward propagation reading the tiles mg_build_tiles(MG_OP_BWD) wrote: the layer stride and the
    // workspace layout are the back-propagation plan's, the kernel is the forward one
    if ((geometry & ~MG_GEO_PERM) != GEO_NN)
      return fail(MG_E_ARG, "forward from back-propagation tiles needs nearest-neighbour geometry");
    Plan Pb, Pf;
    TRY(make_plan(OP_BWD, N, L, B, crossing, geometry, cfg, &Pb));
    TRY(check_ws(Pb, ws, wsb));
    mg_config cf = {Pb.M, 0, 0, 0, 0, (cfg && cfg->split != 3 && cfg->split != 4) ? cfg->split : 0};
    mg_config tf;   // a measured forward configuration of this shape applies if its M matches the tiles'
    if (!cfg && !Pb.perm && lookup_tuned(OP_FWD, crossing, Pb.geometry, N, B, &tf) && tf.M == Pb.M) cf = tf;
    TRY(make_plan(OP_FWD, N, L, B, crossing, geometry, &cf, &Pf));
    Pf.lb = Pb.lb;
    Pf.off_kinds = Pb.off_kinds;
    Pf.off_tiles = Pb.off_tiles;
    Pf.off_perm = Pb.off_perm;   // the forward rows of the tables mg_build_perms wrote for this workspace
    const DevInfo di = dev_info();
    const size_t budget = Pf.split ? (size_t)di.smem_per_sm / 2 - 1024 : (size_t)di.smem_optin - 1024;
    for (;;) {
      Pf.smem = launch_smem(Pf, OP_FWD, 0, L);
      if (Pf.smem <= budget && (size_t)Pf.CL * Pf.lb < (1u << 20)) break;
      if (Pf.CL == 1) return fail(MG_E_CONFIG, "no pipeline depth fits shared memory");
      Pf.CL -= 1;   // the back-propagation tiles are larger than the forward ones the plan was sized for
    }
    TRY(check_ldu(Pf, ldu));
    TRY(check_field(in0, "in0", Pf.real, B > 0));
    TRY(check_field(out0, "out0", Pf.real, B > 0));
    return run_prop(Pf, in0, nullptr, out0, nullptr, ldu, nullptr, 0, 0, static_cast<unsigned char*>(ws),
                    static_cast<cudaStream_t>(stream));
  }
  if (op == MG_OP_BWD_STORED) return fail(MG_E_ARG, "stored-activation back-propagation runs through mg_propagate_range");
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, geometry, cfg, &P));
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(in0, "in0", P.real, B > 0));
  TRY(check_field(in1, "in1", P.real, op == OP_BWD && B > 0));
  TRY(check_field(out0, "out0", P.real, op != OP_BWD && B > 0));
  TRY(check_field(out1, "out1", P.real, op != OP_FWD && B > 0));
  if (op == OP_BWD && dp && ldp < N / 2 * crossing_np(crossing)) return fail(MG_E_ARG, "ldp too small");
  return run_prop(P, in0, in1, out0, out1, ldu, dp, ldp, accumulate, static_cast<unsigned char*>(ws),
                  static_cast<cudaStream_t>(stream));
}

int mg_propagate_wait_test(int op, int N, int L, int B, int crossing, const void* in0, const void* in1, void* out0,
                           void* out1, int ldu, unsigned long long wait_ns, int unarmed_chunk, void* ws, size_t wsb,
                           void* stream) {
  g_err.clear();
  if (op != OP_FWD && op != OP_BWD) return fail(MG_E_ARG, "op must be MG_OP_FWD or MG_OP_BWD");
  if (wait_ns == 0) return fail(MG_E_ARG, "wait_ns must be positive");
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, GEO_NN, nullptr, &P));
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(in0, "in0", P.real, B > 0));
  TRY(check_field(in1, "in1", P.real, op == OP_BWD && B > 0));
  TRY(check_field(out0, "out0", P.real, op != OP_BWD && B > 0));
  TRY(check_field(out1, "out1", P.real, op != OP_FWD && B > 0));
  const int nch = (L + P.CL - 1) / P.CL;
  if (unarmed_chunk < 0 || unarmed_chunk >= nch)
    return fail(MG_E_ARG, "unarmed_chunk=%d outside the launch's %d pipeline chunks", unarmed_chunk, nch);
  return run_prop(P, in0, in1, out0, out1, ldu, nullptr, 0, 0, static_cast<unsigned char*>(ws),
                  static_cast<cudaStream_t>(stream), nullptr, nullptr, 0, wait_ns, unarmed_chunk + 1);
}

int mg_build_perms(int op, int N, int L, int B, int crossing, int geometry, const int* perms, const mg_config* cfg,
                   void* ws, size_t wsb, void* stream) {
  g_err.clear();
  if (op == MG_OP_FWD_BWDTILES) op = OP_BWD;   // the forward kernel on back-propagation tiles shares their workspace
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, geometry, cfg, &P));
  if (!P.perm) return fail(MG_E_ARG, "geometry %d lacks MG_GEO_PERM", geometry);
  TRY(check_ws(P, ws, wsb));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned char* w = static_cast<unsigned char*>(ws);
  int* tab = reinterpret_cast<int*>(w + P.off_perm);
  int* fwd = tab;
  int* bwd = tab + (size_t)(L + 1) * N;
  int* fflags = tab + 2 * (size_t)(L + 1) * N;
  int* bflags = fflags + (L + 1);
  cudaError_t e;
  if (!perms) {
    e = cudaMemsetAsync(fflags, 0, 2 * sizeof(int) * (size_t)(L + 1), st);
    return e == cudaSuccess ? MG_OK : cuda_fail(e, "cudaMemsetAsync(permutation flags)");
  }
  if (reinterpret_cast<uintptr_t>(perms) & 3) return fail(MG_E_ARG, "perms not 4-byte aligned");
  perm_build_kernel<<<L + 1, 256, 0, st>>>(N, L, perms, fwd, bwd, fflags, bflags, reinterpret_cast<int*>(w));
  e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "perm_build_kernel launch");
}

int mg_set_tuned(int op, int crossing, int geometry, int N, int B_lo, int B_hi, const mg_config* cfg) {
  g_err.clear();
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  if (!cfg) {   // clear every entry of this (op, crossing, geometry, N)
    std::vector<Tuned> keep;
    for (const Tuned& t : g_tuned)
      if (!(t.op == op && t.crossing == crossing && t.geometry == geometry && (N == 0 || t.N == N))) keep.push_back(t);
    g_tuned.swap(keep);
    return MG_OK;
  }
  if (op < 0 || op > 2 || N < 2 || B_lo > B_hi) return fail(MG_E_ARG, "bad tuning entry");
  for (Tuned& t : g_tuned)
    if (t.op == op && t.crossing == crossing && t.geometry == geometry && t.N == N && t.Blo == B_lo && t.Bhi == B_hi) {
      t.cfg = *cfg;
      return MG_OK;
    }
  g_tuned.push_back(Tuned{op, crossing, geometry, N, B_lo, B_hi, *cfg});
  return MG_OK;
}

int mg_plan(int op, int N, int L, int B, int crossing, int geometry, const mg_config* cfg, mg_plan_info* out) {
  g_err.clear();
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, geometry, cfg, &P));
  if (out) {
    out->M = P.M; out->V = P.V; out->W = P.W; out->CL = P.CL; out->S = P.S; out->G = P.G; out->grid = P.grid;
    out->nA = P.split ? P.nA : 0;
    out->layer_bytes = P.lb; out->dlayer_bytes = P.dlb; out->smem = P.smem;
    out->off_kinds = P.off_kinds; out->off_tiles = P.off_tiles; out->off_dtiles = P.off_dtiles;
    out->off_partial = P.off_partial; out->total = P.total;
  }
  return MG_OK;
}

int mg_propagate_l2(int N, int L, int B, int crossing, int geometry, const void* y, const void* target, void* x_out,
                    void* g_out, int ldu, float* dp, int ldp, int accumulate, const mg_config* cfg, void* ws, size_t wsb,
                    void* stream) {
  g_err.clear();
  Plan P;
  TRY(make_plan(OP_BWD, N, L, B, crossing, geometry, cfg, &P));
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(y, "y", P.real, B > 0));
  TRY(check_field(target, "target", P.real, B > 0));
  TRY(check_field(x_out, "x_out", P.real, false));
  TRY(check_field(g_out, "g_out", P.real, B > 0));
  if (dp && ldp < N / 2 * crossing_np(crossing)) return fail(MG_E_ARG, "ldp too small");
  return run_prop(P, y, nullptr, x_out, g_out, ldu, dp, ldp, accumulate, static_cast<unsigned char*>(ws),
                  static_cast<cudaStream_t>(stream), target);
}

}  // extern "C"

namespace {

// Layer range [l0, l1) (mg_propagate_range).  With keep_partials, a stored-activation back-propagation
// leaves its per-CTA dJ/dT partials at their layers' places in the full-depth partial buffer (per-CTA blocks
// of L layers) and reduces nothing: the caller reduces all ranges at once (reduce_raw).
int range_impl(int op, int N, int L, int l0, int l1, int B, int crossing, int geometry, const void* in0,
               const void* in1, void* out0, void* out1, int ldu, void* act, void* dT, int accumulate,
               const mg_config* cfg, void* ws, size_t wsb, void* stream, bool keep_partials) {
  if (op != OP_FWD && op != MG_OP_BWD_STORED) return fail(MG_E_ARG, "op %d not in {MG_OP_FWD, MG_OP_BWD_STORED}", op);
  if (l0 < 0 || l1 < l0 || l1 > L) return fail(MG_E_ARG, "layer range [%d, %d) outside [0, %d)", l0, l1, L);
  // layer ranges run uniform CTAs (the stored-activation kernels have no split form)
  mg_config cu = cfg ? *cfg : mg_config{0, 0, 0, 0, 0, 0};
  cu.split = 2;
  cfg = &cu;
  Plan P;
  TRY(make_plan(op, N, L, B, crossing, geometry, cfg, &P));
  if (P.perm) return fail(MG_E_ARG, "layer ranges take no permutations");
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  const bool bwd = op == MG_OP_BWD_STORED;
  if (P.real && act) return fail(MG_E_ARG, "stored activations need a complex crossing");
  if (bwd && !act && B > 0 && l1 > l0) return fail(MG_E_ARG, "stored-activation back-propagation needs act");
  TRY(check_field(act, "act", P.real, false));
  TRY(check_field(in0, "in0", P.real, !bwd && B > 0));
  TRY(check_field(out0, "out0", P.real, false));
  TRY(check_field(in1, "in1", P.real, bwd && B > 0));
  TRY(check_field(out1, "out1", P.real, bwd && B > 0));
  if (bwd && !dT && B > 0 && l1 > l0 && !keep_partials) return fail(MG_E_ARG, "dT is NULL");
  if (dT && (reinterpret_cast<uintptr_t>(dT) & 7)) return fail(MG_E_ARG, "dT not 8-byte aligned");
  if (act && !bwd) {   // the forward kernel's store mode has its own (M, V) instantiations
    if (!(cfg && cfg->V)) P.V = stored_default_v(OP_FWD, P.M);
    if (!instantiated_stored(OP_FWD, P.M, P.V))
      return fail(MG_E_CONFIG, "no activation-storing forward kernel for M=%d V=%d", P.M, P.V);
    const long per_cta = (long)P.W * P.R * P.V;
    P.grid = (int)((B + per_cta - 1) / per_cta);
  }
  const int nl = l1 - l0;
  if (B == 0 || nl == 0) {
    if (bwd && B == 0 && dT && !accumulate && nl > 0) {   // no vectors: dJ/dT of the range is 0
      cudaError_t e = cudaMemsetAsync(static_cast<float2*>(dT) + (size_t)l0 * (N / 2) * 4, 0,
                                      (size_t)nl * (N / 2) * 32, static_cast<cudaStream_t>(stream));
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(dT)");
    }
    if (nl == 0 && B > 0) {   // empty range: the field passes through
      const size_t el = P.real ? 4 : 8;
      const void* src = bwd ? in1 : in0;
      void* dst = bwd ? out1 : out0;
      if (dst && dst != src) {
        cudaError_t e = cudaMemcpy2DAsync(dst, (size_t)ldu * el, src, (size_t)ldu * el, (size_t)N * el, B,
                                          cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync");
      }
    }
    return MG_OK;
  }
  // the launch sees layers [l0, l1) as its own layers [0, nl): tiles and kinds start at l0
  unsigned char* w = static_cast<unsigned char*>(ws);
  const int* kinds_full = reinterpret_cast<const int*>(w + P.off_kinds);
  P.smem = launch_smem(P, P.op, bwd ? 32 : 0, nl);
  PropArgs a{};
  a.target = nullptr;
  a.N = N; a.L = nl; a.B = B; a.ldu = ldu;
  a.G = P.G; a.logG = P.logG; a.W = P.W; a.CL = P.CL; a.S = P.S;
  a.layer_bytes = P.lb; a.dlayer_bytes = 0;
  a.tiles = w + P.off_tiles + (size_t)l0 * P.lb;
  a.dtiles = nullptr;
  a.kinds = kinds_full + l0;
  a.in0 = bwd ? nullptr : in0;
  a.in1 = bwd ? in1 : nullptr;
  a.out0 = bwd ? nullptr : out0;
  a.out1 = bwd ? out1 : nullptr;
  a.partial = reinterpret_cast<float2*>(w + P.off_partial) + (keep_partials ? (size_t)l0 * 4 * P.np2 : 0);
  a.pstride = keep_partials ? L : 0;
  a.status = reinterpret_cast<int*>(w);
  a.act = act;
  a.act_plane = (size_t)B * ldu;
  a.nA = 0;
  a.perm = a.pflags = a.perm_last = a.pflag_last = nullptr;
  LaunchCfg lc;
  lc.grid = dim3(P.grid);
  lc.block = dim3(32 * P.W);
  lc.smem = P.smem;
  lc.stream = static_cast<cudaStream_t>(stream);
  cudaError_t e = launch_prop(P.op, P.real, P.M, P.V, P.G == 32, act ? 4 : 0, lc, a);
  if (e != cudaSuccess) return cuda_fail(e, "prop_kernel launch");
  if (bwd && !keep_partials) {
    const int n = nl * P.np2;
    raw_reduce_kernel<<<(4 * n + kReduceCols - 1) / kReduceCols, kReduceCols * kReduceRows, 0, lc.stream>>>(
        a.partial, P.grid, nl, P.np2, P.M, P.G, N,
                                                             static_cast<float2*>(dT) + (size_t)l0 * (N / 2) * 4,
                                                             accumulate, kinds_full + L + 2 * l0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "raw_reduce_kernel launch");
  }
  return MG_OK;
}

// dT (complex64 [L][N/2][2][2]) from the stored-activation partials that every range launch of a lossy
// back-propagation left at its layers' places (range_impl with keep_partials): one reduction over all layers
int reduce_raw(int N, int L, int B, int geometry, void* dT, int accumulate, void* ws, size_t wsb, void* stream) {
  Plan P;
  mg_config cu{0, 0, 0, 0, 0, 2};
  TRY(make_plan(MG_OP_BWD_STORED, N, L, B, CR_GENERIC, geometry, &cu, &P));
  TRY(check_ws(P, ws, wsb));
  if (!dT) return fail(MG_E_ARG, "dT is NULL");
  if (reinterpret_cast<uintptr_t>(dT) & 7) return fail(MG_E_ARG, "dT not 8-byte aligned");
  unsigned char* w = static_cast<unsigned char*>(ws);
  const int n = L * P.np2;
  raw_reduce_kernel<<<(4 * n + kReduceCols - 1) / kReduceCols, kReduceCols * kReduceRows, 0,
                      static_cast<cudaStream_t>(stream)>>>(reinterpret_cast<const float2*>(w + P.off_partial), P.grid, L,
                                                           P.np2, P.M, P.G, N, static_cast<float2*>(dT), accumulate,
                                                           reinterpret_cast<const int*>(w + P.off_kinds) + L);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "raw_reduce_kernel launch");
}

}  // namespace

extern "C" {

int mg_propagate_range(int op, int N, int L, int l0, int l1, int B, int crossing, int geometry, const void* in0,
                       const void* in1, void* out0, void* out1, int ldu, void* act, void* dT, int accumulate,
                       const mg_config* cfg, void* ws, size_t wsb, void* stream) {
  g_err.clear();
  return range_impl(op, N, L, l0, l1, B, crossing, geometry, in0, in1, out0, out1, ldu, act, dT, accumulate, cfg, ws,
                    wsb, stream, false);
}

int mg_lossy_forward(int N, int L, int B, int geometry, int seg, const void* x, void* y, void* ckpt, int ldu, void* ws,
                     size_t wsb, void* stream) {
  g_err.clear();
  if (seg < 1) return fail(MG_E_ARG, "segment length %d < 1", seg);
  if (L == 0) {
    if (B > 0 && y != x) {
      cudaError_t e = cudaMemcpy2DAsync(y, (size_t)ldu * 8, x, (size_t)ldu * 8, (size_t)N * 8, B,
                                        cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream));
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync");
    }
    return MG_OK;
  }
  if (L > seg && !ckpt && B > 0) return fail(MG_E_ARG, "ckpt is NULL");
  // one launch over all layers; the kernel writes the field after every seg layers into ckpt (chunks of
  // layers are cut so that they end on those layers)
  Plan P;
  TRY(make_plan(OP_FWD, N, L, B, CR_GENERIC, geometry, nullptr, &P));
  TRY(check_ws(P, ws, wsb));
  TRY(check_ldu(P, ldu));
  TRY(check_field(x, "x", false, B > 0));
  TRY(check_field(y, "y", false, B > 0));
  TRY(check_field(ckpt, "ckpt", false, false));
  int cl = std::min(P.CL, seg);
  while (seg % cl) --cl;
  P.CL = cl;
  P.smem = launch_smem(P, OP_FWD, 0, L);
  return run_prop(P, x, nullptr, y, nullptr, ldu, nullptr, 0, 0, static_cast<unsigned char*>(ws),
                  static_cast<cudaStream_t>(stream), nullptr, L > seg ? ckpt : nullptr, seg);
}

int mg_lossy_backward(int N, int L, int B, int geometry, int seg, const void* x, const void* ckpt, const void* gy,
                      void* gx, void* gtmp, void* act, void* dT, int ldu, void* ws_fwd, size_t wsb_fwd, void* ws_bwd,
                      size_t wsb_bwd, void* stream) {
  g_err.clear();
  if (seg < 1) return fail(MG_E_ARG, "segment length %d < 1", seg);
  if (B > 0 && (!gy || !gx || !gtmp || !act || !x)) return fail(MG_E_ARG, "NULL buffer");
  if (L == 0) {
    if (B > 0 && gx != gy) {
      cudaError_t e = cudaMemcpy2DAsync(gx, (size_t)ldu * 8, gy, (size_t)ldu * 8, (size_t)N * 8, B,
                                        cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream));
      if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy2DAsync");
    }
    return MG_OK;
  }
  if (L > seg && !ckpt && B > 0) return fail(MG_E_ARG, "ckpt is NULL");
  const size_t plane = (size_t)B * ldu;
  const int K = (L + seg - 1) / seg;
  const void* g = gy;
  for (int k = K - 1; k >= 0; --k) {
    const int l0 = k * seg, l1 = std::min(L, l0 + seg);
    const void* in = (k == 0) ? x : static_cast<const void*>(static_cast<const float2*>(ckpt) + (size_t)(k - 1) * plane);
    // the layer inputs of the segment, recomputed from its checkpoint
    TRY(range_impl(OP_FWD, N, L, l0, l1, B, CR_GENERIC, geometry, in, nullptr, nullptr, nullptr, ldu, act, nullptr, 0,
                   nullptr, ws_fwd, wsb_fwd, stream, false));
    // back-propagation through them (its dJ/dT partials kept in place); gradients alternate between gx and
    // gtmp and end in gx
    void* out = (k % 2 == 0) ? gx : gtmp;
    TRY(range_impl(MG_OP_BWD_STORED, N, L, l0, l1, B, CR_GENERIC, geometry, nullptr, g, nullptr, out, ldu, act,
                   nullptr, 0, nullptr, ws_bwd, wsb_bwd, stream, true));
    g = out;
  }
  // dJ/dT of all layers from the partials of every segment, in one reduction
  return reduce_raw(N, L, B, geometry, dT, 0, ws_bwd, wsb_bwd, stream);
}

int mg_fma_probe(float* sink, int blocks, int threads, int iters, void* stream) {
  g_err.clear();
  if (!sink || blocks < 1 || threads < 32 || threads > 1024 || iters < 1) return fail(MG_E_ARG, "bad probe arguments");
  fma_probe_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(sink, iters, 0.999f);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "fma_probe launch");
}

int mg_trig_check(const double* x, double* out, int n, void* stream) {
  g_err.clear();
  if (!x || !out || n < 0) return fail(MG_E_ARG, "bad trig check arguments");
  if (n == 0) return MG_OK;
  trig_check_kernel<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, out, n);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "trig_check launch");
}

int mg_fma2_probe(float* sink, int blocks, int threads, int iters, void* stream) {
  g_err.clear();
  if (!sink || blocks < 1 || threads < 32 || threads > 1024 || iters < 1) return fail(MG_E_ARG, "bad probe arguments");
  fma2_probe_kernel<<<blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(sink, iters, 0.999f);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MG_OK : cuda_fail(e, "fma2_probe launch");
}

}  // extern "C"
