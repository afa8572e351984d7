/* meshes_gb300.h - C ABI of the GB300 mesh-propagation library (libmeshes_gb300.so).
 *
 * Plain C: raw device pointers, sizes and a cudaStream_t (passed as void*).  Every entry point is
 * asynchronous on `stream`, returns 0 on success and a negative MG_E* code when an argument is
 * rejected before anything is launched; mg_last_error() then names the problem.  Kernels record
 * run-time faults (a malformed geometry array, a wait that ran past its time limit) in the status
 * word at the start of the workspace; mg_read_status() fetches it.
 *
 * Fields follow the reference GPU API (gpu/mesh.py:147-174): B vectors of N modes, vector b at
 * u + b*ldu (the reference's (N, B) Fortran-order arrays); complex64 (float2) for the mzi and sym
 * crossings, float32 for orth.  Parameters follow the reference grid (gpu/mesh.py:77-81):
 * p[l*ldp + q*n_p + k] for layer l < L, slot q < N/2 and k < n_p (mzi/sym: n_p = 2 (theta, phi),
 * orth: n_p = 1); splitter errors s[l*lds + q*n_s + k] (mzi: n_s = 2 (alpha, beta), sym: 1) or NULL
 * for ideal splitters.  Geometry arrays are device int32 arrays of length L: lens/shifts for
 * nearest-neighbour meshes (Clements, Reck, ...), strides (log2 of the stride) for butterfly meshes.
 *
 * Limits: N even, 2 <= N <= 640 for nearest-neighbour meshes (the reference's own limit,
 * gpu/mesh.py:83) and N a power of two <= 512 for butterfly meshes; ldu >= N and even; u pointers
 * 16-byte aligned (complex) or 8-byte aligned (real).
 */
#ifndef MESHES_GB300_H
#define MESHES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* crossings (gpu/mesh.py:66-73) */
#define MG_MZI 0
#define MG_SYM 1
#define MG_ORTH 2
#define MG_GENERIC 3

/* operations and geometries */
#define MG_OP_FWD 0
#define MG_OP_FWDDIFF 1
#define MG_OP_BWD 2
#define MG_OP_FWD_BWDTILES 3   /* mg_propagate only: forward reading back-propagation tiles */
#define MG_OP_BWD_STORED 4     /* back-propagation from stored layer inputs (lossy crossings) */
#define MG_GEO_NN 0
#define MG_GEO_FFT 1
/* OR-ed into a geometry: the mesh has permutations between layers (mg_build_perms).  Plans made with
 * it reserve the permutation tables in the workspace and a gather scratch in shared memory. */
#define MG_GEO_PERM 4

/* return codes */
#define MG_OK 0
#define MG_E_ARG (-1)         /* invalid argument (see mg_last_error) */
#define MG_E_WORKSPACE (-2)   /* workspace missing or too small */
#define MG_E_CUDA (-3)        /* a CUDA runtime call failed */
#define MG_E_CONFIG (-4)      /* no kernel instantiated for the requested tile configuration */

/* run-time status codes (mg_read_status) */
#define MG_ST_OK 0
#define MG_ST_TIMEOUT 1       /* a shared-memory pipeline wait ran past its time limit */
#define MG_ST_BAD_GEOMETRY 2  /* lens/shifts/strides place MZIs outside the N modes */
#define MG_ST_BAD_WORK 3      /* batched launch: malformed work item */

/* Tile configuration of one launch: modes per lane M (2..16), vectors per lane V, warps per CTA W,
 * layers per pipeline stage CL, pipeline stages S.  Zero fields are filled by the built-in
 * heuristic; the autotuner (mg_autotune, driven by meshes_gb300/autotune.py) measures better choices. */
typedef struct mg_config {
  int M, V, W, CL, S;
  int split;   /* 0: automatic, 1: two CTA kinds per SM (V and V-1 vectors per lane group), 2: uniform CTAs */
} mg_config;

/* ---- library ---------------------------------------------------------------------------- */

/* Last argument error of the calling thread (empty string if none). */
const char* mg_last_error(void);

/* Library version string. */
const char* mg_version(void);

/* Bytes of workspace an entry point needs for (op, N, L, B, crossing, geometry) with config cfg
 * (NULL = heuristic).  The workspace is caller-allocated device memory, 256-byte aligned; its first
 * 256 bytes hold the status word. */
size_t mg_workspace_bytes(int op, int N, int L, int B, int crossing, int geometry, const mg_config* cfg);

/* Zero the status word of a freshly allocated workspace. */
int mg_workspace_init(void* workspace, size_t workspace_bytes, void* stream);

/* Synchronise `stream`, return the workspace's status word (MG_ST_*), clear it if `clear`. */
int mg_read_status(void* workspace, int clear, void* stream);

/* Register a measured configuration for (op, crossing, geometry, N) and batch sizes B in [B_lo, B_hi];
 * calls that pass no config then use it instead of the heuristic.  cfg = NULL removes the entries of
 * that (op, crossing, geometry, N) (N = 0: all N).  Filled by meshes_gb300.autotune. */
int mg_set_tuned(int op, int crossing, int geometry, int N, int B_lo, int B_hi, const mg_config* cfg);

/* Autotuner: time the tile configurations of (op in {MG_OP_FWD, MG_OP_FWDDIFF, MG_OP_BWD}, N, L, B, crossing,
 * geometry) on the caller's mesh (lens/shifts or strides, p/ldp, s/lds: device pointers as for
 * mg_build_tiles) and return the fastest in *best (its median time in *best_ms).  Stage 1 varies the
 * register blocking and CTA width (M, V, W); stage 2 varies layers per stage and stages (CL, S) around the
 * winner and, for forward propagation, the split launch.  Each candidate: tiles built once, two warm-up
 * launches, `reps` launches timed with CUDA events, the L2 flushed (256 MB write) before each; candidates
 * whose launches fail or record a kernel status are dropped.  Allocates its scratch stream-ordered, frees it
 * and synchronises the stream before returning.  record != 0 registers the winner for batch size B
 * (mg_set_tuned).  tried / tried_ms (may be NULL) receive up to max_tried timed candidates; *n_tried (may
 * be NULL) their count. */
int mg_autotune(int op, int N, int L, int B, int crossing, int geometry, const int* lens, const int* shifts,
                const int* strides, const float* p, int ldp, const float* s, int lds, int reps, int record,
                mg_config* best, float* best_ms, mg_config* tried, float* tried_ms, int max_tried, int* n_tried,
                void* stream);

/* The configuration the heuristic picks (filled into *out). */
int mg_default_config(int op, int N, int B, int crossing, mg_config* out);

/* ---- reference-shaped entry points ---------------------------------------------------------
 * Each replaces one CuPy RawKernel launch of the reference: coefficient precompute and the
 * propagation kernel run back to back on `stream`. */

/* Forward propagation u_out = U u_in.  Replaces fwdprop_N{N}_{X} (gpu/fwdprop.cu:25-27, launched at
 * gpu/mesh.py:158-164).  u_in == u_out is allowed. */
int mg_fwdprop(int N, int L, int B, const int* lens, const int* shifts, const float* p, int ldp, const float* s,
               int lds, const void* u_in, void* u_out, int ldu, int crossing, void* workspace,
               size_t workspace_bytes, void* stream);

/* Same for butterfly meshes: replaces fwdprop_ft_N{N}_{X} (gpu/fwdprop.cu with FFT=1, gpu/mzi_ft.cu:15-47). */
int mg_fwdprop_ft(int N, int L, int B, const int* strides, const float* p, int ldp, const float* s, int lds,
                  const void* u_in, void* u_out, int ldu, int crossing, void* workspace, size_t workspace_bytes,
                  void* stream);

/* Forward-mode derivative along dp: (u_out, du_out) = (U u_in, dU u_in + U du_in); du_in may be NULL
 * (zero).  Replaces fwddiff_N{N}_{X} (gpu/fwddiff.cu:24-27, launched at gpu/mesh.py:166-174). */
int mg_fwddiff(int N, int L, int B, const int* lens, const int* shifts, const float* p, const float* dp, int ldp,
               const float* s, int lds, const void* u_in, const void* du_in, void* u_out, void* du_out, int ldu,
               int crossing, void* workspace, size_t workspace_bytes, void* stream);
int mg_fwddiff_ft(int N, int L, int B, const int* strides, const float* p, const float* dp, int ldp, const float* s,
                  int lds, const void* u_in, const void* du_in, void* u_out, void* du_out, int ldu, int crossing,
                  void* workspace, size_t workspace_bytes, void* stream);

/* Back-propagation from the outputs: given u_out and dJdu_out (= 2 dJ/du_out*, the reference's
 * convention, gpu/mesh.py:176-181), reconstruct u_in (may be NULL), write dJdu_in = U^H dJdu_out and
 * dp = dJ/dp in the parameter grid layout.  accumulate = 0 overwrites dp (deterministic; inactive
 * slots get 0), accumulate = 1 adds to it as the reference's atomics do (the reference zeroes dp
 * first, gpu/mesh.py:214).  Replaces backdiff_N{N}_{X} (gpu/backdiff.cu:24-27, launched at
 * gpu/mesh.py:227-231).  Valid for unitary crossings (mzi, sym, orth). */
int mg_backdiff(int N, int L, int B, const int* lens, const int* shifts, const float* p, float* dp, int ldp,
                const float* s, int lds, const void* u_out, const void* dJdu_out, void* u_in, void* dJdu_in, int ldu,
                int crossing, int accumulate, void* workspace, size_t workspace_bytes, void* stream);
int mg_backdiff_ft(int N, int L, int B, const int* strides, const float* p, float* dp, int ldp, const float* s,
                   int lds, const void* u_out, const void* dJdu_out, void* u_in, void* dJdu_in, int ldu, int crossing,
                   int accumulate, void* workspace, size_t workspace_bytes, void* stream);

/* Forward propagation like mg_fwdprop (nearest-neighbour geometry), for callers that cannot allocate
 * device memory - plugin hosts that forbid allocations, loops that must not touch an allocator - and so
 * cannot provide a workspace.  No counterpart in the
 * reference.  The scratch is an 8 MiB array compiled into the library (held on every GPU that loads
 * it until exit); problems needing more return MG_E_WORKSPACE without launching.  The first call on
 * each device looks up the array's device address.  All
 * calls share the array, so calls that overlap on the GPU race: serialise them.  Kernel status codes
 * are not reported by this entry point.  The array's address is cached per device for the life of the
 * process: do not call it again after cudaDeviceReset re-creates the device's context. */
int mg_fwdprop_noalloc(int N, int L, int B, const int* lens, const int* shifts, const float* p, int ldp,
                       const float* s, int lds, const void* u_in, void* u_out, int ldu, int crossing, void* stream);

/* ---- programmed-mesh entry points (coefficients kept resident between calls) -----------------
 * mg_build_tiles runs only the coefficient precompute of `op` into the workspace; mg_propagate runs
 * only the propagation kernel on tiles built earlier with the same (op, N, L, crossing, geometry,
 * cfg).  Used by the autograd function, the batched engine and the server, which re-use one set of
 * tiles across many batches.  Tgen/Dgen (crossing MG_GENERIC) give T per slot as 4 complex64
 * (t00, t01, t10, t11) and, for op MG_OP_BWD, dT/dp0 and dT/dp1 (8 complex64). */
int mg_build_tiles(int op, int N, int L, int geometry, const int* lens, const int* shifts, const int* strides,
                   int crossing, const float* p, int ldp, const float* s, int lds, const float* dp, const void* Tgen,
                   const void* Dgen, int B, const mg_config* cfg, void* workspace, size_t workspace_bytes, void* stream);

/* op MG_OP_FWD_BWDTILES runs the forward kernel on tiles built for MG_OP_BWD (nearest-neighbour
 * geometry), so one coefficient pass serves a forward propagation and its back-propagation. */
int mg_propagate(int op, int N, int L, int B, int crossing, int geometry, const void* in0, const void* in1, void* out0,
                 void* out1, int ldu, float* dp, int ldp, int accumulate, const mg_config* cfg, void* workspace,
                 size_t workspace_bytes, void* stream);

/* Test entry point for the bounded-wait failure path: mg_propagate (op MG_OP_FWD or MG_OP_BWD, nearest-neighbour
 * geometry, tiles built by mg_build_tiles for the same shape, no dp) with every pipeline wait limited to wait_ns
 * and the coefficient copy of pipeline chunk `unarmed_chunk` never issued.  Every CTA gives up at that chunk:
 * it records MG_ST_TIMEOUT in the workspace status word, waits (within the same limit) for the copies it did
 * issue, releases its barriers and returns, leaving the outputs incomplete.  Nothing stays in flight and the
 * context stays usable; the next call on the workspace (after mg_read_status clears the status) runs normally.
 * No counterpart in the reference (its kernels have no time limit). */
int mg_propagate_wait_test(int op, int N, int L, int B, int crossing, const void* in0, const void* in1, void* out0,
                           void* out1, int ldu, unsigned long long wait_ns, int unarmed_chunk, void* workspace,
                           size_t workspace_bytes, void* stream);

/* ---- permutations between layers (the reference's StructuredMeshNetwork.perm, mesh.py:238-277, applied
 * as c/dot.cpp:29-40,150-153,289-292 does; its GPU API forbids them, mesh.py:573) ---------------------
 * With geometry | MG_GEO_PERM, mg_build_perms writes the gather tables of `perms` into a workspace planned
 * for the same (op, N, L, B, crossing, geometry, cfg): perms is (L+1) x N int32 on the device, row l
 * gathered before layer l and row L after the last layer (new[q] = old[perms[l][q]]), or NULL for none.
 * Call it after mg_build_tiles (which resets the tables to the identity on such a workspace).
 * Every later mg_propagate on that workspace applies them; back-propagation goes through the inverse
 * permutations in reverse order (the reference's perms_bk, mesh.py:382).  A row that is not a permutation
 * of 0..N-1 records MG_ST_BAD_GEOMETRY and acts as the identity.  Permuted meshes run their own kernel
 * instantiations (runtime lane groups, default V per (op, M), no split launch, at most 4096 layers); layer
 * ranges, stored activations, the batched engine and the server take no permutations. */
int mg_build_perms(int op, int N, int L, int B, int crossing, int geometry, const int* perms, const mg_config* cfg,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Plan of one launch (for hosts that manage tiles themselves, e.g. the batched engine). */
typedef struct mg_plan_info {
  int M, V, W, CL, S, G, grid;
  int nA;   /* split launch: CTAs holding V vectors per lane group (the other grid - nA hold V-1); 0 if uniform */
  unsigned layer_bytes, dlayer_bytes;
  size_t smem, off_kinds, off_tiles, off_dtiles, off_partial, total;
} mg_plan_info;
int mg_plan(int op, int N, int L, int B, int crossing, int geometry, const mg_config* cfg, mg_plan_info* out);

/* ---- batched meshes: one persistent launch over a (mesh, batch-tile) work queue ----------------
 * Each mesh's coefficient tiles are built beforehand with mg_build_tiles into its own workspace, with
 * the tile configuration of its kernel class and W = 8 (the persistent CTA width):
 *   MG_BCLS_C8  : complex64, M = 8,  N <= 256   (fwd V = 4, bwd V = 4, mzi)
 *   MG_BCLS_C16 : complex64, M = 16, N <= 512   (fwd V = 2, bwd V = 2, mzi)
 *   MG_BCLS_R8  : float32,   M = 8,  N <= 256   (fwd V = 4, bwd V = 4, orth)
 * Work items cover vectors [v0, vend) of one mesh; CTAs take items from a device counter (`head`,
 * zeroed by the caller before each launch, e.g. a memset node of a captured CUDA graph) in array
 * order, so items sorted longest-first balance the load.  Back-propagation items write partials
 * at mesh.partial + part * L * Np/2 (float2); mg_batched_reduce sums them in order into mesh.dp. */
/* OR-ed into mg_batched_propagate's op: every mesh of the launch is nearest-neighbour (lens/shifts), so
 * the launch runs the kernel bodies without strided layers (fewer registers); an item whose mesh has
 * another layer kind records MG_ST_BAD_GEOMETRY and is skipped. */
#define MG_BATCH_NN 16
/* OR-ed into mg_batched_propagate's op: every item's mesh is of kernel class cls, and the launch runs only that
 * class's body, with its own register budget; an item of another class records MG_ST_BAD_WORK and is skipped. */
#define MG_BATCH_ONLY(cls) (((cls) + 1) << 8)
/* OR-ed with MG_BATCH_ONLY(MG_BCLS_C8) or MG_BATCH_ONLY(MG_BCLS_R8): every item's mesh has G = 32 lanes per
 * vector (N in (128, 256]); the launch runs a body compiled for that lane group. */
#define MG_BATCH_FULL_WARP 32
#define MG_BCLS_C8 0
#define MG_BCLS_C16 1
#define MG_BCLS_R8 2
typedef struct mg_batch_mesh {
  int N, L, B, ldu;
  int cls, G, CL, S;
  unsigned layer_bytes;
  int n_items, ldp, n_p;
  const void* tiles;     /* workspace + off_tiles of the mesh's mg_build_tiles */
  const int* kinds;      /* workspace + off_kinds */
  const void* in0;       /* fwd: x; bwd: y */
  const void* in1;       /* bwd: dJ/dy* */
  void* out0;            /* fwd: y; bwd: x (may be NULL) */
  void* out1;            /* bwd: dJ/dx* */
  float* dp;             /* bwd: dJ/dp (L, N/2, n_p), overwritten by mg_batched_reduce */
  void* partial;         /* bwd: n_items * L * Np/2 float2 */
} mg_batch_mesh;
typedef struct mg_batch_item {
  int mesh, v0, vend, part;
} mg_batch_item;

/* Persistent launch of `grid` CTAs of 256 threads with `smem` bytes of dynamic shared memory (the
 * maximum mg_plan_info.smem of the meshes' W = 8 plans).  op is MG_OP_FWD or MG_OP_BWD.  Kernel
 * status (bad work item, expired wait) goes to *status (device int, zeroed by the caller). */
int mg_batched_propagate(int op, const mg_batch_mesh* meshes, int n_meshes, const mg_batch_item* items, int n_items,
                         int* head, int grid, size_t smem, int* status, void* stream);
/* Deterministic sum of the back-propagation partials of every mesh into its dp. */
int mg_batched_reduce(const mg_batch_mesh* meshes, int n_meshes, void* stream);

/* Back-propagation with the L2 loss to a target fused into the kernel: dJ/dy* = 2 (y - target) is
 * formed on load (J = sum |y - target|^2), then as mg_propagate(MG_OP_BWD) with tiles built earlier.
 * The reference computes this gradient in a separate pass (gpu/mesh.py:176-181, 219-221). */
int mg_propagate_l2(int N, int L, int B, int crossing, int geometry, const void* y, const void* target, void* x_out,
                    void* g_out, int ldu, float* dp, int ldp, int accumulate, const mg_config* cfg, void* workspace,
                    size_t workspace_bytes, void* stream);

/* ---- serving: native continuous-batching scheduler over resident meshes ------------------------
 * The meshes' tiles are built beforehand (mg_build_tiles, W = 8 persistent configuration of their kernel
 * class, both ops) and stay resident.  A scheduler thread owned by the server packs queued requests
 * into ticks (admission by free space in a fixed device arena), runs one persistent forward launch
 * per tick and, for gradient requests, one persistent back-propagation launch and reduction, and
 * copies results into the caller's buffers; tags of finished requests come back from mg_server_wait.
 * Inputs and outputs are host memory owned by the caller until the request's tag is returned. */
typedef struct mg_server_mesh {
  int N, L, cls, G, n_p, cap;          /* cls MG_BCLS_*; cap = vectors per work item (8 x 32/G x V) */
  int fwd_CL, fwd_S, bwd_CL, bwd_S;
  unsigned fwd_layer_bytes, bwd_layer_bytes;
  const void* fwd_tiles;
  const int* fwd_kinds;
  const void* bwd_tiles;
  const int* bwd_kinds;
} mg_server_mesh;
typedef struct mg_server mg_server;
/* NULL on error (mg_last_error).  grid: persistent CTAs (the SM count); smem_*: the largest mg_plan_info.smem
 * of the meshes' W = 8 plans per op. */
mg_server* mg_server_create(const mg_server_mesh* meshes, int n_meshes, size_t arena_bytes, int n_streams,
                            int max_per_tick, int grid, size_t smem_fwd, size_t smem_bwd, int device);
/* Device bytes a request needs (admission accounting). */
int mg_server_request_bytes(const mg_server* s, int mesh, int b, int grad, size_t* out);
/* Queue a request: x (b, N) complex64 (float32 for orth), y (b, N) receives U x; with gy (b, N) = 2 dJ/dy*,
 * dp (L, N/2, n_p) float32 receives dJ/dp and gx (b, N) receives 2 dJ/dx*.  MG_E_WORKSPACE if it can
 * never fit the arena. */
int mg_server_submit(mg_server* s, int mesh, int b, const void* x, const void* gy, void* y, float* dp, void* gx,
                     unsigned long long tag);
/* Up to max completed tags (waits up to timeout_us for the first); < 0 once the server has failed. */
int mg_server_wait(mg_server* s, unsigned long long* tags, int max, int timeout_us);
/* out[0] completed requests, out[1] ticks, out[2] queued requests. */
int mg_server_stats(mg_server* s, long long* out);
/* Kernel status word of the server's launches (synchronous read; 0 = ok). */
int mg_server_status(mg_server* s);
/* Stop: with drain, finish queued and in-flight requests first; then free everything. */
void mg_server_destroy(mg_server* s, int drain);

/* ---- lossy meshes: layer ranges and stored activations ----------------------------------------
 * The reference back-propagates by inverting each layer with T^H (c/dot.cpp:75-80, gpu/backprop.cu),
 * which is exact only for unitary crossings; for lossy ones (crossing.py:444-508, gains g_ij) that
 * gradient is wrong.  These calls back-propagate from stored layer inputs instead, for checkpointed
 * adjoints that keep one input every ~sqrt(L) layers and recompute the rest segment by segment.
 * Both run layers [l0, l1) of tiles built earlier by mg_build_tiles for the same (N, L, B, crossing,
 * geometry, cfg): op MG_OP_FWD with tiles of MG_OP_FWD, op MG_OP_BWD_STORED with tiles of
 * MG_OP_BWD_STORED (complex crossings only; MG_GENERIC takes T per slot from Tgen and needs no Dgen).
 *   MG_OP_FWD:        in0 = input of layer l0, out0 = output of layer l1-1 (may be NULL); when act is
 *                     not NULL the input of every layer l of the range is also written to
 *                     act + (l - l0) * B * ldu (complex64 elements).
 *   MG_OP_BWD_STORED: act holds those inputs; in1 = 2 dJ/du* at the output of layer l1-1, out1 =
 *                     2 dJ/du* at the input of layer l0; dT (complex64 [L][N/2][2][2], same slot grid
 *                     as Tgen) receives, for the layers of the range, sum_b g_i conj(x_j) = 2 dJ/dT_ij*
 *                     (0 on inactive slots), overwritten or, with accumulate, added. */
int mg_propagate_range(int op, int N, int L, int l0, int l1, int B, int crossing, int geometry, const void* in0,
                       const void* in1, void* out0, void* out1, int ldu, void* act, void* dT, int accumulate,
                       const mg_config* cfg, void* workspace, size_t workspace_bytes, void* stream);

/* ---- phase screen (the reference's is_phase / phi_pos, c/dot.cpp:97-143; its GPU API forbids it) -----
 * mg_phase_screen: u_out = exp(i sgn ph) u_in elementwise per mode (ph: N floats; fields complex64 (B, N)
 * with leading dimension ldu; u_out may alias u_in); with du_out, also du_out = exp(i sgn ph) du_in +
 * i dph u_out (du_in and dph may be NULL = 0), the forward-mode derivative of the screen.
 * mg_phase_screen_grad: dph[k] (= or, with accumulate, +=) sum_b Re(conj(g_bk) i u_bk) for the field u
 * after the screen and g = 2 dJ/du* there; deterministic. */
int mg_phase_screen(int N, int B, const float* ph, const float* dph, int sgn, const void* u_in, void* u_out,
                    const void* du_in, void* du_out, int ldu, void* stream);
int mg_phase_screen_grad(int N, int B, const void* u, const void* g, int ldu, float* dph, int accumulate,
                         void* stream);

/* The whole checkpointed adjoint of a generic (lossy) mesh in two calls (tiles of MG_OP_FWD in ws /
 * ws_fwd, of MG_OP_BWD_STORED in ws_bwd; complex64 fields with leading dimension ldu).
 * mg_lossy_forward: y = U x by segments of `seg` layers, keeping the input of every segment after the
 * first in ckpt ([ceil(L/seg) - 1][B][ldu]).
 * mg_lossy_backward: from x, ckpt and gy = 2 dJ/dy*: gx = 2 dJ/dx*, and dT (complex64 [L][N/2][2][2]) =
 * sum_b g_i conj(x_j) per slot; segments in reverse, each recomputed into act ([seg][B][ldu]) and
 * back-propagated from it; gtmp is a (B, ldu) scratch field. */
int mg_lossy_forward(int N, int L, int B, int geometry, int seg, const void* x, void* y, void* ckpt, int ldu, void* ws,
                     size_t ws_bytes, void* stream);
int mg_lossy_backward(int N, int L, int B, int geometry, int seg, const void* x, const void* ckpt, const void* gy,
                      void* gx, void* gtmp, void* act, void* dT, int ldu, void* ws_fwd, size_t ws_fwd_bytes,
                      void* ws_bwd, size_t ws_bwd_bytes, void* stream);

/* Lossy generic MZI (crossing.py:444-488) on the device, double precision, one thread per slot:
 * mg_generic_mzi_T: T (complex64, n x [t00, t01, t10, t11]) from p (n x (theta, phi)) and s (n x 14:
 * alpha, beta, 4 fabrication and 4 crosstalk phase errors, 4 log-gains; NULL = 0).
 * mg_generic_mzi_T_vjp: dp (n x 2) = Re sum_ij conj(G_ij) dT_ij/dp for G = 2 dJ/dT* (complex64 n x 4). */
int mg_generic_mzi_T(int n, const double* p, const double* s, void* T, void* stream);
int mg_generic_mzi_T_vjp(int n, const double* p, const double* s, const void* gT, double* dp, void* stream);

/* ---- self-configuration ----------------------------------------------------------------------
 * The nulling pass of the matrix-diagonalisation method (reference configure.py:187-330, diag and its
 * diagHelper_fn), host code in double precision.  U (target), Z (product of the meshes' matrices at their
 * starting phases), VdV and WWd (identity on entry) are N x N complex128 row-major, updated in place and returned
 * in the transposed-or-not form the reference's pass leaves them in.  ijzp: K steps (i, j, ind, p) - zero
 * element (i, j) with MZI ind of the left (p = 0, n1 MZIs) or right (p = 1, n2 MZIs) mesh; s1/s2 (n x 2)
 * splitting errors, c1/c2 (n x 2) (theta, phi) updated in place; type 0 = MZI crossing, 1 = its flipped form
 * (phase shifter at the output); init (K x 2) line-search starting points; noise (K x 2) added to each
 * programmed MZI, or NULL; improved selects the reference's improved updates.  Returns MG_E_ARG (nothing
 * changed) when a step points outside the matrices or meshes.  Does not touch the GPU. */
int mg_diag_configure(int N, int K, void* U, void* Z, void* VdV, void* WWd, int n1, const double* s1, double* c1,
                      int type1, int n2, const double* s2, double* c2, int type2, const int* ijzp, const double* init,
                      const double* noise, int improved);
/* The direct method (reference configure.py:333-410, direct(m, U, 'down') and its directHelper_fn) for a
 * nearest-neighbour mesh of output-phase MZIs (MZICrossingOutPhase) with its phase screen at the input: L layers
 * (lens, shifts), U the N x N complex128 row-major target, s (n_cr x 2) splitting errors and p (n_cr x 2)
 * (theta, phi) in the reference's flat crossing order (layer by layer, top to bottom); p is written in place
 * (crossings outside every diagonal keep their values) and phi_out (N) receives the input screen.  dk_max as the
 * reference's (1, or 2 for some divided Clements rectangles).  Returns MG_E_ARG when the geometry is invalid or two
 * diagonals share an input mode.  Host code; does not touch the GPU. */
int mg_direct_configure(int N, int L, const int* lens, const int* shifts, const void* U, const double* s, double* p,
                        double* phi_out, int dk_max);

/* ---- training ------------------------------------------------------------------------------- */

/* One Adam step (Kingma and Ba 2015, with bias correction) over n float32 parameters p with gradient g and
 * moments m, v (device arrays, updated in place), in one launch on `stream`.  state is a device int[2], zeroed
 * before the first step: state[0] counts the steps taken (the kernel advances it), state[1] is the kernel's own
 * block counter.  lr, the betas, their complements 1 - beta and eps enter the float arithmetic rounded from
 * double.  The step count on the device lets a CUDA graph record the update.  No counterpart in the
 * reference, whose training loops use an external optimizer. */
int mg_adam_step(float* p, const float* g, float* m, float* v, int n, double lr, double beta1, double beta2, double eps,
                 int* state, void* stream);

/* ---- measurement helpers -------------------------------------------------------------------- */

/* FP32 FMA throughput probe: `blocks` x `threads` threads each run `iters` iterations of 64
 * independent FMAs; writes one float per thread to `sink`.  Used by bench.py to measure the FP32
 * CUDA-core peak of the device it runs on. */
int mg_fma_probe(float* sink, int blocks, int threads, int iters, void* stream);
/* Self-check of the coefficient precompute's double-precision sin/cos: out[6i..6i+5] = the differences
 * (sin, cos)(x[i]) own - library for the full-precision version, the tile-precision version (results rounded
 * to float32) and the small-angle version used for splitting errors, for n device doubles x (used by the
 * tests). */
int mg_trig_check(const double* x, double* out, int n, void* stream);
/* The same probe with packed FP32 pairs (fma.rn.f32x2, sm_100+): 128 FMAs per thread-iteration. */
int mg_fma2_probe(float* sink, int blocks, int threads, int iters, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MESHES_GB300_H */
