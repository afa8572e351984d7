// Warp-pair back-propagation: one vector spread over the 64 lanes of two warps.
//
// A plan with M = 8 modes per lane and a full warp per vector (G = 32, N in (128, 256]) stores its coefficient
// tiles and gradient partials for 32 lanes of 8 modes.  The warp-pair launch reads the same tiles and writes the
// same partials, but gives each lane 4 modes: virtual lane jv in [0, 64) of a pair (32 per warp) owns modes
// [4*jv, 4*jv + 4), and the pair holds V vectors.  With V = 7 a pair carries 3.5 vectors per warp, so every SM
// scheduler (two warps) carries 7 vectors: at N = 256, B = 4096 the 147 CTAs of 4 pairs leave one scheduler
// in 27 idle, where warps of 4 whole vectors (8 per scheduler) fill only 128 of the 152 SMs.
//
// Index map onto the M = 8 plan: slot q = 2*jv + e4 (e4 in {0, 1}) is the plan's entry e8 = 2*(jv & 1) + e4
// of plan lane j32 = jv >> 1, so crossing() is called with (e8, G = 32, j32) and finds the tile rows, the
// splitter coefficients and the staging position of the plan.  Lane L of warp h holds virtual lane
// jv = 32*h + 2*(L & 15) + (L >> 4): lanes 0-15 the even, lanes 16-31 the odd virtual lanes, so that each
// half-warp reads (and stages) one contiguous run of the plan's rows - with consecutive lanes on
// consecutive virtual lanes, lanes 2k and 2k+1 would hit the same banks 2 KB apart on every load.  The
// neighbouring virtual lanes are then lanes L + 16 / L - 15 (next) and L - 16 / L + 15 (previous), reached
// with indexed shuffles.
//
// Odd-shift layers couple mode 3 of lane jv with mode 0 of lane jv + 1.  Inside a warp this is the shuffle
// pair of layer_mis.  Across the pair boundary (lane 31 of warp 0, lane 0 of warp 1) both lanes compute that
// one crossing: warp 0 lanes each compute (own 3, next 0) and warp 1 lanes each compute (previous 3, own 0),
// so every lane still runs two crossings per layer, and the two boundary lanes exchange their boundary modes
// through shared memory once per odd layer (a named barrier over the pair's 64 threads, double-buffered
// slots).  Both compute bitwise the same crossing; warp 0 stages its gradient.  Lane 31 of warp 1 stages
// zero for the plan's last odd-layer slot, the one nobody computes (modes N-1 and N: outside every mesh).
//
// Gradient staging is shared by the two warps of a pair (each slot position written by exactly one of them),
// and the chunk reduction sums the W/2 pair regions in a fixed order, as the one-warp launch sums its warps.
#pragma once
#include "mg_prop.cuh"

namespace mg {

// virtual lane of lane L in warp h of a pair, and the lanes holding the next / previous virtual lane
__device__ __forceinline__ int pair_jv(int h, int lane) { return 32 * h + 2 * (lane & 15) + (lane >> 4); }
__device__ __forceinline__ int pair_next_lane(int lane) { return lane < 16 ? lane + 16 : lane - 15; }
__device__ __forceinline__ int pair_prev_lane(int lane) { return lane >= 16 ? lane - 16 : lane + 15; }
__device__ __forceinline__ float2 shfl_idx(float2 v, int src) {
  return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// named barrier over the two warps of pair `pair` (barrier 0 is __syncthreads)
__device__ __forceinline__ void pair_sync(int pair) {
  asm volatile("bar.sync %0, 64;" ::"r"(1 + pair) : "memory");
}

// aligned layer: crossings (0, 1) and (2, 3) of the lane
template <int OP, int V, typename F>
__device__ __forceinline__ void pair_local(const float4* tl, int jv, F (&u)[V][4], F (&w)[V][4], float4* gl) {
  const int j32 = jv >> 1, eb = 2 * (jv & 1);
#pragma unroll
  for (int e = 0; e < 2; ++e)
    crossing<OP, 8, V, false, 1, true>(
        tl, 0, eb + e, 32, j32, 0, [&](int v) -> F& { return u[v][2 * e]; },
        [&](int v) -> F& { return u[v][2 * e + 1]; }, [&](int v) -> F& { return w[v][2 * e]; },
        [&](int v) -> F& { return w[v][2 * e + 1]; }, gl);
}

// odd-shift layer: inner crossing (1, 2) and the boundary crossing with the neighbouring lane
template <int OP, int V, typename F>
__device__ __forceinline__ void pair_mis(const float4* tl, int h, int lane, F (&u)[V][4], F (&w)[V][4], float4* gl,
                                         F* mine, const F* theirs, int pair) {
  const int jv = pair_jv(h, lane);
  const int nxt = pair_next_lane(lane), prv = pair_prev_lane(lane);
  const int j32 = jv >> 1, eb = 2 * (jv & 1);
  // publish the boundary modes for the other warp of the pair
  if (h == 0 && lane == 31) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      mine[v] = u[v][3];
      mine[V + v] = w[v][3];
    }
  }
  if (h == 1 && lane == 0) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      mine[v] = u[v][0];
      mine[V + v] = w[v][0];
    }
  }
  pair_sync(pair);
  F nb[V], nbw[V];   // the neighbour's boundary mode: next lane's mode 0 (warp 0) or previous lane's mode 3 (warp 1)
  if (h == 0) {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      nb[v] = shfl_idx(u[v][0], nxt);
      nbw[v] = shfl_idx(w[v][0], nxt);
    }
    if (lane == 31) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        nb[v] = theirs[v];
        nbw[v] = theirs[V + v];
      }
    }
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) {
      nb[v] = shfl_idx(u[v][3], prv);
      nbw[v] = shfl_idx(w[v][3], prv);
    }
    if (lane == 0) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        nb[v] = theirs[v];
        nbw[v] = theirs[V + v];
      }
    }
  }
  // inner crossing (1, 2): plan entry eb of lane j32
  crossing<OP, 8, V, false, 1, true>(
      tl, 0, eb, 32, j32, 0, [&](int v) -> F& { return u[v][1]; }, [&](int v) -> F& { return u[v][2]; },
      [&](int v) -> F& { return w[v][1]; }, [&](int v) -> F& { return w[v][2]; }, gl);
  if (h == 0) {
    // (own 3, next 0): plan entry eb + 1 of lane j32
    crossing<OP, 8, V, false, 1, true>(
        tl, 0, eb + 1, 32, j32, 0, [&](int v) -> F& { return u[v][3]; }, [&](int v) -> F& { return nb[v]; },
        [&](int v) -> F& { return w[v][3]; }, [&](int v) -> F& { return nbw[v]; }, gl);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const F bu = shfl_idx(nb[v], prv), bw = shfl_idx(nbw[v], prv);
      if (lane != 0) {
        u[v][0] = bu;
        w[v][0] = bw;
      }
    }
  } else {
    // (previous 3, own 0): the entry of virtual lane jv - 1; lane 0 computes warp 0's boundary slot again
    // and leaves its gradient to warp 0
    const int jp = jv - 1;
    crossing<OP, 8, V, false, 1, true>(
        tl, 0, 2 * (jp & 1) + 1, 32, jp >> 1, 0, [&](int v) -> F& { return nb[v]; },
        [&](int v) -> F& { return u[v][0]; }, [&](int v) -> F& { return nbw[v]; }, [&](int v) -> F& { return w[v][0]; },
        gl, lane != 0);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const F bu = shfl_idx(nb[v], nxt), bw = shfl_idx(nbw[v], nxt);
      if (lane != 31) {
        u[v][3] = bu;
        w[v][3] = bw;
      }
    }
    if (lane == 31) reinterpret_cast<float2*>(gl)[3 * 32 + 31] = make_float2(0.f, 0.f);
  }
}

// One batch tile of one mesh by W/2 warp pairs (W = blockDim.x / 32): back-propagation (direct MZI
// gradients) of nearest-neighbour complex meshes, plan M = 8, G = 32.  Pipeline, timeout handling, fused L2
// gradient and the chunk reduction as in prop_body.
template <int V>
__device__ __forceinline__ void prop_pair_body(const PropArgs& a, unsigned char* smem) {
  using F = float2;
  constexpr int OP = OP_BWD;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int h = warp & 1, pair = warp >> 1, npair = a.W >> 1;
  const int jv = pair_jv(h, lane);
  const int np2 = 128;                       // plan slots per layer (G = 32, M = 8)
  const int vb0 = a.v0 + pair * V;

  const size_t ring_bytes = (size_t)a.S * a.CL * a.layer_bytes;
  const size_t gst_layer = (size_t)np2 * 8;
  // the plan sized W staging regions; pairs use W/2 of them and the exchange slots sit in the rest
  const size_t gst_bytes = (size_t)a.W * a.CL * gst_layer;
  unsigned char* ring = smem;
  unsigned char* gst = smem + ring_bytes;
  F* xch = reinterpret_cast<F*>(gst + (size_t)npair * a.CL * gst_layer) + (size_t)pair * 2 * 2 * 2 * V;
  uint64_t* bars = reinterpret_cast<uint64_t*>(gst + gst_bytes);
  int* skinds = reinterpret_cast<int*>(bars + a.S + 1);
  const int* kinds = a.kinds;
  if (a.L <= kMaxSmemKinds) {
    for (int l = tid; l < a.L; l += blockDim.x) skinds[l] = __ldg(a.kinds + l);
    kinds = skinds;
  }

  F u[V][4];
  F w[V][4];
  load_fields<4, V, false>(u, a.in0, vb0, a.vend, a.N, a.ldu, jv);
  if (a.target) {   // fused L2 loss to a target: g = 2 (y - t)
    load_fields<4, V, false>(w, a.target, vb0, a.vend, a.N, a.ldu, jv);
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
      for (int m = 0; m < 4; ++m) w[v][m] = l2_grad(u[v][m], w[v][m]);
  } else {
    load_fields<4, V, false>(w, a.in1, vb0, a.vend, a.N, a.ldu, jv);
  }

  const int nch = (a.L + a.CL - 1) / a.CL;
  if (tid == 0) {
    for (int s = 0; s <= a.S; ++s) mbar_init(smem_u32(bars + s), 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto chunk_lo = [&](int c) { return max(0, a.L - (c + 1) * a.CL); };
  auto chunk_hi = [&](int c) { return a.L - c * a.CL; };
  const uint64_t wlim = a.wait_ns ? a.wait_ns : kWaitLimitNs;
  auto issue = [&](int c) {
    if (c + 1 == a.unarmed) return;
    const int lo = chunk_lo(c), hi = chunk_hi(c);
    const unsigned bytes = (unsigned)(hi - lo) * a.layer_bytes;
    const uint32_t bar = smem_u32(bars + (c % a.S));
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_1d(smem_u32(ring + (size_t)(c % a.S) * a.CL * a.layer_bytes), a.tiles + (size_t)lo * a.layer_bytes,
                bytes, bar);
  };
  int issued = 0;
  if (tid == 0) {
    for (; issued < min(a.S, nch); ++issued) issue(issued);
  }
  unsigned char* gst_pair = gst + (size_t)pair * a.CL * gst_layer;
  F* x_mine = xch;
  int par = 0;
  PropArgs ar = a;
  ar.W = npair;   // the chunk reduction sums the pair regions

  for (int c = 0; c < nch; ++c) {
    const int lo = chunk_lo(c), hi = chunk_hi(c);
    const bool ok = mbar_wait_bounded(smem_u32(bars + (c % a.S)), (uint32_t)((c / a.S) & 1), wlim);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        set_status(a.status, ST_TIMEOUT);
        for (int cc = c + 1; cc < issued; ++cc)
          if (cc + 1 != a.unarmed) mbar_wait_bounded(smem_u32(bars + (cc % a.S)), (uint32_t)((cc / a.S) & 1), wlim);
        for (int s = 0; s <= a.S; ++s) mbar_inval(smem_u32(bars + s));
      }
      return;
    }
    const unsigned char* st = ring + (size_t)(c % a.S) * a.CL * a.layer_bytes;
    const int nl = hi - lo;
    int i = 0;
    while (i < nl) {
      const int l0 = hi - 1 - i;
      const float4* t0 = reinterpret_cast<const float4*>(st + (size_t)(l0 - lo) * a.layer_bytes);
      float4* g0 = reinterpret_cast<float4*>(gst_pair + (size_t)(l0 - lo) * gst_layer);
      if (kinds[l0] == KIND_MIS) {
        F* mine = x_mine + (size_t)(2 * par + h) * 2 * V;
        const F* theirs = x_mine + (size_t)(2 * par + 1 - h) * 2 * V;
        par ^= 1;
        if (i + 1 < nl && kinds[l0 - 1] == 0) {
          // fused (odd-shift, aligned) pair: one straight-line block for the compiler
          const float4* t1 = reinterpret_cast<const float4*>(st + (size_t)(l0 - 1 - lo) * a.layer_bytes);
          float4* g1 = reinterpret_cast<float4*>(gst_pair + (size_t)(l0 - 1 - lo) * gst_layer);
          pair_mis<OP, V>(t0, h, lane, u, w, g0, mine, theirs, pair);
          pair_local<OP, V>(t1, jv, u, w, g1);
          i += 2;
          continue;
        }
        pair_mis<OP, V>(t0, h, lane, u, w, g0, mine, theirs, pair);
      } else {
        pair_local<OP, V>(t0, jv, u, w, g0);
      }
      i += 1;
    }
    __syncthreads();
    chunk_reduce_direct<8, 1>(ar, kinds, lo, nl, gst, np2, 32);
    if (tid == 0 && issued < nch) issue(issued++);
  }
  if (tid == 0)
    for (int s = 0; s <= a.S; ++s) mbar_inval(smem_u32(bars + s));
  store_fields<4, V, false>(u, a.out0, vb0, a.vend, a.N, a.ldu, jv);
  store_fields<4, V, false>(w, a.out1, vb0, a.vend, a.N, a.ldu, jv);
}

template <int V>
__global__ void __launch_bounds__(256, 1) prop_pair_kernel(const PropArgs a0) {
  extern __shared__ __align__(128) unsigned char smem[];
  PropArgs a = a0;
  a.v0 = blockIdx.x * ((a.W >> 1) * V);
  a.vend = a.B;
  a.partial = a0.partial + (size_t)blockIdx.x * (a.pstride ? a.pstride : a.L) * 128;
  prop_pair_body<V>(a, smem);
}

}  // namespace mg
