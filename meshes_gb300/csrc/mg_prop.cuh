// The mesh-propagation kernel family (forward, forward-mode derivative, back-propagation).
//
// Work decomposition (one CTA = one batch tile of one mesh):
//   * a vector of N complex64 modes is held in the registers of a group of G lanes (G a power of
//     two <= 32), lane j owning the M contiguous modes [j*M, j*M+M); a warp holds R = 32/G such
//     groups and every lane holds V vectors ("register block over the batch"), so each coefficient
//     fetched from shared memory is reused V times;
//   * the per-layer coefficient tiles (precomputed by mg_coeffs.cu in the exact order lanes consume
//     them) are streamed through a ring of S shared-memory stages by 1-D bulk TMA copies
//     (cp.async.bulk + mbarrier complete_tx), CL layers per stage, issued by one thread;
//   * layer kinds: pairs inside a lane (nearest-neighbour aligned layers and butterfly strides
//     < M) need no communication; a nearest-neighbour layer with odd shift couples the last mode of
//     lane j with the first of lane j+1 (one __shfl_down / __shfl_up pair per vector); butterfly
//     strides >= M couple lane j with lane j ^ (stride/M) (one __shfl_xor per mode, each lane
//     computing its own outputs);
//   * back-propagation walks the layers in reverse from the OUTPUTS, rebuilding each layer's input
//     with T^H (lossless crossings need no stored activations, as the reference does in
//     gpu/backdiff.cu and c/dot.cpp mode 2), accumulating dJ/dT_ij = sum_b conj(g_i) x_j in
//     registers over the lane's V vectors, reducing over the R groups of a warp with __shfl_xor,
//     staging per-warp sums in shared memory and, once per chunk, summing the warps in a fixed order
//     and contracting with dT/dp into a per-CTA partial (no float atomics: bit-stable results).
//
// Reference counterparts: gpu/fwdprop.cu:25-123, gpu/fwddiff.cu:24-141, gpu/backdiff.cu:24-153,
// gpu/crossing.cu:214-333 (the 2x2 appliers) and c/dot.cpp:146-288.
#pragma once
#include <type_traits>

#include "mg_device.cuh"

namespace mg {

enum { OP_FWD = 0, OP_FWDDIFF = 1, OP_BWD = 2 };

__host__ __device__ constexpr int ilog2_const(int x) { return x <= 1 ? 0 : 1 + ilog2_const(x >> 1); }

// layer kinds written by the coefficient kernel (kinds[l])
//   0..4          : pairs (a, a+2^k) inside one lane (k = 0: aligned nearest-neighbour layer)
//   KIND_MIS      : nearest-neighbour layer with odd shift
//   KIND_XL + e   : butterfly stride 2^e >= M, partner lane j ^ (2^e / M)
constexpr int KIND_MIS = 8;
constexpr int KIND_XL = 16;
// OR-ed into the shared-memory copy of a layer's kind when a permutation precedes the layer
constexpr int KIND_PERM = 1 << 12;

struct PropArgs {
  int N, L, B, ldu;
  int G, logG, W, CL, S;
  unsigned layer_bytes;          // bytes of one layer's coefficient tile
  unsigned dlayer_bytes;         // BWD: bytes of one layer of the dT/dp tile
  const unsigned char* tiles;    // [L][layer_bytes]
  const unsigned char* dtiles;   // BWD: [L][dlayer_bytes]
  const int* kinds;              // [L]
  const void* in0;               // FWD/FWDDIFF: u_in      BWD: u_out
  const void* in1;               // FWDDIFF: du_in (may be null = 0)   BWD: dJ/du_out*
  void* out0;                    // FWD/FWDDIFF: u_out     BWD: u_in (may be null)
  void* out1;                    // FWDDIFF: du_out        BWD: dJ/du_in*
  float2* partial;               // BWD: (dJ/dp0, dJ/dp1) partials of this CTA/item, [L][Np/2]
  int* status;
  int v0, vend;                  // vectors [v0, vend) are handled by this CTA/item
  const void* target;            // BWD: when set, dJ/du_out* = 2 (u_out - target) replaces in1
  void* act;                     // GR 4: per-layer inputs [L][act_plane] (FWD writes them, BWD reads them)
  size_t act_plane;              // elements between the stored inputs of consecutive layers
  int nA;                        // split launch: CTAs [0, nA) hold V vectors per lane group, the rest V-1
  // permutations between layers (reference mesh.py:44-48, 71-72): before layer l, when pflags[l] != 0,
  // every vector is gathered through row l of `perm` (N ints: new[q] = old[perm[q]]); after the last
  // layer through perm_last when *pflag_last != 0.  All null: no permutations.
  const int* perm;
  const int* pflags;
  const int* perm_last;
  const int* pflag_last;
  // forward checkpoints: after layer l (l + 1 < L, (l + 1) % ckpt_every == 0) the field is also written to
  // ckpt + ((l + 1) / ckpt_every - 1) * ckpt_plane; chunk boundaries must fall on those layers
  void* ckpt;
  size_t ckpt_plane;
  int ckpt_every;
  // layers per CTA block of the partial buffer (0: L); lets layer ranges keep every range's partials
  int pstride;
  // time limit of each pipeline wait (0: kWaitLimitNs)
  unsigned long long wait_ns;
  // failure-path test only (mg_propagate_wait_test): chunk + 1 whose coefficient copy is never issued, so
  // that its wait runs out (0: none)
  int unarmed;
};

template <bool REAL> struct Fld { using T = float2; using C = C2x2; };
template <> struct Fld<true> { using T = float; using C = R2x2; };

// ---- coefficient access: complex tiles hold two float4 rows per entry ([e][h][j]), real tiles one
__device__ __forceinline__ void ld_coef(const float4* tl, int e, int G, int j, C2x2& t) {
  const float4 r0 = tl[(2 * e) * G + j], r1 = tl[(2 * e + 1) * G + j];
  t.t00 = make_float2(r0.x, r0.y); t.t01 = make_float2(r0.z, r0.w);
  t.t10 = make_float2(r1.x, r1.y); t.t11 = make_float2(r1.z, r1.w);
}
__device__ __forceinline__ void ld_coef(const float4* tl, int e, int G, int j, R2x2& t) {
  const float4 q = tl[e * G + j];
  t.t00 = q.x; t.t01 = q.y; t.t10 = q.z; t.t11 = q.w;
}
// float4 offset of the dT half of a FWDDIFF layer tile
template <bool REAL, int M> __device__ __forceinline__ int dt_off(int G) { return REAL ? (M / 2) * G : M * G; }

// ---- one 2x2 crossing on one vector
template <typename F, typename CT>
__device__ __forceinline__ void x_fwd(const CT& t, F& a, F& b) {
  const F ya = cfma(t.t01, b, cmul(t.t00, a));
  const F yb = cfma(t.t11, b, cmul(t.t10, a));
  a = ya; b = yb;
}
template <typename F, typename CT>
__device__ __forceinline__ void x_fwddiff(const CT& t, const CT& d, F& a, F& b, F& da, F& db) {
  const F nda = cfma(d.t01, b, cfma(d.t00, a, cfma(t.t01, db, cmul(t.t00, da))));
  const F ndb = cfma(d.t11, b, cfma(d.t10, a, cfma(t.t11, db, cmul(t.t10, da))));
  da = nda; db = ndb;
  x_fwd(t, a, b);
}
// back-propagation of one crossing: (y, g) at the output -> (x, g_in) at the input, G += conj(g) x^T
template <typename F, typename CT>
__device__ __forceinline__ void x_bwd(const CT& t, F& a, F& b, F& ga, F& gb, CT& acc) {
  const F xa = ccfma(t.t10, b, ccmul(t.t00, a));
  const F xb = ccfma(t.t11, b, ccmul(t.t01, a));
  acc.t00 = ccfma(ga, xa, acc.t00); acc.t01 = ccfma(ga, xb, acc.t01);
  acc.t10 = ccfma(gb, xa, acc.t10); acc.t11 = ccfma(gb, xb, acc.t11);
  const F nga = ccfma(t.t10, gb, ccmul(t.t00, ga));
  const F ngb = ccfma(t.t11, gb, ccmul(t.t01, ga));
  a = xa; b = xb; ga = nga; gb = ngb;
}
// back-propagation through one layer whose INPUT x is given (stored activation of a lossy mesh):
// G += conj(g) x^T, g <- T^H g; x is left unchanged
template <typename F, typename CT>
__device__ __forceinline__ void x_bwd_stored(const CT& t, F& xa, F& xb, F& ga, F& gb, CT& acc) {
  acc.t00 = ccfma(ga, xa, acc.t00); acc.t01 = ccfma(ga, xb, acc.t01);
  acc.t10 = ccfma(gb, xa, acc.t10); acc.t11 = ccfma(gb, xb, acc.t11);
  const F nga = ccfma(t.t10, gb, ccmul(t.t00, ga));
  const F ngb = ccfma(t.t11, gb, ccmul(t.t01, ga));
  ga = nga; gb = ngb;
}
template <int OP, int GR, typename F, typename CT>
__device__ __forceinline__ void xop(const CT& t, const CT& d, F& a, F& b, F& wa, F& wb, CT& acc) {
  if constexpr (OP == OP_FWD) x_fwd(t, a, b);
  else if constexpr (OP == OP_FWDDIFF) x_fwddiff(t, d, a, b, wa, wb);
  else if constexpr (GR == 4) x_bwd_stored(t, a, b, wa, wb, acc);
  else x_bwd(t, a, b, wa, wb, acc);
}

// Back-propagation with the parameter gradient taken directly (no 2x2 dJ/dT accumulator).
// MZI (GR = 1), from T = S(beta) P(th) S(alpha) P(ph):
//   dJ/dph = Re(i x_a conj(g_in,a))            (input-side field and gradient of mode a)
//   dJ/dth = Re(i m conj(h)),  m = (S(beta)^H y)_a, h = (S(beta)^H g)_a,  (c, s) = cos, sin(pi/4 + beta)
// orth (GR = 2): dJ/dth = (g_a y_b - g_b y_a) / 2 (the 1/2 is applied in the chunk reduction).
__device__ __forceinline__ void x_bwd_direct(const C2x2& t, float2 cs, float2& a, float2& b, float2& ga, float2& gb,
                                             float& ath, float& aph) {
  const float c = cs.x, s = cs.y;
  const float m0x = fmaf(c, a.x, s * b.y), m0y = fmaf(c, a.y, -s * b.x);
  const float h0x = fmaf(c, ga.x, s * gb.y), h0y = fmaf(c, ga.y, -s * gb.x);
  ath = fmaf(h0y, m0x, fmaf(-h0x, m0y, ath));
  const float2 xa = ccfma(t.t10, b, ccmul(t.t00, a));
  const float2 xb = ccfma(t.t11, b, ccmul(t.t01, a));
  const float2 nga = ccfma(t.t10, gb, ccmul(t.t00, ga));
  const float2 ngb = ccfma(t.t11, gb, ccmul(t.t01, ga));
  aph = fmaf(nga.y, xa.x, fmaf(-nga.x, xa.y, aph));
  a = xa; b = xb; ga = nga; gb = ngb;
}
__device__ __forceinline__ void x_bwd_direct(const R2x2& t, float2, float& a, float& b, float& ga, float& gb,
                                             float& ath, float&) {
  ath = fmaf(ga, b, fmaf(-gb, a, ath));
  const float xa = fmaf(t.t10, b, t.t00 * a), xb = fmaf(t.t11, b, t.t01 * a);
  const float nga = fmaf(t.t10, gb, t.t00 * ga), ngb = fmaf(t.t11, gb, t.t01 * ga);
  a = xa; b = xb; ga = nga; gb = ngb;
}

// ---- the complex crossings on two vectors at once (vectors v, v+1 of the lane, same crossing).
// Each scalar FMA of the one-vector forms above becomes one packed f32x2 FMA with the same operands in
// the same order, so every field result is bitwise the one-vector result; half the instructions issue.
// Coefficients enter as pairs (re, re), (im, im), (-im, -im) built once per crossing.
struct PC {
  float2 r, i, n;
};
__device__ __forceinline__ PC pc(float2 c) { return PC{pdup(c.x), pdup(c.y), pdup(-c.y)}; }
// y = c1 b + c0 a:  cfma(c1, b, cmul(c0, a))
__device__ __forceinline__ void p_lin(const PC& c0, const PC& c1, float2 ar, float2 ai, float2 br, float2 bi,
                                      float2& yr, float2& yi) {
  yr = pfma(c1.r, br, pfma(c1.n, bi, pfma(c0.r, ar, pmul(c0.n, ai))));
  yi = pfma(c1.r, bi, pfma(c1.i, br, pfma(c0.r, ai, pmul(c0.i, ar))));
}
// y = conj(c1) b + conj(c0) a:  ccfma(c1, b, ccmul(c0, a))
__device__ __forceinline__ void p_clin(const PC& c0, const PC& c1, float2 ar, float2 ai, float2 br, float2 bi,
                                       float2& yr, float2& yi) {
  yr = pfma(c1.r, br, pfma(c1.i, bi, pfma(c0.r, ar, pmul(c0.i, ai))));
  yi = pfma(c1.r, bi, pfma(c1.n, br, pfma(c0.r, ai, pmul(c0.n, ar))));
}
// acc += c x:  cfma(c, x, acc)
__device__ __forceinline__ void p_acc(const PC& c, float2 xr, float2 xi, float2& accr, float2& acci) {
  accr = pfma(c.r, xr, pfma(c.n, xi, accr));
  acci = pfma(c.r, xi, pfma(c.i, xr, acci));
}
__device__ __forceinline__ void x_fwd2(const PC (&c)[4], float2& a0, float2& b0, float2& a1, float2& b1) {
  const float2 ar = make_float2(a0.x, a1.x), ai = make_float2(a0.y, a1.y);
  const float2 br = make_float2(b0.x, b1.x), bi = make_float2(b0.y, b1.y);
  float2 yar, yai, ybr, ybi;
  p_lin(c[0], c[1], ar, ai, br, bi, yar, yai);   // ya = t01 b + t00 a
  p_lin(c[2], c[3], ar, ai, br, bi, ybr, ybi);   // yb = t11 b + t10 a
  a0 = make_float2(yar.x, yai.x); a1 = make_float2(yar.y, yai.y);
  b0 = make_float2(ybr.x, ybi.x); b1 = make_float2(ybr.y, ybi.y);
}
// x_fwddiff on two vectors (dc: the packed dT/dp coefficients)
__device__ __forceinline__ void x_fwddiff2(const PC (&c)[4], const PC (&dc)[4], float2& a0, float2& b0, float2& da0,
                                           float2& db0, float2& a1, float2& b1, float2& da1, float2& db1) {
  const float2 ar = make_float2(a0.x, a1.x), ai = make_float2(a0.y, a1.y);
  const float2 br = make_float2(b0.x, b1.x), bi = make_float2(b0.y, b1.y);
  const float2 dar = make_float2(da0.x, da1.x), dai = make_float2(da0.y, da1.y);
  const float2 dbr = make_float2(db0.x, db1.x), dbi = make_float2(db0.y, db1.y);
  float2 nar, nai, nbr, nbi;
  p_lin(c[0], c[1], dar, dai, dbr, dbi, nar, nai);   // nda = d01 b + d00 a + t01 db + t00 da
  p_acc(dc[0], ar, ai, nar, nai);
  p_acc(dc[1], br, bi, nar, nai);
  p_lin(c[2], c[3], dar, dai, dbr, dbi, nbr, nbi);   // ndb = d11 b + d10 a + t11 db + t10 da
  p_acc(dc[2], ar, ai, nbr, nbi);
  p_acc(dc[3], br, bi, nbr, nbi);
  da0 = make_float2(nar.x, nai.x); da1 = make_float2(nar.y, nai.y);
  db0 = make_float2(nbr.x, nbi.x); db1 = make_float2(nbr.y, nbi.y);
  x_fwd2(c, a0, b0, a1, b1);
}
// x_bwd_direct on two vectors; cc = (c, c), (s, s), (-s, -s), (-c, -c).  The dJ/dth terms use
// -h0x = fmaf(-c, ga.x, -s * gb.y), the exact negation of h0x; the dJ/dph terms of the pair are kept as
// two sums (+nga.y xa.x and +nga.x xa.y) that the caller subtracts once per crossing.
__device__ __forceinline__ void x_bwd_direct2(const PC (&c)[4], const float2 (&cc)[4], float2& a0, float2& b0,
                                              float2& ga0, float2& gb0, float2& a1, float2& b1, float2& ga1,
                                              float2& gb1, float2& ath, float2& aph_p, float2& aph_q) {
  const float2 ar = make_float2(a0.x, a1.x), ai = make_float2(a0.y, a1.y);
  const float2 br = make_float2(b0.x, b1.x), bi = make_float2(b0.y, b1.y);
  const float2 gar = make_float2(ga0.x, ga1.x), gai = make_float2(ga0.y, ga1.y);
  const float2 gbr = make_float2(gb0.x, gb1.x), gbi = make_float2(gb0.y, gb1.y);
  const float2 m0x = pfma(cc[0], ar, pmul(cc[1], bi)), m0y = pfma(cc[0], ai, pmul(cc[2], br));
  const float2 nh0x = pfma(cc[3], gar, pmul(cc[2], gbi)), h0y = pfma(cc[0], gai, pmul(cc[2], gbr));
  ath = pfma(h0y, m0x, pfma(nh0x, m0y, ath));
  float2 xar, xai, xbr, xbi, gxar, gxai, gxbr, gxbi;
  p_clin(c[0], c[2], ar, ai, br, bi, xar, xai);       // xa = conj(t10) b + conj(t00) a
  p_clin(c[1], c[3], ar, ai, br, bi, xbr, xbi);       // xb = conj(t11) b + conj(t01) a
  p_clin(c[0], c[2], gar, gai, gbr, gbi, gxar, gxai);
  p_clin(c[1], c[3], gar, gai, gbr, gbi, gxbr, gxbi);
  aph_p = pfma(gxai, xar, aph_p);
  aph_q = pfma(gxar, xai, aph_q);
  a0 = make_float2(xar.x, xai.x); a1 = make_float2(xar.y, xai.y);
  b0 = make_float2(xbr.x, xbi.x); b1 = make_float2(xbr.y, xbi.y);
  ga0 = make_float2(gxar.x, gxai.x); ga1 = make_float2(gxar.y, gxai.y);
  gb0 = make_float2(gxbr.x, gxbi.x); gb1 = make_float2(gxbr.y, gxbi.y);
}

// stage a warp's (dJ/dth, dJ/dph) of one slot position
__device__ __forceinline__ void acc2_stage(float2* gl2, int pos, int G, int r, float ath, float aph, bool store) {
  for (int off = G; off < 32; off <<= 1) {
    ath += __shfl_xor_sync(0xffffffffu, ath, off, 32);
    aph += __shfl_xor_sync(0xffffffffu, aph, off, 32);
  }
  if (store && r == 0) gl2[pos] = make_float2(ath, aph);
}
// float4 offset of the (c, s) splitter coefficients in a direct MZI back-propagation tile
template <int M> __device__ __forceinline__ int cs_off(int G) { return M * G; }
// compact index of an "a" lane (bit d clear) among the G/2 a-lanes of a cross-lane layer
__device__ __forceinline__ int a_lane_index(int j, int d) { return ((j / (2 * d)) * d) | (j & (d - 1)); }

__device__ __forceinline__ float2 l2_grad(float2 y, float2 t) { return make_float2(2.f * (y.x - t.x), 2.f * (y.y - t.y)); }
__device__ __forceinline__ float l2_grad(float y, float t) { return 2.f * (y - t); }

__device__ __forceinline__ void acc_zero(C2x2& a) { a = c2x2_zero(); }
__device__ __forceinline__ void acc_zero(R2x2& a) { a.t00 = a.t01 = a.t10 = a.t11 = 0.f; }

__device__ __forceinline__ void acc_xor_reduce(C2x2& a, int G) {
  for (int off = G; off < 32; off <<= 1) {
    a.t00 = cadd(a.t00, shfl_xor(a.t00, off, 32)); a.t01 = cadd(a.t01, shfl_xor(a.t01, off, 32));
    a.t10 = cadd(a.t10, shfl_xor(a.t10, off, 32)); a.t11 = cadd(a.t11, shfl_xor(a.t11, off, 32));
  }
}
__device__ __forceinline__ void acc_xor_reduce(R2x2& a, int G) {
  for (int off = G; off < 32; off <<= 1) {
    a.t00 += shfl_xor(a.t00, off, 32); a.t01 += shfl_xor(a.t01, off, 32);
    a.t10 += shfl_xor(a.t10, off, 32); a.t11 += shfl_xor(a.t11, off, 32);
  }
}
// stage the warp's dJ/dT of entry e (same [e][h][j] layout as the coefficient tile)
__device__ __forceinline__ void acc_stage(float4* gl, int e, int G, int j, int r, C2x2& a) {
  acc_xor_reduce(a, G);
  if (r == 0) {
    gl[(2 * e) * G + j] = make_float4(a.t00.x, a.t00.y, a.t01.x, a.t01.y);
    gl[(2 * e + 1) * G + j] = make_float4(a.t10.x, a.t10.y, a.t11.x, a.t11.y);
  }
}
__device__ __forceinline__ void acc_stage(float4* gl, int e, int G, int j, int r, R2x2& a) {
  acc_xor_reduce(a, G);
  if (r == 0) gl[e * G + j] = make_float4(a.t00, a.t01, a.t10, a.t11);
}

// Lane geometry of one launch.  With GT > 0 the group size is a compile-time constant (GT = 32: a
// vector fills the warp) and every index, shuffle width and group reduction folds away.
template <int GT>
struct Lanes {
  int G, j, r;
  __device__ __forceinline__ Lanes(int g_runtime, int log_g) {
    const int lane = threadIdx.x & 31;
    G = GT ? GT : g_runtime;
    j = lane & (G - 1);
    r = GT ? (lane / (GT ? GT : 1)) : (lane >> log_g);
  }
};

#ifndef MG_PACKED_CROSSINGS
#define MG_PACKED_CROSSINGS 1   // 0: every crossing in its one-vector form (for comparisons)
#endif
// ---- one crossing entry e of a layer applied to all V vectors of the lane; ua(v), ub(v) (wa, wb: the
// second field) name the vector's two modes.  Complex forward and forward-mode derivative (M >= 4,
// M*V >= 16) and direct MZI back-propagation take the vectors two at a time through the packed forms:
// measured on GB300 over Clements, Reck and FFT meshes of N = 32..600, back-propagation 4-18% and
// forward up to 16% faster.
template <int OP, int M, int V, bool REAL, int GR, bool PK, typename UA, typename UB, typename WA, typename WB>
__device__ __forceinline__ void crossing(const float4* tl, int doff, int e, int G, int j, int r, UA ua, UB ub, WA wa,
                                         WB wb, float4* gl, bool store = true) {
  using CT = typename Fld<REAL>::C;
  CT t, d, acc;
  ld_coef(tl, e, G, j, t);
  if constexpr (OP == OP_BWD && (GR == 1 || GR == 2)) {
    float2 cs = make_float2(0.f, 0.f);
    if constexpr (GR == 1) cs = reinterpret_cast<const float2*>(tl + cs_off<M>(G))[e * G + j];
    float ath = 0.f, aph = 0.f;
    if constexpr (PK && MG_PACKED_CROSSINGS && !REAL && GR == 1 && V >= 2) {
      const PC c[4] = {pc(t.t00), pc(t.t01), pc(t.t10), pc(t.t11)};
      const float2 cc[4] = {pdup(cs.x), pdup(cs.y), pdup(-cs.y), pdup(-cs.x)};
      float2 ath2 = make_float2(0.f, 0.f), aph_p = ath2, aph_q = ath2;
#pragma unroll
      for (int v = 0; v + 1 < V; v += 2)
        x_bwd_direct2(c, cc, ua(v), ub(v), wa(v), wb(v), ua(v + 1), ub(v + 1), wa(v + 1), wb(v + 1), ath2, aph_p,
                      aph_q);
      const float2 dph = psub(aph_p, aph_q);
      ath = ath2.x + ath2.y;
      aph = dph.x + dph.y;
      if constexpr (V & 1) x_bwd_direct(t, cs, ua(V - 1), ub(V - 1), wa(V - 1), wb(V - 1), ath, aph);
    } else {
#pragma unroll
      for (int v = 0; v < V; ++v) x_bwd_direct(t, cs, ua(v), ub(v), wa(v), wb(v), ath, aph);
    }
    acc2_stage(reinterpret_cast<float2*>(gl), e * G + j, G, r, ath, aph, store);
  } else if constexpr (PK && MG_PACKED_CROSSINGS && OP == OP_FWD && !REAL && V >= 2 && M >= 4 && M * V >= 16) {
    // (smaller forward tiles keep the one-vector form: the coefficient pairs made them spill; measured on
    // GB300 at N = 32 and 64: 7% slower)
    const PC c[4] = {pc(t.t00), pc(t.t01), pc(t.t10), pc(t.t11)};
#pragma unroll
    for (int v = 0; v + 1 < V; v += 2) x_fwd2(c, ua(v), ub(v), ua(v + 1), ub(v + 1));
    if constexpr (V & 1) x_fwd(t, ua(V - 1), ub(V - 1));
  } else if constexpr (PK && MG_PACKED_CROSSINGS && OP == OP_FWDDIFF && !REAL && V >= 2 && M >= 4 && M * V >= 16) {
    ld_coef(tl + doff, e, G, j, d);
    const PC c[4] = {pc(t.t00), pc(t.t01), pc(t.t10), pc(t.t11)};
    const PC dc[4] = {pc(d.t00), pc(d.t01), pc(d.t10), pc(d.t11)};
#pragma unroll
    for (int v = 0; v + 1 < V; v += 2)
      x_fwddiff2(c, dc, ua(v), ub(v), wa(v), wb(v), ua(v + 1), ub(v + 1), wa(v + 1), wb(v + 1));
    if constexpr (V & 1) x_fwddiff(t, d, ua(V - 1), ub(V - 1), wa(V - 1), wb(V - 1));
  } else {
    if constexpr (OP == OP_FWDDIFF) ld_coef(tl + doff, e, G, j, d);
    if constexpr (OP == OP_BWD) acc_zero(acc);
#pragma unroll
    for (int v = 0; v < V; ++v) xop<OP, GR>(t, d, ua(v), ub(v), wa(v), wb(v), acc);
    if constexpr (OP == OP_BWD) acc_stage(gl, e, G, j, r, acc);
  }
}
// ---- entry e between the lane's own modes a and b
template <int OP, int M, int V, bool REAL, int GR, bool PK, typename F>
__device__ __forceinline__ void entry(const float4* tl, int doff, int e, int a, int b, int G, int j, int r,
                                      F (&u)[V][M], F (&w)[V][M], float4* gl) {
  crossing<OP, M, V, REAL, GR, PK>(
      tl, doff, e, G, j, r, [&](int v) -> F& { return u[v][a]; }, [&](int v) -> F& { return u[v][b]; },
      [&](int v) -> F& { return w[v][a]; }, [&](int v) -> F& { return w[v][b]; }, gl);
}

// ---- layer with all pairs inside the lane: (a, a+SS), a = 2*SS*(e/SS) + e%SS
template <int OP, int M, int V, bool REAL, int GR, int SS, bool PK = true, typename F>
__device__ __forceinline__ void layer_local(const float4* tl, int G, int j, int r, F (&u)[V][M], F (&w)[V][M],
                                            float4* gl) {
  const int doff = dt_off<REAL, M>(G);
#pragma unroll
  for (int e = 0; e < M / 2; ++e) {
    const int a = 2 * SS * (e / SS) + (e % SS);
    entry<OP, M, V, REAL, GR, PK>(tl, doff, e, a, a + SS, G, j, r, u, w, gl);
  }
}

// ---- nearest-neighbour layer with odd shift: pairs (2e+1, 2e+2) and the lane-boundary pair
// (mode M-1 of lane j, mode 0 of lane j+1) computed by lane j (reference gpu/fwdprop.cu:98-106)
template <int OP, int M, int V, bool REAL, int GR, bool PK = true, typename F>
__device__ __forceinline__ void layer_mis(const float4* tl, int G, int j, int r, F (&u)[V][M], F (&w)[V][M],
                                          float4* gl) {
  const int doff = dt_off<REAL, M>(G);
  F nu[V], nw[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    nu[v] = shfl_down(u[v][0], 1, G);
    if constexpr (OP != OP_FWD) nw[v] = shfl_down(w[v][0], 1, G);
  }
#pragma unroll
  for (int e = 0; e < M / 2 - 1; ++e) entry<OP, M, V, REAL, GR, PK>(tl, doff, e, 2 * e + 1, 2 * e + 2, G, j, r, u, w, gl);
  crossing<OP, M, V, REAL, GR, PK>(
      tl, doff, M / 2 - 1, G, j, r, [&](int v) -> F& { return u[v][M - 1]; }, [&](int v) -> F& { return nu[v]; },
      [&](int v) -> F& { return w[v][M - 1]; }, [&](int v) -> F& { return nw[v]; }, gl);
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const F bu = shfl_up(nu[v], 1, G);
    if (j != 0) u[v][0] = bu;
    if constexpr (OP != OP_FWD) {
      const F bw = shfl_up(nw[v], 1, G);
      if (j != 0) w[v][0] = bw;
    }
  }
}

__device__ __forceinline__ float2 fadd(float2 a, float2 b) { return cadd(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return a + b; }
// staged row of the own mode m: (G_own,own, G_own,partner)
__device__ __forceinline__ void stage_xl(float4* gl, int m, int G, int j, float2 aoo, float2 aop) {
  gl[m * G + j] = make_float4(aoo.x, aoo.y, aop.x, aop.y);
}
__device__ __forceinline__ void stage_xl(float4* gl, int m, int G, int j, float aoo, float aop) {
  reinterpret_cast<float2*>(&gl[(m >> 1) * G + j])[m & 1] = make_float2(aoo, aop);
}

// ---- butterfly layer whose stride spans lanes: partner lane j ^ d holds the paired mode at the
// same register index; each lane computes its own output u' = c_self u + c_part u_partner.
__device__ __forceinline__ void ld_xl(const float4* tl, int m, int G, int j, float2& cs, float2& cp) {
  const float4 q = tl[m * G + j];
  cs = make_float2(q.x, q.y); cp = make_float2(q.z, q.w);
}
__device__ __forceinline__ void ld_xl(const float4* tl, int m, int G, int j, float& cs, float& cp) {
  const float4 q = tl[(m >> 1) * G + j];
  if (m & 1) { cs = q.z; cp = q.w; } else { cs = q.x; cp = q.y; }
}
template <int OP, int M, int V, bool REAL, int GR, typename F>
__device__ __forceinline__ void layer_xl(const float4* tl, int d, int G, int j, int r, F (&u)[V][M], F (&w)[V][M],
                                         float4* gl) {
  const int doff = dt_off<REAL, M>(G);
  const bool is_a = (j & d) == 0;
  const int ja = a_lane_index(j, d);
#pragma unroll
  for (int m = 0; m < M; ++m) {
    F cs, cp;
    ld_xl(tl, m, G, j, cs, cp);
    if constexpr (OP == OP_FWD) {
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const F ru = shfl_xor(u[v][m], d, G);
        u[v][m] = cfma(cp, ru, cmul(cs, u[v][m]));
      }
    } else if constexpr (OP == OP_FWDDIFF) {
      F ds, dp;
      ld_xl(tl + doff, m, G, j, ds, dp);
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const F ru = shfl_xor(u[v][m], d, G);
        const F rw = shfl_xor(w[v][m], d, G);
        w[v][m] = cfma(dp, ru, cfma(ds, u[v][m], cfma(cp, rw, cmul(cs, w[v][m]))));
        u[v][m] = cfma(cp, ru, cmul(cs, u[v][m]));
      }
    } else if constexpr (GR == 1 || GR == 2) {
      // coefficients of the BWD tile are the own row of T^H; a-lanes (bit d clear) own the slot's
      // gradient (their mode is the slot's first mode), b-lanes compute and discard it
      float2 sc = make_float2(0.f, 0.f);
      if constexpr (GR == 1) sc = reinterpret_cast<const float2*>(tl + cs_off<M>(G))[m * (G / 2) + ja];
      float ath = 0.f, aph = 0.f;
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const F ry = shfl_xor(u[v][m], d, G);
        const F rg = shfl_xor(w[v][m], d, G);
        const F x = cfma(cp, ry, cmul(cs, u[v][m]));
        const F ng = cfma(cp, rg, cmul(cs, w[v][m]));
        if constexpr (GR == 1) {
          const float m0x = fmaf(sc.x, u[v][m].x, sc.y * ry.y), m0y = fmaf(sc.x, u[v][m].y, -sc.y * ry.x);
          const float h0x = fmaf(sc.x, w[v][m].x, sc.y * rg.y), h0y = fmaf(sc.x, w[v][m].y, -sc.y * rg.x);
          ath = fmaf(h0y, m0x, fmaf(-h0x, m0y, ath));
          aph = fmaf(ng.y, x.x, fmaf(-ng.x, x.y, aph));
        } else {
          ath = fmaf(w[v][m], ry, fmaf(-rg, u[v][m], ath));
        }
        w[v][m] = ng;
        u[v][m] = x;
      }
      acc2_stage(reinterpret_cast<float2*>(gl), m * (G / 2) + ja, G, r, ath, aph, is_a);
    } else {
      // coefficients of the BWD tile are the own row of T^H
      F aoo = fzero<F>(), aop = fzero<F>();
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const F ry = shfl_xor(u[v][m], d, G);
        const F rg = shfl_xor(w[v][m], d, G);
        // GR 4: u already holds the layer input (stored); otherwise rebuild it with T^H
        const F x = (GR == 4) ? u[v][m] : cfma(cp, ry, cmul(cs, u[v][m]));
        const F rx = (GR == 4) ? ry : shfl_xor(x, d, G);
        aoo = ccfma(w[v][m], x, aoo);
        aop = ccfma(w[v][m], rx, aop);
        w[v][m] = cfma(cp, rg, cmul(cs, w[v][m]));
        u[v][m] = x;
      }
      for (int off = G; off < 32; off <<= 1) {
        aoo = fadd(aoo, shfl_xor(aoo, off, 32));
        aop = fadd(aop, shfl_xor(aop, off, 32));
      }
      if (r == 0) stage_xl(gl, m, G, j, aoo, aop);
    }
  }
}

// ---- one layer of any kind; NN (nearest-neighbour instantiations): kinds 0 and KIND_MIS only, which keeps
// the strided and butterfly bodies, and their registers, out of the kernel
template <int OP, int M, int V, bool REAL, int GR, bool NN = false, bool PK = true, typename F>
__device__ __forceinline__ void layer_any(int kind, const float4* tl, int G, int j, int r, F (&u)[V][M],
                                          F (&w)[V][M], float4* gl) {
  if constexpr (NN) {
    if (kind == KIND_MIS) layer_mis<OP, M, V, REAL, GR, PK>(tl, G, j, r, u, w, gl);
    else layer_local<OP, M, V, REAL, GR, 1, PK>(tl, G, j, r, u, w, gl);
    return;
  }
  switch (kind) {
    case 0: layer_local<OP, M, V, REAL, GR, 1, PK>(tl, G, j, r, u, w, gl); break;
    case 1: if constexpr (M >= 4) layer_local<OP, M, V, REAL, GR, 2, PK>(tl, G, j, r, u, w, gl); break;
    case 2: if constexpr (M >= 8) layer_local<OP, M, V, REAL, GR, 4, PK>(tl, G, j, r, u, w, gl); break;
    case 3: if constexpr (M >= 16) layer_local<OP, M, V, REAL, GR, 8, PK>(tl, G, j, r, u, w, gl); break;
    case KIND_MIS: layer_mis<OP, M, V, REAL, GR, PK>(tl, G, j, r, u, w, gl); break;
    default: layer_xl<OP, M, V, REAL, GR>(tl, 1 << (kind - KIND_XL - ilog2_const(M)), G, j, r, u, w, gl);
  }
}

// ---- permutation of the modes of every vector: new[q] = old[row[q]] for q < N (padding modes stay),
// through the lane group's shared-memory scratch of G*M fields (mode-major, scr[m*G + j] = mode j*M+m,
// so that the writes of a warp hit distinct banks).  Entries outside [0, N) leave their mode in place:
// the table is validated when it is built, and this keeps every access in bounds regardless.
template <int M, int V, typename F>
__device__ __forceinline__ void gather_group(F (&u)[V][M], const int (&src)[M], F* scr, int G, int j) {
#pragma unroll
  for (int v = 0; v < V; ++v) {
#pragma unroll
    for (int m = 0; m < M; ++m) scr[m * G + j] = u[v][m];
    __syncwarp();
#pragma unroll
    for (int m = 0; m < M; ++m) u[v][m] = scr[src[m]];
    __syncwarp();
  }
}
// SKIP_U: back-propagation from stored activations reloads the field, only the gradient moves
template <int OP, int M, int V, bool SKIP_U, typename F>
__device__ __forceinline__ void permute_fields(const int* __restrict__ row, int N, F* scr, int G, int j, F (&u)[V][M],
                                            F (&w)[V][M]) {
  int src[M];
#pragma unroll
  for (int m = 0; m < M; ++m) {
    const int q = j * M + m;
    int t = q;
    if (q < N) {
      const int r = __ldg(row + q);
      if ((unsigned)r < (unsigned)N) t = r;
    }
    src[m] = (t & (M - 1)) * G + t / M;
  }
  if constexpr (!SKIP_U) gather_group<M, V>(u, src, scr, G, j);
  if constexpr (OP != OP_FWD) gather_group<M, V>(w, src, scr, G, j);
}

// ---- field I/O: lane j of the vector's group owns modes [j*M, j*M+M); out-of-range modes read 0
template <int M, int V, bool REAL, typename F>
__device__ __forceinline__ void load_fields(F (&u)[V][M], const void* src, int vb0, int B, int N, int ldu, int j) {
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int b = vb0 + v;
    const bool okb = (src != nullptr) && (b < B);
    if constexpr (!REAL) {
      const float4* p = reinterpret_cast<const float4*>(static_cast<const float2*>(src) + (size_t)b * ldu + j * M);
#pragma unroll
      for (int k = 0; k < M / 2; ++k) {
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        if (okb && j * M + 2 * k < N) q = p[k];
        u[v][2 * k] = make_float2(q.x, q.y);
        u[v][2 * k + 1] = make_float2(q.z, q.w);
      }
    } else {
      const float2* p = reinterpret_cast<const float2*>(static_cast<const float*>(src) + (size_t)b * ldu + j * M);
#pragma unroll
      for (int k = 0; k < M / 2; ++k) {
        float2 q = make_float2(0.f, 0.f);
        if (okb && j * M + 2 * k < N) q = p[k];
        u[v][2 * k] = q.x;
        u[v][2 * k + 1] = q.y;
      }
    }
  }
}
template <int M, int V, bool REAL, typename F>
__device__ __forceinline__ void store_fields(const F (&u)[V][M], void* dst, int vb0, int B, int N, int ldu, int j) {
  if (dst == nullptr) return;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int b = vb0 + v;
    if (b >= B) continue;
    if constexpr (!REAL) {
      float4* p = reinterpret_cast<float4*>(static_cast<float2*>(dst) + (size_t)b * ldu + j * M);
#pragma unroll
      for (int k = 0; k < M / 2; ++k)
        if (j * M + 2 * k < N) p[k] = make_float4(u[v][2 * k].x, u[v][2 * k].y, u[v][2 * k + 1].x, u[v][2 * k + 1].y);
    } else {
      float2* p = reinterpret_cast<float2*>(static_cast<float*>(dst) + (size_t)b * ldu + j * M);
#pragma unroll
      for (int k = 0; k < M / 2; ++k)
        if (j * M + 2 * k < N) p[k] = make_float2(u[v][2 * k], u[v][2 * k + 1]);
    }
  }
}

// Layer kinds are staged in shared memory when L is at most this (else read through the L1 cache).
constexpr int kMaxSmemKinds = 4096;

// Permutation scratch: it starts at the first 16-byte boundary after the rest of the layout and holds
// 32*M fields per warp.
__host__ __device__ inline size_t perm_scratch_offset(size_t end) { return (end + 15) & ~size_t(15); }
__host__ __device__ inline size_t perm_scratch_bytes(int W, int M, bool real) {
  return (size_t)W * 32 * M * (real ? 4 : 8);
}

// Shared-memory footprint of one launch (host and device agree on this layout):
//   [ring: S*CL*layer_bytes][BWD: dT/dp chunk CL*dlayer_bytes][BWD: per-warp dJ/dT W*CL*Np/2*gslot]
//   [mbarriers: S+1][layer kinds: L ints when L <= kMaxSmemKinds]
//   gslot: bytes staged per slot per warp in back-propagation (32 complex dJ/dT, 16 real dJ/dT,
//   8 for the direct (dJ/dth, dJ/dph) modes); dlayer_bytes is 0 when no dT/dp tile is needed.
__host__ __device__ inline size_t prop_smem_bytes(int op, int gslot, int M, int G, int W, int CL, int S,
                                                  unsigned layer_bytes, unsigned dlayer_bytes, int L) {
  size_t b = (size_t)S * CL * layer_bytes;
  if (op == OP_BWD) {
    const size_t np2 = (size_t)G * M / 2;
    b += (size_t)CL * dlayer_bytes + (size_t)W * CL * np2 * gslot;
  }
  b += 8 * (size_t)(S + 1);
  if (L <= kMaxSmemKinds) b += 4 * (size_t)L;
  return b;
}

// Slot position of slot q in the lane-major order used by the dT/dp tiles and the gradient partials:
// pos = e*G + j for q = j*(M/2) + e, so that consecutive threads of the chunk reduction touch
// consecutive shared-memory words (no bank conflicts) and consecutive global addresses.
__host__ __device__ inline int slot_pos(int q, int M, int G) { return (q % (M / 2)) * G + q / (M / 2); }
__host__ __device__ inline int pos_slot(int pos, int M, int G) { return (pos % G) * (M / 2) + pos / G; }

// ---- chunk-end gradient reduction (BWD): sum the W warps' staged dJ/dT of every slot of the chunk
// in a fixed order, contract with dT/dp and write this CTA's partial (dJ/dp0, dJ/dp1).
template <int M, bool REAL>
__device__ __forceinline__ void chunk_reduce(const PropArgs& a, const int* kinds, int lo, int nl,
                                             const unsigned char* gst, const unsigned char* dbuf, int np2, int G) {
  const size_t gst_layer = (size_t)np2 * (REAL ? 16 : 32);
  for (int idx = threadIdx.x; idx < nl * np2; idx += blockDim.x) {
    const int li = idx / np2, pos = idx - li * np2;
    const int l = lo + li;
    const int kind = kinds[l] & ~KIND_PERM;
    const int e = pos / G, j = pos - e * G;
    int la = j, lb = j, ia, ib, mrow_a = 0, mrow_b = 0;
    const bool xl = kind >= KIND_XL;
    if (!xl) {
      ia = REAL ? e : 2 * e;
      ib = REAL ? e : 2 * e + 1;
    } else {
      const int q = j * (M / 2) + e;
      const int st = 1 << (kind - KIND_XL);
      const int ma = 2 * st * (q / st) + (q % st), mb = ma + st;
      la = ma / M; lb = mb / M;
      mrow_a = ma % M; mrow_b = mb % M;
      ia = REAL ? (mrow_a >> 1) : mrow_a;
      ib = REAL ? (mrow_b >> 1) : mrow_b;
    }
    float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb = ra;
    for (int w = 0; w < a.W; ++w) {
      const float4* gl = reinterpret_cast<const float4*>(gst + ((size_t)w * a.CL + li) * gst_layer);
      const float4 x = gl[ia * G + la];
      ra.x += x.x; ra.y += x.y; ra.z += x.z; ra.w += x.w;
      if (!REAL || xl) {
        const float4 y = gl[ib * G + lb];
        rb.x += y.x; rb.y += y.y; rb.z += y.z; rb.w += y.w;
      }
    }
    float dth = 0.f, dph = 0.f;
    const float4* D = reinterpret_cast<const float4*>(dbuf + (size_t)li * a.dlayer_bytes);
    if constexpr (!REAL) {
      // G = [[g00, g01], [g10, g11]]; XL rows are a = (G_aa, G_ab), b = (G_bb, G_ba)
      const float2 g00 = make_float2(ra.x, ra.y), g01 = make_float2(ra.z, ra.w);
      const float2 g10 = xl ? make_float2(rb.z, rb.w) : make_float2(rb.x, rb.y);
      const float2 g11 = xl ? make_float2(rb.x, rb.y) : make_float2(rb.z, rb.w);
      const float4 d0r0 = D[pos], d0r1 = D[np2 + pos], d1r0 = D[2 * np2 + pos], d1r1 = D[3 * np2 + pos];
      dth = d0r0.x * g00.x - d0r0.y * g00.y + d0r0.z * g01.x - d0r0.w * g01.y +
            d0r1.x * g10.x - d0r1.y * g10.y + d0r1.z * g11.x - d0r1.w * g11.y;
      dph = d1r0.x * g00.x - d1r0.y * g00.y + d1r0.z * g01.x - d1r0.w * g01.y +
            d1r1.x * g10.x - d1r1.y * g10.y + d1r1.z * g11.x - d1r1.w * g11.y;
    } else {
      float g00, g01, g10, g11;
      if (!xl) {
        g00 = ra.x; g01 = ra.y; g10 = ra.z; g11 = ra.w;
      } else {
        const float2 A = (mrow_a & 1) ? make_float2(ra.z, ra.w) : make_float2(ra.x, ra.y);
        const float2 Bq = (mrow_b & 1) ? make_float2(rb.z, rb.w) : make_float2(rb.x, rb.y);
        g00 = A.x; g01 = A.y; g11 = Bq.x; g10 = Bq.y;
      }
      const float4 d = D[pos];
      dth = d.x * g00 + d.y * g01 + d.z * g10 + d.w * g11;
    }
    a.partial[(size_t)l * np2 + pos] = make_float2(dth, dph);
  }
}

// ---- chunk-end reduction of the direct modes: sum the W warps' (dJ/dth, dJ/dph) per slot
// (nearest-neighbour kernels: every slot stays in place, so two slots go per 16-byte load; the sums run in the
// same warp order, so the results are bitwise those of the general form)
template <int M, int GR, bool NN = false>
__device__ __forceinline__ void chunk_reduce_direct(const PropArgs& a, const int* kinds, int lo, int nl,
                                                    const unsigned char* gst, int np2, int G) {
  const size_t gst_layer = (size_t)np2 * 8;
  if constexpr (NN) {
    const int half = np2 >> 1;
    if ((half & (half - 1)) == 0) {
      const int lg = __ffs(half) - 1;
      for (int idx = threadIdx.x; idx < (nl << lg); idx += blockDim.x) {
        const int li = idx >> lg, q = idx & (half - 1);
        float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
        for (int w = 0; w < a.W; ++w) {
          const float4 v = reinterpret_cast<const float4*>(gst + ((size_t)w * a.CL + li) * gst_layer)[q];
          t.x += v.x;
          t.y += v.y;
          t.z += v.z;
          t.w += v.w;
        }
        if constexpr (GR == 2) {
          t.x *= 0.5f;
          t.z *= 0.5f;
        }
        reinterpret_cast<float4*>(a.partial + (size_t)(lo + li) * np2)[q] = t;
      }
      return;
    }
  }
  for (int idx = threadIdx.x; idx < nl * np2; idx += blockDim.x) {
    const int li = idx / np2, pos = idx - li * np2;
    const int l = lo + li;
    const int kind = kinds[l] & ~KIND_PERM;
    int sp = pos;
    if (kind >= KIND_XL) {
      const int q = pos_slot(pos, M, G);
      const int st = 1 << (kind - KIND_XL);
      const int ma = 2 * st * (q / st) + (q % st);
      sp = (ma % M) * (G / 2) + a_lane_index(ma / M, st / M);
    }
    float sx = 0.f, sy = 0.f;
    for (int w = 0; w < a.W; ++w) {
      const float2 v = reinterpret_cast<const float2*>(gst + ((size_t)w * a.CL + li) * gst_layer)[sp];
      sx += v.x;
      sy += v.y;
    }
    a.partial[(size_t)l * np2 + pos] = make_float2(GR == 2 ? 0.5f * sx : sx, sy);
  }
}

// ---- chunk-end reduction of the raw dJ/dT modes (generic crossings): sum the W warps' staged
// dJ/dT_ij of every slot in a fixed order; partial layout [l][k][pos] float2, k = (00, 01, 10, 11)
template <int M>
__device__ __forceinline__ void chunk_reduce_raw(const PropArgs& a, const int* kinds, int lo, int nl,
                                                 const unsigned char* gst, int np2, int G) {
  const size_t gst_layer = (size_t)np2 * 32;
  for (int idx = threadIdx.x; idx < nl * np2; idx += blockDim.x) {
    const int li = idx / np2, pos = idx - li * np2;
    const int l = lo + li;
    const int kind = kinds[l] & ~KIND_PERM;
    const int e = pos / G, j = pos - e * G;
    int la = j, lb = j, ia = 2 * e, ib = 2 * e + 1;
    const bool xl = kind >= KIND_XL;
    if (xl) {
      const int q = j * (M / 2) + e;
      const int st = 1 << (kind - KIND_XL);
      const int ma = 2 * st * (q / st) + (q % st), mb = ma + st;
      la = ma / M; lb = mb / M;
      ia = ma % M; ib = mb % M;
    }
    float4 ra = make_float4(0.f, 0.f, 0.f, 0.f), rb = ra;
    for (int w = 0; w < a.W; ++w) {
      const float4* gl = reinterpret_cast<const float4*>(gst + ((size_t)w * a.CL + li) * gst_layer);
      const float4 x = gl[ia * G + la], y = gl[ib * G + lb];
      ra.x += x.x; ra.y += x.y; ra.z += x.z; ra.w += x.w;
      rb.x += y.x; rb.y += y.y; rb.z += y.z; rb.w += y.w;
    }
    float2* o = a.partial + (size_t)l * 4 * np2 + pos;
    o[0] = make_float2(ra.x, ra.y);                                        // G00 (XL: G_aa)
    o[np2] = make_float2(ra.z, ra.w);                                      // G01 (XL: G_ab)
    o[2 * np2] = xl ? make_float2(rb.z, rb.w) : make_float2(rb.x, rb.y);   // G10 (XL: G_ba)
    o[3 * np2] = xl ? make_float2(rb.x, rb.y) : make_float2(rb.z, rb.w);   // G11 (XL: G_bb)
  }
}

template <int OP, int M, int V, bool REAL>
struct PropTraits {
  static constexpr int kMaxThreads = ((OP == OP_FWD && M * V <= 16) || (OP == OP_BWD && M * V <= 8)) ? 512 : 256;
};

// Layer loop body: fused (aligned, odd-shift) pairs of nearest-neighbour layers run as one
// straight-line block (the compiler interleaves the two layers' crossings); other kinds one by one.
// GR 4 (stored activations, for lossy crossings) goes layer by layer: the forward pass writes each
// layer's input to a.act before applying it, back-propagation reloads it in place of T^H reconstruction.
// PERM (the permuted-mesh instantiations): a layer whose kind carries KIND_PERM is preceded by the gather of
// its row of pa.perm (the shared-memory copy of the kinds carries the flags).
template <int OP, int M, int V, bool REAL, int GR, bool PERM, bool NN, bool PK, typename F>
__device__ __forceinline__ void run_chunk(const PropArgs& pa, int vb0, const int* kinds, const unsigned char* st,
                                          unsigned layer_bytes, int lo, int hi, unsigned char* gst_warp,
                                          size_t gst_layer, int G, int j, int r, F (&u)[V][M], F (&w)[V][M],
                                          F* pscr) {
  static_assert(!(PERM && GR == 4), "stored-activation kernels take no permutations");
  const int nl = hi - lo;
  if constexpr (GR == 4) {
    for (int i = 0; i < nl; ++i) {
      const int l = (OP == OP_BWD) ? (hi - 1 - i) : (lo + i);
      F* plane = static_cast<F*>(pa.act) + (size_t)l * pa.act_plane;
      if constexpr (OP == OP_BWD) load_fields<M, V, REAL>(u, plane, vb0, pa.vend, pa.N, pa.ldu, j);
      else store_fields<M, V, REAL>(u, plane, vb0, pa.vend, pa.N, pa.ldu, j);
      layer_any<OP, M, V, REAL, GR, false, PK>(kinds[l], reinterpret_cast<const float4*>(st + (size_t)(l - lo) * layer_bytes), G,
                                    j, r, u, w, reinterpret_cast<float4*>(gst_warp + (size_t)(l - lo) * gst_layer));
    }
    return;
  }
  int i = 0;
  while (i < nl) {
    const int l0 = (OP == OP_BWD) ? (hi - 1 - i) : (lo + i);
    int k0 = kinds[l0];
    const float4* t0 = reinterpret_cast<const float4*>(st + (size_t)(l0 - lo) * layer_bytes);
    float4* g0 = reinterpret_cast<float4*>(gst_warp + (size_t)(l0 - lo) * gst_layer);
    if constexpr (PERM) {
      if (k0 & KIND_PERM) {   // (a permuted second layer fails the pair test below by its kind)
        permute_fields<OP, M, V, false>(pa.perm + (size_t)l0 * pa.N, pa.N, pscr, G, j, u, w);
        k0 &= ~KIND_PERM;
      }
    }
    if constexpr (NN && (OP == OP_FWD || OP == OP_FWDDIFF) && !PERM) {
      // four nearest-neighbour layers (aligned, odd, aligned, odd) as one straight-line block: more independent
      // crossings for the scheduler than a fused pair.  Measured on GB300 with bitwise the same results: forward
      // N=256 B=4096 2% faster, N=64 B=1024 13% faster, forward-mode derivative N=256 1.5% faster; eight layers
      // were slower at N=256 (0.106 against 0.101 ms), and back-propagation spilled with four
      if (i + 3 < nl && k0 == 0 && kinds[l0 + 1] == KIND_MIS && kinds[l0 + 2] == 0 && kinds[l0 + 3] == KIND_MIS) {
        const float4* t1 = reinterpret_cast<const float4*>(st + (size_t)(l0 + 1 - lo) * layer_bytes);
        const float4* t2 = reinterpret_cast<const float4*>(st + (size_t)(l0 + 2 - lo) * layer_bytes);
        const float4* t3 = reinterpret_cast<const float4*>(st + (size_t)(l0 + 3 - lo) * layer_bytes);
        layer_local<OP, M, V, REAL, GR, 1, PK>(t0, G, j, r, u, w, g0);
        layer_mis<OP, M, V, REAL, GR, PK>(t1, G, j, r, u, w, g0);
        layer_local<OP, M, V, REAL, GR, 1, PK>(t2, G, j, r, u, w, g0);
        layer_mis<OP, M, V, REAL, GR, PK>(t3, G, j, r, u, w, g0);
        i += 4;
        continue;
      }
    }
    if (i + 1 < nl && (k0 == 0 || k0 == KIND_MIS)) {
      const int l1 = (OP == OP_BWD) ? (l0 - 1) : (l0 + 1);
      const int k1 = kinds[l1];
      const float4* t1 = reinterpret_cast<const float4*>(st + (size_t)(l1 - lo) * layer_bytes);
      float4* g1 = reinterpret_cast<float4*>(gst_warp + (size_t)(l1 - lo) * gst_layer);
      // the nearest-neighbour instantiations fuse only the order their walk meets in an alternating mesh
      // (aligned then odd-shift going forward, odd-shift then aligned going back): the second fused body
      // made the back-propagation kernel spill (measured on GB300: 5% slower with both bodies)
      if ((!NN || OP != OP_BWD) && k0 == 0 && k1 == KIND_MIS) {
        layer_local<OP, M, V, REAL, GR, 1, PK>(t0, G, j, r, u, w, g0);
        layer_mis<OP, M, V, REAL, GR, PK>(t1, G, j, r, u, w, g1);
        i += 2;
        continue;
      }
      if ((!NN || OP == OP_BWD) && k0 == KIND_MIS && k1 == 0) {
        layer_mis<OP, M, V, REAL, GR, PK>(t0, G, j, r, u, w, g0);
        layer_local<OP, M, V, REAL, GR, 1, PK>(t1, G, j, r, u, w, g1);
        i += 2;
        continue;
      }
    }
    layer_any<OP, M, V, REAL, GR, NN, PK>(k0, t0, G, j, r, u, w, g0);
    i += 1;
  }
}

// One batch tile of one mesh: vectors [a.v0, a.vend), all L layers, by the W warps of the CTA.
// Shared by the one-mesh kernel (prop_kernel) and the persistent multi-mesh kernel (mg_batched.cu).
// PK: complex forward and direct back-propagation crossings take vectors in pairs (packed f32x2 forms).
// Permuted and stored-activation kernels, and forward kernels of lane groups narrower than the warp, keep
// the one-vector forms: measured on GB300 the packed forms made them 3-14% slower (more registers, spills).
template <int OP, int M, int V, bool REAL, int GT, int GR, bool PERM = false, bool NN = false, bool PK = true>
__device__ __forceinline__ void prop_body(const PropArgs& a, unsigned char* smem) {
  using F = typename Fld<REAL>::T;
  constexpr bool kPacked = PK && !PERM && GR != 4 && (OP == OP_BWD || GT == 32);
  const int tid = threadIdx.x, warp = tid >> 5;
  const Lanes<GT> ln(a.G, a.logG);
  const int G = ln.G, j = ln.j, r = ln.r, R = 32 / G;
  const int np2 = (G * M) >> 1;
  const int vb0 = a.v0 + (warp * R + r) * V;

  const size_t ring_bytes = (size_t)a.S * a.CL * a.layer_bytes;
  constexpr bool kDT = (OP == OP_BWD && GR == 0);          // dT/dp tiles needed
  const size_t dbuf_bytes = kDT ? (size_t)a.CL * a.dlayer_bytes : 0;
  constexpr bool kDirect = (GR == 1 || GR == 2);
  const size_t gst_layer = (size_t)np2 * (kDirect ? 8 : (REAL ? 16 : 32));
  const size_t gst_bytes = (OP == OP_BWD) ? (size_t)a.W * a.CL * gst_layer : 0;
  unsigned char* ring = smem;
  unsigned char* dbuf = smem + ring_bytes;
  unsigned char* gst = dbuf + dbuf_bytes;
  uint64_t* bars = reinterpret_cast<uint64_t*>(gst + gst_bytes);   // [S] ring, [S] = dT/dp buffer
  int* skinds = reinterpret_cast<int*>(bars + a.S + 1);
  const int* kinds = a.kinds;

  if (a.L <= kMaxSmemKinds) {
    for (int l = tid; l < a.L; l += blockDim.x) {
      int k = __ldg(a.kinds + l);
      if constexpr (PERM) k |= (__ldg(a.pflags + l) != 0) ? KIND_PERM : 0;
      skinds[l] = k;
    }
    kinds = skinds;
  }
  // permutation scratch: 32*M fields per warp after the kinds, 16-byte aligned (perm_scratch_offset); the
  // host admits permuted launches only with the kinds in shared memory (L <= kMaxSmemKinds)
  F* pscr = nullptr;
  if constexpr (PERM) {
    const size_t off = perm_scratch_offset(static_cast<size_t>(reinterpret_cast<unsigned char*>(skinds + a.L) - smem));
    pscr = reinterpret_cast<F*>(smem + off) + (size_t)(warp * 32 + r * G) * M;
  }

  F u[V][M];
  F w[V][M];
  load_fields<M, V, REAL>(u, a.in0, vb0, a.vend, a.N, a.ldu, j);
  if constexpr (OP == OP_BWD) {
    if (a.target) {   // fused L2 loss to a target: g = 2 (y - t)
      load_fields<M, V, REAL>(w, a.target, vb0, a.vend, a.N, a.ldu, j);
#pragma unroll
      for (int v = 0; v < V; ++v)
#pragma unroll
        for (int m = 0; m < M; ++m) w[v][m] = l2_grad(u[v][m], w[v][m]);
    } else {
      load_fields<M, V, REAL>(w, a.in1, vb0, a.vend, a.N, a.ldu, j);
    }
  } else if constexpr (OP != OP_FWD) {
    load_fields<M, V, REAL>(w, a.in1, vb0, a.vend, a.N, a.ldu, j);
  }

  const int nch = (a.L + a.CL - 1) / a.CL;
  if (tid == 0) {
    for (int s = 0; s <= a.S; ++s) mbar_init(smem_u32(bars + s), 1);
    fence_mbar_init();
  }
  __syncthreads();

  auto chunk_lo = [&](int c) { return (OP == OP_BWD) ? max(0, a.L - (c + 1) * a.CL) : c * a.CL; };
  auto chunk_hi = [&](int c) { return (OP == OP_BWD) ? a.L - c * a.CL : min(a.L, (c + 1) * a.CL); };
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
  auto issue_d = [&](int c) {
    const int lo = chunk_lo(c), hi = chunk_hi(c);
    const unsigned bytes = (unsigned)(hi - lo) * a.dlayer_bytes;
    const uint32_t bar = smem_u32(bars + a.S);
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_1d(smem_u32(dbuf), a.dtiles + (size_t)lo * a.dlayer_bytes, bytes, bar);
  };
  int issued = 0;
  if (tid == 0) {
    for (; issued < min(a.S, nch); ++issued) issue(issued);
  }
  unsigned char* gst_warp = gst + (size_t)warp * a.CL * gst_layer;

  for (int c = 0; c < nch; ++c) {
    const int lo = chunk_lo(c), hi = chunk_hi(c);
    const bool ok = mbar_wait_bounded(smem_u32(bars + (c % a.S)), (uint32_t)((c / a.S) & 1), wlim);
    if (__syncthreads_or(!ok)) {
      // give up: record, wait (bounded) for the copies still in flight, release the barriers, leave
      if (tid == 0) {
        set_status(a.status, ST_TIMEOUT);
        for (int cc = c + 1; cc < issued; ++cc)
          if (cc + 1 != a.unarmed) mbar_wait_bounded(smem_u32(bars + (cc % a.S)), (uint32_t)((cc / a.S) & 1), wlim);
        for (int s = 0; s <= a.S; ++s) mbar_inval(smem_u32(bars + s));
      }
      return;
    }
    if constexpr (kDT) {
      if (tid == 0) issue_d(c);
    }
    const unsigned char* st = ring + (size_t)(c % a.S) * a.CL * a.layer_bytes;
    run_chunk<OP, M, V, REAL, GR, PERM, NN, kPacked>(a, vb0, kinds, st, a.layer_bytes, lo, hi, gst_warp, gst_layer, G, j, r, u,
                                            w, pscr);
    if constexpr (OP == OP_FWD && GR == 0) {
      if (a.ckpt != nullptr && hi < a.L && hi % a.ckpt_every == 0)
        store_fields<M, V, REAL>(u, static_cast<F*>(a.ckpt) + (size_t)(hi / a.ckpt_every - 1) * a.ckpt_plane, vb0,
                                 a.vend, a.N, a.ldu, j);
    }
    __syncthreads();
    if constexpr (OP == OP_BWD && kDirect) chunk_reduce_direct<M, GR, NN>(a, kinds, lo, hi - lo, gst, np2, G);
    if constexpr (OP == OP_BWD && GR == 4) chunk_reduce_raw<M>(a, kinds, lo, hi - lo, gst, np2, G);
    if constexpr (kDT) {
      const bool okd = mbar_wait_bounded(smem_u32(bars + a.S), (uint32_t)(c & 1), wlim);
      if (__syncthreads_or(!okd)) {
        if (tid == 0) {
          set_status(a.status, ST_TIMEOUT);
          for (int cc = c + 1; cc < issued; ++cc)
          if (cc + 1 != a.unarmed) mbar_wait_bounded(smem_u32(bars + (cc % a.S)), (uint32_t)((cc / a.S) & 1), wlim);
          for (int s = 0; s <= a.S; ++s) mbar_inval(smem_u32(bars + s));
        }
        return;
      }
      chunk_reduce<M, REAL>(a, kinds, lo, hi - lo, gst, dbuf, np2, G);
    }
    if (tid == 0 && issued < nch) issue(issued++);
  }
  // every copy has been waited for and every thread is past its last wait (the barrier after the last
  // chunk): release the mbarriers so that a persistent caller can initialise them again
  if (tid == 0)
    for (int s = 0; s <= a.S; ++s) mbar_inval(smem_u32(bars + s));
  (void)R;
  if constexpr (PERM) {
    if (a.perm_last != nullptr && __ldg(a.pflag_last) != 0) permute_fields<OP, M, V, false>(a.perm_last, a.N, pscr, G, j, u, w);
  }
  store_fields<M, V, REAL>(u, a.out0, vb0, a.vend, a.N, a.ldu, j);
  if constexpr (OP != OP_FWD) store_fields<M, V, REAL>(w, a.out1, vb0, a.vend, a.N, a.ldu, j);
}

// MINB > 1: compiled for MINB resident CTAs of 256 threads per SM (at most 65536 / (256 * MINB) registers per
// thread), for batch tiles small enough that several CTAs share an SM
template <int OP, int M, int V, bool REAL, int GT, int GR, bool PERM = false, bool NN = false, int MINB = 1>
__global__ void __launch_bounds__(MINB > 1 ? 256 : PropTraits<OP, M, V, REAL>::kMaxThreads, MINB)
prop_kernel(const PropArgs a0) {
  extern __shared__ __align__(128) unsigned char smem[];
  PropArgs a = a0;
  const int G = GT ? GT : a.G;
  a.v0 = blockIdx.x * (a.W * (32 / G) * V);
  a.vend = a.B;
  if (OP == OP_BWD)
    a.partial = a0.partial + (size_t)blockIdx.x * (a.pstride ? a.pstride : a.L) * ((G * M) >> 1) * (GR == 4 ? 4 : 1);
  prop_body<OP, M, V, REAL, GT, GR, PERM, NN>(a, smem);
}

// Split launch for a batch that one wave of full CTAs cannot spread evenly: two CTAs per SM, the first
// nA CTAs with V vectors per lane group, the others with V-1, so that each SM scheduler carries one
// warp of each kind (2V-1 vectors) instead of two full warps on some SMs and none on others.  The two
// bodies are separate code paths chosen once per CTA.
template <int OP, int M, int V, bool REAL, int GT, int GR, bool NN = false>
__global__ void __launch_bounds__(PropTraits<OP, M, V, REAL>::kMaxThreads, 1)
prop_split_kernel(const PropArgs a0) {
  static_assert(V >= 2, "a split launch needs V >= 2");
  extern __shared__ __align__(128) unsigned char smem[];
  PropArgs a = a0;
  const int G = GT ? GT : a.G;
  const int groups = a.W * (32 / G);
  a.vend = a.B;
  if (OP == OP_BWD)
    a.partial = a0.partial + (size_t)blockIdx.x * (a.pstride ? a.pstride : a.L) * ((G * M) >> 1) * (GR == 4 ? 4 : 1);
  if ((int)blockIdx.x < a.nA) {
    a.v0 = blockIdx.x * groups * V;
    prop_body<OP, M, V, REAL, GT, GR, false, NN>(a, smem);
  } else {
    a.v0 = a.nA * groups * V + (blockIdx.x - a.nA) * groups * (V - 1);
    prop_body<OP, M, V - 1, REAL, GT, GR, false, NN>(a, smem);
  }
}

}  // namespace mg
