// Coefficient precompute: (p, s[, dp]) -> per-layer tiles in the order the propagation kernel's
// lanes read them, plus the layer kinds and (back-propagation) the dT/dp tiles.
//
// The reference rebuilds T inside every propagation block for every chunk of layers with the
// fast-math __sincosf (gpu/gmem.cu:242-318, gpu/crossing.cu:36-148): redundant work that grows with
// the number of blocks.  Here T is built once per call (or once per programmed mesh) with the
// accurate sincosf, and inactive slots become identities so the hot loop never branches on the
// layout.  Layout of the parameter grid follows gpu/mesh.py:77-81: p[l*ldp + q*n_p + k] with
// q < N/2 the MZI slot of the layer; a nearest-neighbour slot q is active iff
// shift/2 <= q < shift/2 + len (gpu/gmem.cu:236-238); a butterfly layer with stride 2^e couples
// modes (2*2^e*(q/2^e) + q%2^e, +2^e) (gpu/fwdprop.cu:52-93).
#pragma once
#include "mg_ffcoef.cuh"
#include "mg_prop.cuh"

namespace mg {

enum { CR_MZI = 0, CR_SYM = 1, CR_ORTH = 2, CR_GENERIC = 3 };
enum { GEO_NN = 0, GEO_FFT = 1 };

struct CoefArgs {
  int N, L, crossing, geometry, op;
  int gr;                // back-propagation gradient mode (0: dJ/dT + dT/dp tiles, 1: MZI direct, 2: orth direct)
  int M, G;
  const int* lens;
  const int* shifts;
  const int* strides;
  const float* p;        // [L][ldp]
  int ldp;
  const float* s;        // [L][lds] or null
  int lds;
  const float* dp;       // FWDDIFF direction, layout of p (or null = 0)
  const float2* Tgen;    // CR_GENERIC: [L][N/2][4] (t00, t01, t10, t11)
  const float2* Dgen;    // CR_GENERIC back-propagation: [L][N/2][2][4] (dT/dp0, dT/dp1)
  unsigned char* tiles;  // [L][layer_bytes]
  unsigned layer_bytes;
  unsigned char* dtiles; // BWD: [L][dlayer_bytes]
  unsigned dlayer_bytes;
  int* kinds;            // [L] layer kinds, followed by [L][2] (shift, len) of the active slot range
  int* status;
};

__host__ __device__ inline int crossing_np(int c) { return c == CR_ORTH ? 1 : 2; }
__host__ __device__ inline int crossing_ns(int c) { return c == CR_MZI ? 2 : (c == CR_SYM ? 1 : 0); }

// csb (MZI crossings): receives (cos, sin)(pi/4 + beta) of an active slot
// QUAD: the four lanes of a quad compute the same slot together (mzi_T_ff_quad); only for MZI crossings
// without derivative tiles, which the host guarantees when it launches the quad form.
template <bool QUAD = false>
__device__ __forceinline__ void slot_T(const CoefArgs& a, int l, int q, bool active, C2x2& T, C2x2& D0, C2x2& D1,
                                       float2* csb = nullptr) {
  if (!active) {
    T = c2x2_identity(); D0 = c2x2_zero(); D1 = c2x2_zero();
    return;
  }
  if (a.crossing == CR_GENERIC) {
    const float2* t = a.Tgen + ((size_t)l * (a.N / 2) + q) * 4;
    T.t00 = t[0]; T.t01 = t[1]; T.t10 = t[2]; T.t11 = t[3];
    if (a.Dgen) {
      const float2* d = a.Dgen + ((size_t)l * (a.N / 2) + q) * 8;
      D0.t00 = d[0]; D0.t01 = d[1]; D0.t10 = d[2]; D0.t11 = d[3];
      D1.t00 = d[4]; D1.t01 = d[5]; D1.t10 = d[6]; D1.t11 = d[7];
    } else {
      D0 = c2x2_zero(); D1 = c2x2_zero();
    }
    return;
  }
  const int n_p = crossing_np(a.crossing), n_s = crossing_ns(a.crossing);
  const float* pp = a.p + (size_t)l * a.ldp + (size_t)q * n_p;
  const float* ss = a.s ? a.s + (size_t)l * a.lds + (size_t)q * n_s : nullptr;
  // dT/dp only where a tile needs it: forward-mode tiles and the dT/dp tiles of back-propagation
  // without a direct-gradient mode
  const bool need_d = a.op == OP_FWDDIFF || (a.op == OP_BWD && a.gr == 0);
  if (!need_d) {
    D0 = c2x2_zero();
    D1 = c2x2_zero();
  }
  if (a.crossing == CR_MZI) {
    // T alone (and the splitter pair of the direct gradient) in float-float on the FP32 pipe; with derivative
    // tiles, or angles beyond the float-float range, the double-precision form
    const float al = ss ? ss[0] : 0.f, be = ss ? ss[1] : 0.f;
    if (need_d ||
        !(QUAD ? mzi_T_ff_quad(pp[0], pp[1], al, be, ss == nullptr, &T, csb) : mzi_T_ff(pp[0], pp[1], al, be, &T, csb)))
      mzi_T(pp[0], pp[1], al, be, &T, need_d ? &D0 : nullptr, need_d ? &D1 : nullptr, csb);
  } else {   // CR_SYM
    sym_T(pp[0], pp[1], ss ? ss[0] : 0.f, &T, need_d ? &D0 : nullptr, need_d ? &D1 : nullptr);
  }
}

__device__ __forceinline__ void slot_R(const CoefArgs& a, int l, int q, bool active, R2x2& T, R2x2& D0) {
  if (!active) {
    T.t00 = 1.f; T.t01 = 0.f; T.t10 = 0.f; T.t11 = 1.f;
    D0.t00 = D0.t01 = D0.t10 = D0.t11 = 0.f;
    return;
  }
  const bool need_d = a.op == OP_FWDDIFF || (a.op == OP_BWD && a.gr == 0);
  if (!need_d) D0.t00 = D0.t01 = D0.t10 = D0.t11 = 0.f;
  orth_T(a.p[(size_t)l * a.ldp + q], &T, need_d ? &D0 : nullptr);
}

// kind of layer l and whether slot q is active; flags malformed geometry
__device__ __forceinline__ int layer_kind(const CoefArgs& a, int l, int q, bool* active) {
  if (a.geometry == GEO_NN) {
    const int sh = __ldg(a.shifts + l), ln = __ldg(a.lens + l);
    const bool ok = sh >= 0 && ln >= 0 && sh + 2 * ln <= a.N;
    if (!ok && q == 0) set_status(a.status, ST_BAD_GEOMETRY);
    *active = ok && q >= sh / 2 && q < sh / 2 + ln;
    return (sh & 1) ? KIND_MIS : 0;
  }
  const int e = __ldg(a.strides + l);
  const bool ok = e >= 0 && e < 30 && (2 << e) <= a.N && (a.N % (2 << e)) == 0;
  if (!ok && q == 0) set_status(a.status, ST_BAD_GEOMETRY);
  *active = ok && q < a.N / 2;
  const int st = 1 << (ok ? e : 0);
  return (2 * st <= a.M) ? (ok ? e : 0) : KIND_XL + e;
}

// Thread t of the coefficient pass: one thread per slot, or (QUAD) one quad of lanes per slot - a quad shares its
// slot, so quads leave at the bounds check whole, and its first lane writes.
template <bool QUAD>
__device__ __forceinline__ void coef_body(const CoefArgs& a, int t) {
  const int np2 = a.G * a.M / 2;
  const int idx = QUAD ? (t >> 2) : t;
  const bool writer = !QUAD || (t & 3) == 0;
  if (idx >= a.L * np2) return;
  const int l = idx / np2, q = idx - l * np2;
  bool active = false;
  const int kind = layer_kind(a, l, q, &active);
  if (q == 0 && writer) {
    a.kinds[l] = kind;
    int sh = 0, ln = 0;
    if (a.geometry == GEO_NN) {
      sh = __ldg(a.shifts + l);
      ln = __ldg(a.lens + l);
      if (sh < 0 || ln < 0 || sh + 2 * ln > a.N) sh = ln = 0;
    } else {
      bool any = false;
      layer_kind(a, l, 0, &any);
      ln = any ? a.N / 2 : 0;
    }
    a.kinds[a.L + 2 * l] = sh;
    a.kinds[a.L + 2 * l + 1] = ln;
  }
  const int M = a.M, G = a.G;
  const bool real = a.crossing == CR_ORTH;
  float4* tl = reinterpret_cast<float4*>(a.tiles + (size_t)l * a.layer_bytes);
  const bool xl = kind >= KIND_XL;
  int la = 0, ma = 0, lb = 0, mb = 0;
  if (xl) {
    const int st = 1 << (kind - KIND_XL);
    const int A = 2 * st * (q / st) + (q % st), Bm = A + st;
    la = A / M; ma = A % M; lb = Bm / M; mb = Bm % M;
  }
  const int j = q / (M / 2), e = q % (M / 2);
  if (!real) {
    C2x2 T, D0, D1;
    float2 csv = make_float2(0.f, 0.f);   // (cos, sin)(pi/4 + beta) for the direct MZI gradient; 0 if inactive
    slot_T<QUAD>(a, l, q, active, T, D0, D1, (a.op == OP_BWD && a.gr == 1) ? &csv : nullptr);
    if (!writer) return;
    if (a.op == OP_BWD && a.gr == 1) {
      float2* cs = reinterpret_cast<float2*>(tl + M * G);
      if (!xl) cs[e * G + j] = csv;
      else {
        const int d = (1 << (kind - KIND_XL)) / M;
        cs[ma * (G / 2) + a_lane_index(la, d)] = csv;
      }
    }
    if (a.op == OP_BWD && a.gr == 0) {   // planes [k][pos]: D0 row 0, D0 row 1, D1 row 0, D1 row 1
      float4* D = reinterpret_cast<float4*>(a.dtiles + (size_t)l * a.dlayer_bytes) + slot_pos(q, M, G);
      D[0] = make_float4(D0.t00.x, D0.t00.y, D0.t01.x, D0.t01.y);
      D[np2] = make_float4(D0.t10.x, D0.t10.y, D0.t11.x, D0.t11.y);
      D[2 * np2] = make_float4(D1.t00.x, D1.t00.y, D1.t01.x, D1.t01.y);
      D[3 * np2] = make_float4(D1.t10.x, D1.t10.y, D1.t11.x, D1.t11.y);
    }
    C2x2 dT = c2x2_zero();
    if (a.op == OP_FWDDIFF && active && a.dp) {
      const int n_p = crossing_np(a.crossing);
      const float* d = a.dp + (size_t)l * a.ldp + (size_t)q * n_p;
      const float d0 = d[0], d1 = (n_p > 1) ? d[1] : 0.f;
      dT.t00 = cadd(cscale(d0, D0.t00), cscale(d1, D1.t00));
      dT.t01 = cadd(cscale(d0, D0.t01), cscale(d1, D1.t01));
      dT.t10 = cadd(cscale(d0, D0.t10), cscale(d1, D1.t10));
      dT.t11 = cadd(cscale(d0, D0.t11), cscale(d1, D1.t11));
    }
    const int doff = M * G;
    if (!xl) {
      tl[(2 * e) * G + j] = make_float4(T.t00.x, T.t00.y, T.t01.x, T.t01.y);
      tl[(2 * e + 1) * G + j] = make_float4(T.t10.x, T.t10.y, T.t11.x, T.t11.y);
      if (a.op == OP_FWDDIFF) {
        tl[doff + (2 * e) * G + j] = make_float4(dT.t00.x, dT.t00.y, dT.t01.x, dT.t01.y);
        tl[doff + (2 * e + 1) * G + j] = make_float4(dT.t10.x, dT.t10.y, dT.t11.x, dT.t11.y);
      }
    } else if (a.op == OP_BWD) {   // own rows of T^H: a -> (conj t00, conj t10), b -> (conj t11, conj t01)
      tl[ma * G + la] = make_float4(T.t00.x, -T.t00.y, T.t10.x, -T.t10.y);
      tl[mb * G + lb] = make_float4(T.t11.x, -T.t11.y, T.t01.x, -T.t01.y);
    } else {                        // own rows of T: a -> (t00, t01), b -> (t11, t10)
      tl[ma * G + la] = make_float4(T.t00.x, T.t00.y, T.t01.x, T.t01.y);
      tl[mb * G + lb] = make_float4(T.t11.x, T.t11.y, T.t10.x, T.t10.y);
      if (a.op == OP_FWDDIFF) {
        tl[doff + ma * G + la] = make_float4(dT.t00.x, dT.t00.y, dT.t01.x, dT.t01.y);
        tl[doff + mb * G + lb] = make_float4(dT.t11.x, dT.t11.y, dT.t10.x, dT.t10.y);
      }
    }
  } else {
    R2x2 T, D0;
    slot_R(a, l, q, active, T, D0);
    if (!writer) return;
    if (a.op == OP_BWD && a.gr == 0) {
      float4* D = reinterpret_cast<float4*>(a.dtiles + (size_t)l * a.dlayer_bytes) + slot_pos(q, M, G);
      D[0] = make_float4(D0.t00, D0.t01, D0.t10, D0.t11);
    }
    R2x2 dT;
    dT.t00 = dT.t01 = dT.t10 = dT.t11 = 0.f;
    if (a.op == OP_FWDDIFF && active && a.dp) {
      const float d0 = a.dp[(size_t)l * a.ldp + q];
      dT.t00 = d0 * D0.t00; dT.t01 = d0 * D0.t01; dT.t10 = d0 * D0.t10; dT.t11 = d0 * D0.t11;
    }
    const int doff = (M / 2) * G;
    if (!xl) {
      tl[e * G + j] = make_float4(T.t00, T.t01, T.t10, T.t11);
      if (a.op == OP_FWDDIFF) tl[doff + e * G + j] = make_float4(dT.t00, dT.t01, dT.t10, dT.t11);
    } else {
      float2* ta = reinterpret_cast<float2*>(&tl[(ma >> 1) * G + la]) + (ma & 1);
      float2* tb = reinterpret_cast<float2*>(&tl[(mb >> 1) * G + lb]) + (mb & 1);
      if (a.op == OP_BWD) {        // rows of T^T
        *ta = make_float2(T.t00, T.t10);
        *tb = make_float2(T.t11, T.t01);
      } else {
        *ta = make_float2(T.t00, T.t01);
        *tb = make_float2(T.t11, T.t10);
        if (a.op == OP_FWDDIFF) {
          float2* da = reinterpret_cast<float2*>(&tl[doff + (ma >> 1) * G + la]) + (ma & 1);
          float2* db = reinterpret_cast<float2*>(&tl[doff + (mb >> 1) * G + lb]) + (mb & 1);
          *da = make_float2(dT.t00, dT.t01);
          *db = make_float2(dT.t11, dT.t10);
        }
      }
    }
  }
}

template <bool QUAD>
__global__ void coef_kernel(const CoefArgs a) {
  coef_body<QUAD>(a, blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace mg
