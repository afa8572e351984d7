// MZI transfer matrices for the coefficient tiles in float-float arithmetic on the FP32 pipe.
//
// The tiles hold float32 values, and a deep mesh accumulates any systematic rounding error linearly, so each
// entry must be the float32 nearest to the exact value (then the rounding errors are unbiased and grow only
// as sqrt(L)).  The double-precision path (mzi_T in mg_device.cuh) delivers that, but GB300's FP64 pipe is
// narrow: it bounds the coefficient pass of a training step.  Here the same closed form is evaluated in
// float-float ("double-single") arithmetic - Dekker's exact two-product and Knuth's exact two-sum, a value is
// the unevaluated sum hi + lo of two floats, about 48 significant bits - so the result is correct to ~1e-13
// before its single rounding to float32, far below the float32 half-unit (3e-8), and the FP32 pipe does the
// work at many times the FP64 rate.
//
// sin and cos: Cody-Waite reduction by pi/2 (pi/2 split into three floats, the first two of 16 significant
// bits so that k * P1 and k * P2 are exact for |k| < 256), then the Taylor series on |r| <= pi/4, its first
// terms in float-float and the small tail in float (truncation below 1e-14).  Arguments of 400 or more in
// magnitude take the double-precision path.
#pragma once
#include "mg_device.cuh"

namespace mg {

struct ff {
  float h, l;
};

// exact a*b as hi + lo (FMA)
__device__ __forceinline__ ff ff_two_prod(float a, float b) {
  const float p = a * b;
  return {p, __fmaf_rn(a, b, -p)};
}
// exact a+b as hi + lo (Knuth)
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// renormalise hi + lo with |hi| >= |lo|
__device__ __forceinline__ ff ff_quick(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const ff s = ff_two_sum(a.h, b.h);
  return ff_quick(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff{-b.h, -b.l}); }
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = a.h * b.h;
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return ff_quick(p, e);
}
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  const float p = a.h * b;
  float e = __fmaf_rn(a.h, b, -p);
  e = __fmaf_rn(a.l, b, e);
  return ff_quick(p, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }
// the float nearest to hi + lo
__device__ __forceinline__ float ff_round(ff a) { return __fadd_rn(a.h, a.l); }

struct ffz {
  ff x, y;
};
__device__ __forceinline__ ffz ffz_mul(ffz a, ffz b) {
  return {ff_sub(ff_mul(a.x, b.x), ff_mul(a.y, b.y)), ff_add(ff_mul(a.x, b.y), ff_mul(a.y, b.x))};
}
__device__ __forceinline__ float2 ffz_round(ffz a) { return make_float2(ff_round(a.x), ff_round(a.y)); }

// sin and cos of a float x with |x| < 400 in float-float; returns false (nothing written) beyond
__device__ __forceinline__ bool ff_sincos(float x, ff* s, ff* c) {
  if (!(fabsf(x) < 400.f)) return false;
  // Cody-Waite: pi/2 = P1 + P2 + P3 (residual 1.2e-18); k * P1, k * P2 exact for |k| < 256
  constexpr float P1 = 1.57080078125f, P2 = -4.4543994590640068e-06f, P3 = -5.5644315544167711e-11f;
  const float k = rintf(x * 0.636619747f);
  ff r = ff_two_sum(x, -k * P1);
  r = ff_add(r, ff{-k * P2, 0.f});
  r = ff_add(r, ff_neg(ff_two_prod(k, P3)));
  const ff r2 = ff_mul(r, r);
  const float t = r2.h;
  // sin r = r + r^3 (-1/3! + r^2 (1/5! + r^2 (-1/7! + r^2 q))), q in float (|r^9 q| < 3e-7)
  const float qs = __fmaf_rn(t, __fmaf_rn(t, __fmaf_rn(t, 1.60590444e-10f, -2.50521079e-08f), 2.75573188e-06f), 0.f);
  ff ps = ff_add(ff{-0.000198412701f, 2.72559687e-12f}, ff{qs, 0.f});                 // -1/7! + r^2 q
  ps = ff_add(ff{0.00833333377f, -4.34617203e-10f}, ff_mul(r2, ps));                   // 1/5!
  ps = ff_add(ff{-0.166666672f, 4.96705388e-09f}, ff_mul(r2, ps));                     // -1/3!
  const ff sr = ff_add(r, ff_mul(ff_mul(r, r2), ps));
  // cos r = 1 + r^2 (-1/2 + r^2 (1/4! + r^2 (-1/6! + r^2 q)))
  const float qc = __fmaf_rn(t, __fmaf_rn(t, __fmaf_rn(t, -1.14707454e-11f, 2.08767559e-09f), -2.755732e-07f),
                             2.48015876e-05f);
  ff pc = ff_add(ff{-0.00138888892f, 3.36310944e-11f}, ff_mulf(r2, qc));                // -1/6! + r^2 q
  pc = ff_add(ff{0.0416666679f, -1.24176347e-09f}, ff_mul(r2, pc));                    // 1/4!
  pc = ff_add(ff{-0.5f, 0.f}, ff_mul(r2, pc));                                         // -1/2!
  const ff cr = ff_add(ff{1.f, 0.f}, ff_mul(r2, pc));
  switch (static_cast<int>(k) & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = ff_neg(sr); break;
    case 2: *s = ff_neg(sr); *c = ff_neg(cr); break;
    default: *s = ff_neg(cr); *c = sr; break;
  }
  return true;
}

// The standard MZI T (mzi_T in mg_device.cuh, reference crossing.py:216-221) from the float-float sin/cos of
// th/2, ph, alpha and beta, and, when given, the (cos, sin)(pi/4 + beta) pair of the direct gradient.
__device__ __forceinline__ void mzi_T_ff_from(ff S, ff C, ff Sph, ff Cph, ff sa, ff ca, ff sb, ff cb, C2x2* T,
                                              float2* csb) {
  const ff Cp = ff_sub(ff_mul(ca, cb), ff_mul(sa, sb)), Sp = ff_add(ff_mul(sa, cb), ff_mul(ca, sb));
  const ff Cm = ff_add(ff_mul(ca, cb), ff_mul(sa, sb)), Sm = ff_sub(ff_mul(sa, cb), ff_mul(ca, sb));
  if (csb) {
    const ff r2 = {0.707106769f, 1.21016175e-08f};                                    // 1/sqrt 2
    *csb = make_float2(ff_round(ff_mul(r2, ff_sub(cb, sb))), ff_round(ff_mul(r2, ff_add(cb, sb))));
  }
  const ffz E0 = {C, S};                                    // e^{i th/2}
  const ffz E1 = ffz_mul(E0, ffz{Cph, Sph});                // e^{i(th/2 + ph)}
  const ff CSp = ff_mul(C, Sp), SCm = ff_mul(S, Cm), SSm = ff_mul(S, Sm), CCp = ff_mul(C, Cp);
  const ffz A00 = {ff_neg(CSp), SCm}, A01 = {ff_neg(SSm), CCp};
  const ffz A10 = {SSm, CCp}, A11 = {ff_neg(CSp), ff_neg(SCm)};
  T->t00 = ffz_round(ffz_mul(E1, A00));
  T->t01 = ffz_round(ffz_mul(E0, A01));
  T->t10 = ffz_round(ffz_mul(E1, A10));
  T->t11 = ffz_round(ffz_mul(E0, A11));
}

// The same for ideal splitters (alpha = beta = 0: cos = 1, sin = 0), without the splitter products.  Each entry is
// the value mzi_T_ff_from computes for those angles, its operations reduced to the ones that are not exact
// multiplications by 1 or additions of 0.
__device__ __forceinline__ void mzi_T_ff_ideal(ff S, ff C, ff Sph, ff Cph, C2x2* T, float2* csb) {
  if (csb) {
    const float r = 0.707106769f;   // (1/sqrt 2)(cos 0 -+ sin 0), rounded
    *csb = make_float2(r, r);
  }
  const ffz E1 = ffz_mul(ffz{C, S}, ffz{Cph, Sph});        // e^{i(th/2 + ph)}
  const ff E1yS = ff_mul(E1.y, S), E1xS = ff_mul(E1.x, S), E1yC = ff_mul(E1.y, C), E1xC = ff_mul(E1.x, C);
  const ff SC = ff_mul(S, C), CC = ff_mul(C, C), SS = ff_mul(S, S), CS = ff_mul(C, S);
  T->t00 = make_float2(ff_round(ff_neg(E1yS)), ff_round(E1xS));   // e^{i(th/2+ph)} (i S)
  T->t01 = make_float2(ff_round(ff_neg(SC)), ff_round(CC));       // e^{i th/2} (i C)
  T->t10 = make_float2(ff_round(ff_neg(E1yC)), ff_round(E1xC));   // e^{i(th/2+ph)} (i C)
  T->t11 = make_float2(ff_round(SS), ff_round(ff_neg(CS)));       // e^{i th/2} (-i S)
}

// mzi_T_ff_from on the angles of one thread; false (nothing written) when an angle is outside the float-float
// range, and the caller takes the double path.
__device__ __forceinline__ bool mzi_T_ff(float th, float ph, float al, float be, C2x2* T, float2* csb) {
  ff S, C, Sph, Cph, sa, ca, sb, cb;
  if (!ff_sincos(0.5f * th, &S, &C) || !ff_sincos(ph, &Sph, &Cph) || !ff_sincos(al, &sa, &ca) ||
      !ff_sincos(be, &sb, &cb))
    return false;
  mzi_T_ff_from(S, C, Sph, Cph, sa, ca, sb, cb, T, csb);
  return true;
}

// The same over the four lanes of a quad (lanes 4k..4k+3 of a warp, all given the same angles and all calling
// it): lane k of the quad takes the sin/cos of angle k (th/2, ph, alpha, beta), the quad exchanges them by
// shuffles, and every lane combines all four.  The four sin/cos chains, the longest part, then run side by side,
// and the results are bitwise those of mzi_T_ff.  false on every lane of the quad when any angle is out of range.
// ideal (uniform over the launch): no splitter array, alpha = beta = 0, and the lanes 2 and 3 of the quad idle.
__device__ __forceinline__ bool mzi_T_ff_quad(float th, float ph, float al, float be, bool ideal, C2x2* T,
                                              float2* csb) {
  const int lane = threadIdx.x & 31, base = lane & ~3, sub = lane & 3;
  const unsigned qmask = 0xFu << base;
  const float x = sub == 0 ? 0.5f * th : (sub == 1 ? ph : (sub == 2 ? al : be));
  ff s = {0.f, 0.f}, c = {1.f, 0.f};
  int ok = ff_sincos(x, &s, &c) ? 1 : 0;
  ok &= __shfl_xor_sync(qmask, ok, 1);
  ok &= __shfl_xor_sync(qmask, ok, 2);
  if (!ok) return false;
  ff v[4][2];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k][0] = ff{__shfl_sync(qmask, s.h, base + k), __shfl_sync(qmask, s.l, base + k)};
    v[k][1] = ff{__shfl_sync(qmask, c.h, base + k), __shfl_sync(qmask, c.l, base + k)};
  }
  if (ideal) mzi_T_ff_ideal(v[0][0], v[0][1], v[1][0], v[1][1], T, csb);
  else mzi_T_ff_from(v[0][0], v[0][1], v[1][0], v[1][1], v[2][0], v[2][1], v[3][0], v[3][1], T, csb);
  return true;
}

}  // namespace mg
