// Device-side building blocks shared by every kernel of the library:
//   * complex64 arithmetic on float2 (explicit FMA forms so the compiler emits one FFMA per term)
//   * mbarrier / bulk-TMA (cp.async.bulk) wrappers in inline PTX for sm_103a
//   * bounded waits: every spin on an mbarrier gives up after a time limit, records an error code in
//     the caller's status word and lets the kernel return (no __trap, no unbounded loop)
//   * the closed forms of the crossing matrices T(p, s) and their derivatives dT/dp (double precision)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mg {

// ---------------------------------------------------------------------------------------------
// status codes written by kernels into the status word of the workspace
// ---------------------------------------------------------------------------------------------
enum : int {
  ST_OK = 0,
  ST_TIMEOUT = 1,        // an mbarrier wait ran past its time limit
  ST_BAD_GEOMETRY = 2,   // lens/shifts/strides describe MZIs outside the N modes
  ST_BAD_WORK = 3,       // persistent kernel: malformed work item
};

// ---------------------------------------------------------------------------------------------
// complex helpers (float2 = complex64)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {          // a*b
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {  // c + a*b
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 ccmul(float2 a, float2 b) {         // conj(a)*b
  return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.x, b.y, -a.y * b.x));
}
__device__ __forceinline__ float2 ccfma(float2 a, float2 b, float2 c) {  // c + conj(a)*b
  return make_float2(fmaf(a.x, b.x, fmaf(a.y, b.y, c.x)), fmaf(a.x, b.y, fmaf(-a.y, b.x, c.y)));
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__device__ __forceinline__ float2 cscale(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
__device__ __forceinline__ float2 ci(float2 a) { return make_float2(-a.y, a.x); }  // i*a

// ---------------------------------------------------------------------------------------------
// packed pairs: one float2 holds the same component of two vectors and goes through the f32x2
// arithmetic of sm_100 and later (fma.rn.f32x2 etc.: one instruction, two results, each rounded
// exactly as the scalar fmaf / mul / sub would round it)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 pfma(float2 a, float2 b, float2 c) {   // a*b + c
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
      "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}
__device__ __forceinline__ float2 pmul(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 psub(float2 a, float2 b) {
  float2 d;
  asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
      "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return d;
}
__device__ __forceinline__ float2 pdup(float x) { return make_float2(x, x); }

// real "complex" overloads used by the real (orth) instantiation of the same templates
__device__ __forceinline__ float cmul(float a, float b) { return a * b; }
__device__ __forceinline__ float cfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ float ccmul(float a, float b) { return a * b; }
__device__ __forceinline__ float ccfma(float a, float b, float c) { return fmaf(a, b, c); }

__device__ __forceinline__ float2 shfl_down(float2 v, int d, int w) {
  return make_float2(__shfl_down_sync(0xffffffffu, v.x, d, w), __shfl_down_sync(0xffffffffu, v.y, d, w));
}
__device__ __forceinline__ float2 shfl_up(float2 v, int d, int w) {
  return make_float2(__shfl_up_sync(0xffffffffu, v.x, d, w), __shfl_up_sync(0xffffffffu, v.y, d, w));
}
__device__ __forceinline__ float2 shfl_xor(float2 v, int d, int w) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, d, w), __shfl_xor_sync(0xffffffffu, v.y, d, w));
}
__device__ __forceinline__ float shfl_down(float v, int d, int w) { return __shfl_down_sync(0xffffffffu, v, d, w); }
__device__ __forceinline__ float shfl_up(float v, int d, int w) { return __shfl_up_sync(0xffffffffu, v, d, w); }
__device__ __forceinline__ float shfl_xor(float v, int d, int w) { return __shfl_xor_sync(0xffffffffu, v, d, w); }

template <typename F> __device__ __forceinline__ F fzero();
template <> __device__ __forceinline__ float2 fzero<float2>() { return make_float2(0.f, 0.f); }
template <> __device__ __forceinline__ float fzero<float>() { return 0.f; }

// ---------------------------------------------------------------------------------------------
// mbarrier + bulk TMA (inline PTX, sm_90+ forms valid on sm_103a)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// An mbarrier must be invalidated before its shared memory is initialised again or reused: a persistent
// kernel that runs several work items per CTA re-initialises its barriers for every item, and
// mbarrier.init on a still-valid barrier does not reliably reset its phase.
__device__ __forceinline__ void mbar_inval(uint32_t bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// 1-D bulk copy global -> this CTA's shared memory, completion signalled on `bar` (complete_tx).
// Both addresses 16-byte aligned, bytes a multiple of 16 (checked by the host launchers).
__device__ __forceinline__ void tma_load_1d(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Time limit of one mbarrier wait.  A bulk copy of a few tens of KB completes in microseconds; the
// limit only has to separate "slow" from "never" (profilers replaying kernels are slow, not stuck).
constexpr uint64_t kWaitLimitNs = 4000000000ull;   // 4 s

// Wait for phase `parity` of `bar`; false after `limit_ns` (the caller then records ST_TIMEOUT).
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 63u) == 0 && globaltimer_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void set_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// ---------------------------------------------------------------------------------------------
// crossing matrices.  Ct = complex 2x2 (t00, t01, t10, t11).
// ---------------------------------------------------------------------------------------------
struct C2x2 {
  float2 t00, t01, t10, t11;
};
struct R2x2 {
  float t00, t01, t10, t11;
};

__device__ __forceinline__ C2x2 c2x2_identity() {
  C2x2 r;
  r.t00 = make_float2(1.f, 0.f); r.t01 = make_float2(0.f, 0.f);
  r.t10 = make_float2(0.f, 0.f); r.t11 = make_float2(1.f, 0.f);
  return r;
}
__device__ __forceinline__ C2x2 c2x2_zero() {
  C2x2 r;
  r.t00 = r.t01 = r.t10 = r.t11 = make_float2(0.f, 0.f);
  return r;
}

// The closed forms below are evaluated in double precision and rounded once to float32.  Float32
// sincosf carries a small systematic error that a deep mesh accumulates coherently (the relative
// error then grows linearly with the depth L: 1.1e-5 at L = 512 measured on a GB300); double
// trigonometry rounded to float32 leaves only unbiased rounding, whose effect grows as sqrt(L).
// This runs once per slot per call (or once per programmed mesh), never in the propagation loop.
struct Z {
  double x, y;
};
__device__ __forceinline__ Z zmul(Z a, Z b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ Z zadd(Z a, Z b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ Z zscale(double s, Z a) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ Z zi(Z a) { return {-a.y, a.x}; }
__device__ __forceinline__ float2 zf(Z a) { return make_float2((float)a.x, (float)a.y); }

// sin and cos in double precision for the coefficient precompute (GB300's FP64 pipe is narrow, and
// this runs for every slot of every training step).  Cody-Waite reduction by pi/2 with a two-term
// constant (PIO2_HI has its low 27 bits clear, so k * PIO2_HI is exact for |k| < 2^26; the split's
// residual is 6e-25), then the Taylor series of sin and cos on [-pi/4, pi/4] evaluated by Horner's rule
// to r^17 / r^18 (truncation below 1e-19; a shorter series below |r| < 1/8, truncation below 1e-20).
// Arguments beyond 2^20 go to the library sincos.  Tested against the library sincos in the GPU tests.
__device__ __forceinline__ void sincos_series(double r, double* s, double* c) {
  const double r2 = r * r;
  if (fabs(r) < 0.125) {
    *s = r * fma(r2, fma(r2, fma(r2, fma(r2, fma(r2, -2.505210838544172e-08, 2.7557319223985893e-06),
                                                -1.984126984126984e-04), 8.333333333333333e-03),
                         -0.16666666666666666), 1.0);
    *c = fma(r2, fma(r2, fma(r2, fma(r2, fma(r2, fma(r2, 2.08767569878681e-09, -2.755731922398589e-07),
                                                 2.48015873015873e-05), -1.388888888888889e-03),
                                 0.041666666666666664), -0.5), 1.0);
    return;
  }
  double ps = 2.8114572543455206e-15;                                     // 1/17!
  ps = fma(ps, r2, -7.647163731819816e-13);                               // 1/15!
  ps = fma(ps, r2, 1.6059043836821613e-10);                               // 1/13!
  ps = fma(ps, r2, -2.505210838544172e-08);                               // 1/11!
  ps = fma(ps, r2, 2.7557319223985893e-06);                               // 1/9!
  ps = fma(ps, r2, -1.984126984126984e-04);                               // 1/7!
  ps = fma(ps, r2, 8.333333333333333e-03);                                // 1/5!
  ps = fma(ps, r2, -0.16666666666666666);                                 // 1/3!
  *s = fma(r * r2, ps, r);
  double pc = -1.5619206968586225e-16;                                    // 1/18!
  pc = fma(pc, r2, 4.779477332387385e-14);                                // 1/16!
  pc = fma(pc, r2, -1.1470745597729725e-11);                              // 1/14!
  pc = fma(pc, r2, 2.08767569878681e-09);                                 // 1/12!
  pc = fma(pc, r2, -2.755731922398589e-07);                               // 1/10!
  pc = fma(pc, r2, 2.48015873015873e-05);                                 // 1/8!
  pc = fma(pc, r2, -1.388888888888889e-03);                               // 1/6!
  pc = fma(pc, r2, 0.041666666666666664);                                 // 1/4!
  pc = fma(pc, r2, -0.5);                                                 // 1/2!
  *c = fma(r2, pc, 1.0);
}
__device__ __forceinline__ void sincos_d(double x, double* s, double* c) {
  if (!(fabs(x) < 1048576.0)) {
    sincos(x, s, c);
    return;
  }
  const double k = rint(x * 0.63661977236758134308);                     // nearest multiple of pi/2
  const double r = fma(-k, 1.5893254773528196e-08, fma(-k, 1.5707963109016418, x));
  double sr, cr;
  sincos_series(r, &sr, &cr);
  switch (static_cast<int>(k) & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

// sin and cos for the coefficient tiles, whose entries are rounded to float32: the same reduction with a
// shorter series (sin to r^13, cos to r^14 on |r| <= pi/4: truncation below 2e-14), so that every value
// is correct to ~1e-13 before its float32 rounding - far below the float32 half-unit of 3e-8, so the
// rounding stays unbiased (a systematically biased single-precision sin/cos made the forward error grow
// linearly with depth) - at two thirds of the FP64 operations of sincos_d.
__device__ __forceinline__ void sincos_c(double x, double* s, double* c) {
  if (!(fabs(x) < 1048576.0)) {
    sincos(x, s, c);
    return;
  }
  const double k = rint(x * 0.63661977236758134308);
  const double r = fma(-k, 1.5893254773528196e-08, fma(-k, 1.5707963109016418, x));
  const double r2 = r * r;
  double ps = 1.6059043836821613e-10;                                     // 1/13!
  ps = fma(ps, r2, -2.505210838544172e-08);                               // 1/11!
  ps = fma(ps, r2, 2.7557319223985893e-06);                               // 1/9!
  ps = fma(ps, r2, -1.984126984126984e-04);                               // 1/7!
  ps = fma(ps, r2, 8.333333333333333e-03);                                // 1/5!
  ps = fma(ps, r2, -0.16666666666666666);                                 // 1/3!
  const double sr = fma(r * r2, ps, r);
  double pc = -1.1470745597729725e-11;                                    // 1/14!
  pc = fma(pc, r2, 2.08767569878681e-09);                                 // 1/12!
  pc = fma(pc, r2, -2.755731922398589e-07);                               // 1/10!
  pc = fma(pc, r2, 2.48015873015873e-05);                                 // 1/8!
  pc = fma(pc, r2, -1.388888888888889e-03);                               // 1/6!
  pc = fma(pc, r2, 0.041666666666666664);                                 // 1/4!
  pc = fma(pc, r2, -0.5);                                                 // 1/2!
  const double cr = fma(r2, pc, 1.0);
  switch (static_cast<int>(k) & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

// sin and cos of a small angle (|x| < 1/8, the splitter errors of a crossing) without range reduction: the
// Taylor series of sin to x^9 and of cos to x^10 by Horner's rule (truncation below 3e-18), about half
// the FP64 operations of sincos_c.  Other angles take sincos_c.
__device__ __forceinline__ void sincos_small(double x, double* s, double* c) {
  if (!(fabs(x) < 0.125)) {
    sincos_c(x, s, c);
    return;
  }
  const double x2 = x * x;
  double ps = 2.7557319223985893e-06;                                     // 1/9!
  ps = fma(ps, x2, -1.984126984126984e-04);                               // 1/7!
  ps = fma(ps, x2, 8.333333333333333e-03);                                // 1/5!
  ps = fma(ps, x2, -0.16666666666666666);                                 // 1/3!
  *s = fma(x * x2, ps, x);
  double pc = -2.755731922398589e-07;                                     // 1/10!
  pc = fma(pc, x2, 2.48015873015873e-05);                                 // 1/8!
  pc = fma(pc, x2, -1.388888888888889e-03);                               // 1/6!
  pc = fma(pc, x2, 0.041666666666666664);                                 // 1/4!
  pc = fma(pc, x2, -0.5);                                                 // 1/2!
  *c = fma(x2, pc, 1.0);
}

// Standard MZI T = S(beta) P(theta) S(alpha) P(phi) (reference crossing.py:216-221):
//   T = e^{i th/2} [[e^{i ph}(i S Cm - C Sp),  i C Cp - S Sm],
//                   [e^{i ph}(i C Cp + S Sm), -i S Cm - C Sp]]
// with C,S = cos,sin(th/2) and C+-,S+- = cos,sin(alpha +- beta).  D0 = dT/dth, D1 = dT/dph
// (crossing.py:223-231): dE/dth = (i/2)E for both exponentials, dT/dph = T diag(i, 0).  The splitter
// terms come from sin/cos of alpha and beta by the angle-sum formulas; csb, when given, receives
// (cos, sin)(pi/4 + beta) = ((cos b - sin b), (cos b + sin b)) / sqrt 2 for the direct MZI gradient.
__device__ __forceinline__ void mzi_T(float th, float ph, float al, float be, C2x2* T, C2x2* D0, C2x2* D1,
                                      float2* csb = nullptr) {
  double S, C, Sph, Cph, Sp = 0.0, Cp = 1.0, Sm = 0.0, Cm = 1.0, sb = 0.0, cb = 1.0;
  sincos_c(0.5 * (double)th, &S, &C);
  sincos_c((double)ph, &Sph, &Cph);
  if (al != 0.f || be != 0.f) {
    double sa, ca;
    sincos_small((double)al, &sa, &ca);
    sincos_small((double)be, &sb, &cb);
    Cp = ca * cb - sa * sb;
    Sp = sa * cb + ca * sb;
    Cm = ca * cb + sa * sb;
    Sm = sa * cb - ca * sb;
  }
  if (csb) {
    constexpr double kRsqrt2 = 0.70710678118654752440;
    *csb = make_float2((float)(kRsqrt2 * (cb - sb)), (float)(kRsqrt2 * (cb + sb)));
  }
  const Z E0 = {C, S};                                      // e^{i th/2}
  const Z E1 = zmul(E0, Z{Cph, Sph});                       // e^{i(th/2+ph)}
  const Z A00 = {-C * Sp, S * Cm}, A01 = {-S * Sm, C * Cp};
  const Z A10 = {S * Sm, C * Cp}, A11 = {-C * Sp, -S * Cm};
  const Z T00 = zmul(E1, A00), T01 = zmul(E0, A01), T10 = zmul(E1, A10), T11 = zmul(E0, A11);
  T->t00 = zf(T00); T->t01 = zf(T01); T->t10 = zf(T10); T->t11 = zf(T11);
  if (D0) {
    // dA/dth with dC = -S/2, dS = C/2
    const Z dA00 = {0.5 * S * Sp, 0.5 * C * Cm}, dA01 = {-0.5 * C * Sm, -0.5 * S * Cp};
    const Z dA10 = {0.5 * C * Sm, -0.5 * S * Cp}, dA11 = {0.5 * S * Sp, -0.5 * C * Cm};
    D0->t00 = zf(zmul(E1, zadd(zscale(0.5, zi(A00)), dA00)));
    D0->t01 = zf(zmul(E0, zadd(zscale(0.5, zi(A01)), dA01)));
    D0->t10 = zf(zmul(E1, zadd(zscale(0.5, zi(A10)), dA10)));
    D0->t11 = zf(zmul(E0, zadd(zscale(0.5, zi(A11)), dA11)));
  }
  if (D1) {
    D1->t00 = zf(zi(T00)); D1->t10 = zf(zi(T10));
    D1->t01 = make_float2(0.f, 0.f); D1->t11 = make_float2(0.f, 0.f);
  }
}

// Symmetric crossing (reference crossing.py:377-381, gpu/crossing.cu:90-126):
//   T = [[e^{i ph}(S + i C sin2a), i C cos2a], [i C cos2a, e^{-i ph}(S - i C sin2a)]]
__device__ __forceinline__ void sym_T(float th, float ph, float al, C2x2* T, C2x2* D0, C2x2* D1) {
  double S, C, Sph, Cph, S2a = 0.0, C2a = 1.0;
  sincos_c(0.5 * (double)th, &S, &C);
  sincos_c((double)ph, &Sph, &Cph);
  if (al != 0.f) sincos_small(2.0 * (double)al, &S2a, &C2a);
  const Z e = {Cph, Sph}, em = {Cph, -Sph};
  const Z T00 = zmul(e, Z{S, C * S2a}), T11 = zmul(em, Z{S, -C * S2a});
  T->t00 = zf(T00);
  T->t01 = T->t10 = zf(Z{0.0, C * C2a});
  T->t11 = zf(T11);
  if (D0) {
    D0->t00 = zf(zmul(e, Z{0.5 * C, -0.5 * S * S2a}));
    D0->t01 = D0->t10 = zf(Z{0.0, -0.5 * S * C2a});
    D0->t11 = zf(zmul(em, Z{0.5 * C, 0.5 * S * S2a}));
  }
  if (D1) {
    D1->t00 = zf(zi(T00));
    D1->t11 = zf(zscale(-1.0, zi(T11)));
    D1->t01 = D1->t10 = make_float2(0.f, 0.f);
  }
}

// Real orthogonal crossing (reference gpu/crossing.cu:132-148): T = [[S, -C], [C, S]], S,C of th/2.
__device__ __forceinline__ void orth_T(float th, R2x2* T, R2x2* D0) {
  double S, C;
  sincos_c(0.5 * (double)th, &S, &C);
  T->t00 = (float)S; T->t01 = (float)-C; T->t10 = (float)C; T->t11 = (float)S;
  if (D0) {
    D0->t00 = (float)(0.5 * C); D0->t01 = (float)(0.5 * S); D0->t10 = (float)(-0.5 * S); D0->t11 = (float)(0.5 * C);
  }
}

}  // namespace mg
