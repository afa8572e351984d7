// CPU restatement of the reference's mesh propagation (TEST INFRASTRUCTURE ONLY: the checker and the
// timed CPU baseline; the product path never links or calls it).
//
// Algorithm of the reference's c/dot.cpp meshdot_helper<real> (c/dot.cpp:49-308), re-expressed here:
//   * fields v (N, B) row-major, split into real and imaginary planes for vectorisation
//     (c/dot.cpp:8-26);
//   * OpenMP over blocks of batch columns (c/dot.cpp:85-93);
//   * per layer n, per MZI k of the layer: modes (shifts[n] + 2k, +1) <- T_k (.,.), with the T array
//     packed (2, 2, nT) and inds[n] the first MZI of layer n (c/dot.cpp:146-238);
//   * mode 1: forward derivative dv <- dT v + T dv (c/dot.cpp:180-203);
//   * mode 2: layers in reverse with T -> T^H, rebuilding the input, accumulating
//     dJ/dT_ij += conj(g_i) x_j and propagating g <- T^H g (c/dot.cpp:70-80, 240-288);
//   * optional phase screen before (pos 0) or after (pos 1) the mesh and per-layer permutations
//     (c/dot.cpp:29-42, 97-143, 150-152, 290-296).
// One deliberate difference: the reference accumulates dJ/dT (and the phase-screen gradient) from all
// OpenMP threads into shared arrays without synchronisation (c/dot.cpp:135, 281-284); here every
// thread accumulates privately and the partial sums are added in thread order afterwards.
//
// Same C ABI as the reference (mesh.py:86-89) so the timing harness can call either:
//   meshdot_port32 / meshdot_port64 (N, B, nT, L, T, dT, ph, dph, v, dv, inds, lens, shifts, perms,
//                                    is_perm, pos, mode, threads)
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class R>
struct Planes {
  std::vector<R> re, im;
  void split(const R* src, size_t n) {
    re.resize(n);
    im.resize(n);
    for (size_t i = 0; i < n; ++i) {
      re[i] = src[2 * i];
      im[i] = src[2 * i + 1];
    }
  }
  void merge(R* dst) const {
    for (size_t i = 0; i < re.size(); ++i) {
      dst[2 * i] = re[i];
      dst[2 * i + 1] = im[i];
    }
  }
};

// apply 2x2 complex matrix (a b; c d) to rows r1, r2 over columns [0, w)
template <class R>
inline void rot(R* __restrict x1r, R* __restrict x1i, R* __restrict x2r, R* __restrict x2i, int w, R ar, R ai, R br,
                R bi, R cr, R ci, R dr, R di) {
  for (int l = 0; l < w; ++l) {
    const R ur = x1r[l], ui = x1i[l], vr = x2r[l], vi = x2i[l];
    x1r[l] = ar * ur - ai * ui + br * vr - bi * vi;
    x1i[l] = ar * ui + ai * ur + br * vi + bi * vr;
    x2r[l] = cr * ur - ci * ui + dr * vr - di * vi;
    x2i[l] = cr * ui + ci * ur + dr * vi + di * vr;
  }
}

template <class R>
void permute_rows(int N, int B, int w, const int* perm, R* re, R* im, std::vector<R>& tmp) {
  tmp.resize((size_t)N * w);
  for (int k = 0; k < N; ++k) std::memcpy(&tmp[(size_t)k * w], re + (size_t)B * perm[k], sizeof(R) * w);
  for (int k = 0; k < N; ++k) std::memcpy(re + (size_t)B * k, &tmp[(size_t)k * w], sizeof(R) * w);
  for (int k = 0; k < N; ++k) std::memcpy(&tmp[(size_t)k * w], im + (size_t)B * perm[k], sizeof(R) * w);
  for (int k = 0; k < N; ++k) std::memcpy(im + (size_t)B * k, &tmp[(size_t)k * w], sizeof(R) * w);
}

template <class R>
void mesh_port(int N, int B, int nT, int L, R* T, R* dT, R* ph, R* dph, R* v, R* dv, const int* inds, const int* lens,
               const int* shifts, const int* perms, int is_perm, int pos, int mode, int threads) {
  const bool fd = mode == 1, bd = mode == 2;
  Planes<R> t, dt, x, dx;
  t.split(T, 4 * (size_t)nT);
  x.split(v, (size_t)N * B);
  if (fd || bd) {
    dt.split(dT, 4 * (size_t)nT);
    dx.split(dv, (size_t)N * B);
  }
  // T packed (2, 2, nT): entry (i, j) at (2i + j) * nT.  Mode 2 uses T^H: (i, j) <- conj(T(j, i)).
  auto tr = [&](int i, int j, int k, R& re, R& im) {
    if (bd) {
      re = t.re[(size_t)(2 * j + i) * nT + k];
      im = -t.im[(size_t)(2 * j + i) * nT + k];
    } else {
      re = t.re[(size_t)(2 * i + j) * nT + k];
      im = t.im[(size_t)(2 * i + j) * nT + k];
    }
  };
  if (threads < 1) threads = 1;
  const int blk = ((B - 1) / (threads * 8) + 1) * 8;
  const int nblk = (B + blk - 1) / blk;
  // per-block private accumulators (mode 2), reduced in block order afterwards
  std::vector<R> accT(bd ? (size_t)nblk * 8 * nT : 0, R(0)), accP(bd ? (size_t)nblk * N : 0, R(0));
  std::vector<R> screen_re(N), screen_im(N);
  if (pos >= 0)
    for (int k = 0; k < N; ++k) {
      const R a = bd ? -ph[k] : ph[k];
      screen_re[k] = std::cos(a);
      screen_im[k] = std::sin(a);
    }
  const int spos = (pos >= 0) ? (bd ? 1 - pos : pos) : -1;

#pragma omp parallel for num_threads(threads) schedule(static)
  for (int bi = 0; bi < nblk; ++bi) {
    const int c0 = bi * blk, w = std::min(blk, B - c0);
    R *xr = x.re.data() + c0, *xi = x.im.data() + c0;
    R *dxr = (fd || bd) ? dx.re.data() + c0 : nullptr, *dxi = (fd || bd) ? dx.im.data() + c0 : nullptr;
    std::vector<R> tmp;
    R* aT = bd ? &accT[(size_t)bi * 8 * nT] : nullptr;
    R* aP = bd ? &accP[(size_t)bi * N] : nullptr;
    auto screen = [&]() {
      for (int k = 0; k < N; ++k) {
        const R cr = screen_re[k], ci = screen_im[k];
        R* ur = xr + (size_t)k * B;
        R* ui = xi + (size_t)k * B;
        for (int l = 0; l < w; ++l) {
          const R a = ur[l] * cr - ui[l] * ci, b = ur[l] * ci + ui[l] * cr;
          ur[l] = a;
          ui[l] = b;
        }
        if (fd) {
          R* gr = dxr + (size_t)k * B;
          R* gi = dxi + (size_t)k * B;
          for (int l = 0; l < w; ++l) {
            const R a = gr[l] * cr - gi[l] * ci - ui[l] * dph[k];
            const R b = gr[l] * ci + gi[l] * cr + ur[l] * dph[k];
            gr[l] = a;
            gi[l] = b;
          }
        }
        if (bd) {
          R* gr = dxr + (size_t)k * B;
          R* gi = dxi + (size_t)k * B;
          for (int l = 0; l < w; ++l) {
            const R a = gr[l] * cr - gi[l] * ci, b = gr[l] * ci + gi[l] * cr;
            gr[l] = a;
            gi[l] = b;
            aP[k] += ur[l] * gi[l] - ui[l] * gr[l];
          }
        }
      }
    };
    if (spos == 0) screen();
    for (int s = 0; s < L; ++s) {
      const int n = bd ? L - 1 - s : s;
      if (is_perm) {
        const int* p = perms + (size_t)(n + (bd ? 1 : 0)) * N;
        permute_rows(N, B, w, p, xr, xi, tmp);
        if (fd || bd) permute_rows(N, B, w, p, dxr, dxi, tmp);
      }
      for (int k = 0; k < lens[n]; ++k) {
        const int it = inds[n] + k, m1 = shifts[n] + 2 * k;
        R* x1r = xr + (size_t)m1 * B;
        R* x1i = xi + (size_t)m1 * B;
        R* x2r = x1r + B;
        R* x2i = x1i + B;
        R ar, ai, br, bi_, cr, ci, dr, di;
        tr(0, 0, it, ar, ai);
        tr(0, 1, it, br, bi_);
        tr(1, 0, it, cr, ci);
        tr(1, 1, it, dr, di);
        if (fd) {
          const R er = dt.re[it], ei = dt.im[it], fr = dt.re[nT + it], fi = dt.im[nT + it];
          const R gr = dt.re[2 * (size_t)nT + it], gi = dt.im[2 * (size_t)nT + it];
          const R hr = dt.re[3 * (size_t)nT + it], hi = dt.im[3 * (size_t)nT + it];
          R* d1r = dxr + (size_t)m1 * B;
          R* d1i = dxi + (size_t)m1 * B;
          R* d2r = d1r + B;
          R* d2i = d1i + B;
          for (int l = 0; l < w; ++l) {
            const R ur = x1r[l], ui = x1i[l], vr = x2r[l], vi = x2i[l];
            const R pr = d1r[l], pi = d1i[l], qr = d2r[l], qi = d2i[l];
            d1r[l] = er * ur - ei * ui + fr * vr - fi * vi + ar * pr - ai * pi + br * qr - bi_ * qi;
            d1i[l] = er * ui + ei * ur + fr * vi + fi * vr + ar * pi + ai * pr + br * qi + bi_ * qr;
            d2r[l] = gr * ur - gi * ui + hr * vr - hi * vi + cr * pr - ci * pi + dr * qr - di * qi;
            d2i[l] = gr * ui + gi * ur + hr * vi + hi * vr + cr * pi + ci * pr + dr * qi + di * qr;
          }
        }
        rot(x1r, x1i, x2r, x2i, w, ar, ai, br, bi_, cr, ci, dr, di);
        if (bd) {
          R* g1r = dxr + (size_t)m1 * B;
          R* g1i = dxi + (size_t)m1 * B;
          R* g2r = g1r + B;
          R* g2i = g1i + B;
          R s00r = 0, s00i = 0, s01r = 0, s01i = 0, s10r = 0, s10i = 0, s11r = 0, s11i = 0;
          for (int l = 0; l < w; ++l) {
            const R ur = x1r[l], ui = x1i[l], vr = x2r[l], vi = x2i[l];
            const R gar = g1r[l], gai = g1i[l], gbr = g2r[l], gbi = g2i[l];
            s00r += gar * ur + gai * ui; s00i += gar * ui - gai * ur;
            s01r += gar * vr + gai * vi; s01i += gar * vi - gai * vr;
            s10r += gbr * ur + gbi * ui; s10i += gbr * ui - gbi * ur;
            s11r += gbr * vr + gbi * vi; s11i += gbr * vi - gbi * vr;
          }
          R* a = aT + (size_t)8 * it;
          a[0] += s00r; a[1] += s00i; a[2] += s01r; a[3] += s01i;
          a[4] += s10r; a[5] += s10i; a[6] += s11r; a[7] += s11i;
          rot(g1r, g1i, g2r, g2i, w, ar, ai, br, bi_, cr, ci, dr, di);
        }
      }
    }
    if (is_perm) {
      const int* p = perms + (size_t)(bd ? 0 : L) * N;
      permute_rows(N, B, w, p, xr, xi, tmp);
      if (fd || bd) permute_rows(N, B, w, p, dxr, dxi, tmp);
    }
    if (spos == 1) screen();
  }

  x.merge(v);
  if (fd) dx.merge(dv);
  if (bd) {
    dx.merge(dv);
    // dJ/dT in the packed (2, 2, nT) complex layout of dT
    for (int k = 0; k < nT; ++k)
      for (int e = 0; e < 4; ++e) {
        R sr = 0, si = 0;
        for (int b = 0; b < nblk; ++b) {
          sr += accT[(size_t)b * 8 * nT + 8 * k + 2 * e];
          si += accT[(size_t)b * 8 * nT + 8 * k + 2 * e + 1];
        }
        dT[2 * ((size_t)e * nT + k)] += sr;
        dT[2 * ((size_t)e * nT + k) + 1] += si;
      }
    if (pos >= 0)
      for (int k = 0; k < N; ++k) {
        R s = 0;
        for (int b = 0; b < nblk; ++b) s += accP[(size_t)b * N + k];
        dph[k] += s;
      }
  }
}

}  // namespace

extern "C" {
void meshdot_port32(int N, int B, int nT, int L, float* T, float* dT, float* ph, float* dph, float* v, float* dv,
                    int* inds, int* lens, int* shifts, int* perms, int is_perm, int pos, int mode, int threads) {
  mesh_port<float>(N, B, nT, L, T, dT, ph, dph, v, dv, inds, lens, shifts, perms, is_perm, pos, mode, threads);
}
void meshdot_port64(int N, int B, int nT, int L, double* T, double* dT, double* ph, double* dph, double* v, double* dv,
                    int* inds, int* lens, int* shifts, int* perms, int is_perm, int pos, int mode, int threads) {
  mesh_port<double>(N, B, nT, L, T, dT, ph, dph, v, dv, inds, lens, shifts, perms, is_perm, pos, mode, threads);
}
}
