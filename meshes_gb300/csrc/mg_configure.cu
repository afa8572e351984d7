// Self-configuration by matrix diagonalisation: the sequential nulling pass of the reference's diag()
// (configure.py:187-330, its JIT-compiled diagHelper_fn) as native host code.
//
// The pass walks a list of (i, j, ind, p) steps: each step zeroes matrix element (i, j) of the running
// target U with one MZI (index ind of the left mesh, p = 0, or of the right mesh, p = 1), solving the MZI's
// (theta, phi) by a 10-iteration alternating line search (configure.py:92-98) and updating two rows of U, of
// Z (the product of the meshes' matrices at their random start, evaluated on the GPU by the caller) and, in
// the original (not "improved") method, of the bookkeeping matrices VdV and WWd.  The steps are sequential
// and each touches O(N) numbers, so the pass runs on the host in double precision; the meshes' matrices
// around it come from the GPU propagation kernels.
//
// Buffers follow the reference exactly, including its in-place transposes: U, Z (and WWd in the original
// method) are held transposed while steps act on the left mesh (p = 0) and untransposed for the right mesh,
// switching when p changes (configure.py:257-262, 289-292), and are returned in whichever form the last step
// left them, as the reference's caller reads them (configure.py:246).
//
// mg_direct_configure is the reference's direct method (configure.py:333-410, its JIT-compiled
// directHelper_fn): the MZIs are grouped into diagonals, each diagonal driven through its own input mode, and
// programmed one MZI at a time from the target's column of that input (a closed-form solve of T[0][0] per MZI)
// while a running product Upost of the diagonals already set is kept.  O(N) work per MZI plus an N x 2 column
// update per diagonal step, sequential: host code in double precision, no propagation needed.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "../../include/meshes_gb300.h"
#include "mg_launch.h"

namespace {

using cd = std::complex<double>;
const cd kI(0.0, 1.0);

struct M2 {
  cd a00, a01, a10, a11;
};

// MZICrossing (crossing.py:216-221, configure.py:39-47) and its flipped form MZICrossingOutPhase
// (configure.py:49-57), two splitter errors (alpha, beta)
M2 T_cross(const double* p, const double* s, bool outphase) {
  const double theta = p[0], phi = p[1];
  const double Cp = std::cos(s[0] + s[1]), Cm = std::cos(s[0] - s[1]), C = std::cos(theta / 2);
  const double Sp = std::sin(s[0] + s[1]), Sm = std::sin(s[0] - s[1]), S = std::sin(theta / 2);
  const cd f(std::cos(phi), std::sin(phi)), t(std::cos(theta / 2), std::sin(theta / 2));
  const cd x00(-C * Sp, S * Cm), x01(-S * Sm, C * Cp), x10(S * Sm, C * Cp), x11(-C * Sp, -S * Cm);
  if (outphase) return {t * x00, t * x01, t * (f * x10), t * (f * x11)};
  return {t * (f * x00), t * x01, t * (f * x10), t * x11};
}

M2 inv2(const M2& m) {
  const cd det = m.a00 * m.a11 - m.a01 * m.a10;
  return {m.a11 / det, -m.a01 / det, -m.a10 / det, m.a00 / det};
}

double angle(cd z) { return std::atan2(z.imag(), z.real()); }

// minimise |A + B e^ix + C e^iy + D e^i(x+y)| by alternating exact line searches (configure.py:92-98)
void linesearch(cd A, cd B, cd C, cd D, int n, double theta, double phi, double* out) {
  for (int i = 0; i < n; ++i) {
    cd temp(std::cos(theta), std::sin(theta));
    phi = angle(-(A + temp * B)) - angle(C + temp * D);
    temp = cd(std::cos(phi), std::sin(phi));
    theta = angle(-(A + temp * C)) - angle(B + temp * D);
  }
  out[0] = theta;
  out[1] = phi;
}

// solve <a|T(theta, phi)|b> = c (configure.py:101-126)
void tsolve_abc(const double* sp, const cd* a, const cd* b, cd c, const double* init, bool outphase, double* out) {
  const double Ca = std::cos(sp[0] + M_PI / 4), Cb = std::cos(sp[1] + M_PI / 4);
  const double Sa = std::sin(sp[0] + M_PI / 4), Sb = std::sin(sp[1] + M_PI / 4);
  cd A, B, C, D;
  if (!outphase) {
    const cd a1p = a[0] * Cb + kI * a[1] * Sb, a2p = a[1] * Cb + kI * a[0] * Sb;
    A = a2p * b[1] * Ca - c;
    B = kI * a1p * b[1] * Sa;
    C = kI * a2p * b[0] * Sa;
    D = a1p * b[0] * Ca;
  } else {
    const cd b1p = b[0] * Ca + kI * b[1] * Sa, b2p = b[1] * Ca + kI * b[0] * Sa;
    A = kI * a[0] * b2p * Sb - c;
    B = a[0] * b1p * Cb;
    C = a[1] * b2p * Cb;
    D = kI * a[1] * b1p * Sb;
  }
  linesearch(A, B, C, D, 10, init[0], init[1], out);
}

void transpose(cd* X, int N) {
  for (int r = 0; r < N; ++r)
    for (int c = r + 1; c < N; ++c) std::swap(X[r * N + c], X[c * N + r]);
}

// rows r0, r0+1 of X <- M @ rows
void rows2(cd* X, int N, int r0, const M2& M) {
  for (int k = 0; k < N; ++k) {
    const cd x = X[r0 * N + k], y = X[(r0 + 1) * N + k];
    X[r0 * N + k] = M.a00 * x + M.a01 * y;
    X[(r0 + 1) * N + k] = M.a10 * x + M.a11 * y;
  }
}
// columns c0, c0+1 of X <- cols @ M
void cols2(cd* X, int N, int c0, const M2& M) {
  for (int k = 0; k < N; ++k) {
    const cd x = X[k * N + c0], y = X[k * N + c0 + 1];
    X[k * N + c0] = x * M.a00 + y * M.a10;
    X[k * N + c0 + 1] = x * M.a01 + y * M.a11;
  }
}
M2 transposed(const M2& m) { return {m.a00, m.a10, m.a01, m.a11}; }
M2 conjugated(const M2& m) { return {std::conj(m.a00), std::conj(m.a01), std::conj(m.a10), std::conj(m.a11)}; }

}  // namespace

extern "C" int mg_diag_configure(int N, int K, void* U_, void* Z_, void* VdV_, void* WWd_, int n1, const double* s1,
                                 double* c1, int type1, int n2, const double* s2, double* c2, int type2,
                                 const int* ijzp, const double* init, const double* noise, int improved) {
  using mg::set_last_error;
  if (N < 2 || K < 0 || !U_ || !Z_ || !VdV_ || !WWd_ || !ijzp || !init || n1 < 0 || n2 < 0 || (n1 && (!s1 || !c1)) ||
      (n2 && (!s2 || !c2)) || type1 < 0 || type1 > 1 || type2 < 0 || type2 > 1)
    return set_last_error(MG_E_ARG, "mg_diag_configure: bad arguments");
  for (int k = 0; k < K; ++k) {
    const int i = ijzp[4 * k], j = ijzp[4 * k + 1], ind = ijzp[4 * k + 2], p = ijzp[4 * k + 3];
    const bool upper = i < j;
    const int r0 = (p == 0) ? (upper ? j - 1 : j) : (upper ? i : i - 1);
    if (i < 0 || j < 0 || i >= N || j >= N || (p != 0 && p != 1) || ind < 0 || ind >= (p == 0 ? n1 : n2) || r0 < 0 ||
        r0 + 1 >= N)
      return set_last_error(MG_E_ARG, "mg_diag_configure: step %d (i=%d j=%d ind=%d p=%d) out of range", k, i, j, ind, p);
  }
  cd* U = static_cast<cd*>(U_);
  cd* Z = static_cast<cd*>(Z_);
  cd* VdV = static_cast<cd*>(VdV_);
  cd* WWd = static_cast<cd*>(WWd_);
  std::vector<cd> wj(N), vi(N);
  int p_prev = 1;
  for (int k = 0; k < K; ++k) {
    const int i = ijzp[4 * k], j = ijzp[4 * k + 1], ind = ijzp[4 * k + 2], p = ijzp[4 * k + 3];
    const bool upper = i < j;
    const double* ik = init + 2 * k;
    if (p == 0) {
      // left mesh: U, Z (and WWd) held transposed
      if (p != p_prev) {
        if (!improved) transpose(WWd, N);
        transpose(Z, N);
        transpose(U, N);
        p_prev = p;
      }
      const int j1 = upper ? j - 1 : j;
      cd u = U[j1 * N + i], v = U[(j1 + 1) * N + i];
      if (u == 0.0 && v == 0.0) {   // (1, 0) above the diagonal, else (0, 1)
        u = upper ? cd(1, 0) : cd(0, 0);
        v = upper ? cd(0, 0) : cd(1, 0);
      }
      const double nrm = std::sqrt(std::norm(u) + std::norm(v));
      M2 T0dag = {v / nrm, std::conj(u) / nrm, -u / nrm, std::conj(v) / nrm};
      if (upper) T0dag = {T0dag.a01, T0dag.a00, T0dag.a11, T0dag.a10};
      rows2(Z, N, j1, transposed(inv2(T_cross(c1 + 2 * ind, s1 + 2 * ind, type1 == 1))));
      const int col = j - j1;
      const cd w0 = col ? T0dag.a01 : T0dag.a00, w1 = col ? T0dag.a11 : T0dag.a10;   // T0dag[:, j-j1]
      if (improved) {
        const cd a2[2] = {Z[j1 * N + i], Z[(j1 + 1) * N + i]};
        const cd b2[2] = {w0, w1};
        tsolve_abc(s1 + 2 * ind, a2, b2, cd(0, 0), ik, type1 == 1, c1 + 2 * ind);
      } else {
        for (int c = 0; c < N; ++c) wj[c] = w0 * WWd[j1 * N + c] + w1 * WWd[(j1 + 1) * N + c];
        for (int r = 0; r < N; ++r) {
          cd acc = 0;
          for (int c = 0; c < N; ++c) acc += Z[r * N + c] * VdV[i * N + c];
          vi[r] = acc;
        }
        cd res = 0;
        for (int c = 0; c < N; ++c) res += wj[c] * vi[c];
        res -= wj[j1] * vi[j1] + wj[j1 + 1] * vi[j1 + 1];
        const cd a2[2] = {vi[j1], vi[j1 + 1]};
        const cd b2[2] = {wj[j1], wj[j1 + 1]};
        tsolve_abc(s1 + 2 * ind, a2, b2, -res, ik, type1 == 1, c1 + 2 * ind);
      }
      if (noise) {
        c1[2 * ind] += noise[2 * k];
        c1[2 * ind + 1] += noise[2 * k + 1];
      }
      const M2 T = T_cross(c1 + 2 * ind, s1 + 2 * ind, type1 == 1);
      if (improved) {
        rows2(U, N, j1, conjugated(T));
      } else {
        rows2(U, N, j1, transposed(T0dag));
        rows2(WWd, N, j1, transposed(T0dag));
        cols2(WWd, N, j1, transposed(T));
      }
    } else {
      // right mesh: U, Z (and WWd) held untransposed
      if (p != p_prev) {
        if (!improved) transpose(WWd, N);
        transpose(Z, N);
        transpose(U, N);
        p_prev = p;
      }
      const int i1 = upper ? i : i - 1;
      cd u = U[i1 * N + j], v = U[(i1 + 1) * N + j];
      if (u == 0.0 && v == 0.0) {   // (0, 1) above the diagonal, else (1, 0)
        u = upper ? cd(0, 0) : cd(1, 0);
        v = upper ? cd(1, 0) : cd(0, 0);
      }
      const double nrm = std::sqrt(std::norm(u) + std::norm(v));
      M2 T0dag = {std::conj(u) / nrm, std::conj(v) / nrm, v / nrm, -u / nrm};
      if (upper) T0dag = {T0dag.a10, T0dag.a11, T0dag.a00, T0dag.a01};
      rows2(Z, N, i1, inv2(T_cross(c2 + 2 * ind, s2 + 2 * ind, type2 == 1)));
      const int row = i - i1;
      const cd t0 = row ? T0dag.a10 : T0dag.a00, t1 = row ? T0dag.a11 : T0dag.a01;   // T0dag[i-i1, :]
      if (improved) {
        const cd a2[2] = {t0, t1};
        const cd b2[2] = {Z[i1 * N + j], Z[(i1 + 1) * N + j]};
        tsolve_abc(s2 + 2 * ind, a2, b2, cd(0, 0), ik, type2 == 1, c2 + 2 * ind);
      } else {
        for (int r = 0; r < N; ++r) {
          cd acc = 0;
          for (int c = 0; c < N; ++c) acc += Z[r * N + c] * WWd[c * N + j];
          wj[r] = acc;
        }
        for (int c = 0; c < N; ++c) vi[c] = t0 * VdV[i1 * N + c] + t1 * VdV[(i1 + 1) * N + c];
        cd res = 0;
        for (int c = 0; c < N; ++c) res += wj[c] * vi[c];
        res -= wj[i1] * vi[i1] + wj[i1 + 1] * vi[i1 + 1];
        const cd a2[2] = {vi[i1], vi[i1 + 1]};
        const cd b2[2] = {wj[i1], wj[i1 + 1]};
        tsolve_abc(s2 + 2 * ind, a2, b2, -res, ik, type2 == 1, c2 + 2 * ind);
      }
      if (noise) {
        c2[2 * ind] += noise[2 * k];
        c2[2 * ind + 1] += noise[2 * k + 1];
      }
      const M2 T = T_cross(c2 + 2 * ind, s2 + 2 * ind, type2 == 1);
      if (improved) {
        rows2(U, N, i1, conjugated(transposed(T)));
      } else {
        rows2(U, N, i1, T0dag);
        rows2(VdV, N, i1, T0dag);
        cols2(VdV, N, i1, T);
      }
    }
  }
  return MG_OK;
}

namespace {

// the MZI phases (theta, phi) with T(theta, phi)[0][0] = t for splitter errors (alpha, beta) (configure.py:163-172);
// a target outside the reachable range clips to the nearest splitting ratio, and an undefined ratio gives theta 0
void tsolve_11(cd t, const double* s, double* out) {
  const double Cm = std::cos(s[0] - s[1]), Sp = std::sin(s[0] + s[1]);
  const double a = std::abs(t);
  const double S2 = (a * a - Sp * Sp) / (Cm * Cm - Sp * Sp);
  double h = 0.0;
  if (!std::isnan(S2)) {
    h = std::asin(std::sqrt(std::min(std::max(S2, 0.0), 1.0)));
    if (std::isnan(h)) h = 0.0;
  }
  out[0] = 2.0 * h;
  out[1] = angle(t) - angle(cd(-std::cos(h) * Sp, Cm * std::sin(h))) - h;
}

struct Cross {
  int i, j, ind, d;   // layer, index in the layer, top mode, diagonal label i - ind
};

}  // namespace

extern "C" int mg_direct_configure(int N, int L, const int* lens, const int* shifts, const void* U_, const double* s,
                                   double* p, double* phi_out, int dk_max) {
  using mg::set_last_error;
  if (N < 2 || L < 0 || (L && (!lens || !shifts)) || !U_ || !phi_out || dk_max < 1)
    return set_last_error(MG_E_ARG, "mg_direct_configure: bad arguments");
  std::vector<int> inds(L + 1, 0);
  for (int i = 0; i < L; ++i) {
    if (lens[i] < 0 || shifts[i] < 0 || shifts[i] + 2 * lens[i] > N)
      return set_last_error(MG_E_ARG, "mg_direct_configure: layer %d (shift %d, len %d) outside N=%d", i, shifts[i],
                            lens[i], N);
    inds[i + 1] = inds[i] + lens[i];
  }
  const int n_cr = inds[L];
  if (n_cr && (!s || !p)) return set_last_error(MG_E_ARG, "mg_direct_configure: s or p is NULL");
  const cd* U = static_cast<const cd*>(U_);
  for (int k = 0; k < N; ++k) phi_out[k] = 0.0;

  // diagonals (configure.py:348-350): crossings ordered by label descending, then layer descending, split where
  // the label changes.  The reference's split drops its first piece, which holds every crossing when there is
  // only one label, so a mesh with a single diagonal is left as it is.
  std::vector<Cross> cr;
  cr.reserve(n_cr);
  int max_key = 0;
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < lens[i]; ++j) {
      const int ind = shifts[i] + 2 * j;
      cr.push_back({i, j, ind, i - ind});
      max_key = std::max(max_key, i + ind);
    }
  std::sort(cr.begin(), cr.end(), [](const Cross& a, const Cross& b) { return a.d != b.d ? a.d > b.d : a.i > b.i; });
  std::vector<int> start;
  for (int c = 0; c < n_cr; ++c)
    if (c == 0 || cr[c].d != cr[c - 1].d) start.push_back(c);
  if (start.size() < 2) return MG_OK;
  start.push_back(n_cr);
  const int n_diag = (int)start.size() - 1;
  for (int g = 1; g < n_diag; ++g)   // each diagonal has its own input mode, increasing (configure.py:351)
    if (cr[start[g + 1] - 1].ind <= cr[start[g] - 1].ind)
      return set_last_error(MG_E_ARG, "mg_direct_configure: diagonals %d and %d share an input mode", g - 1, g);

  // output field of each anti-diagonal i + ind: its topmost crossing's mode (configure.py:354-356)
  const int n_of = 2 * max_key + 5;
  std::vector<int> of(n_of, 0), is_of(n_of, 0);
  for (const Cross& c : cr) {
    const int key = c.i + c.ind;
    if (!is_of[key] || c.ind < of[key]) of[key] = c.ind;
    is_of[key] = 1;
  }
  // env[i]: the highest top mode of layers i..L-1 (configure.py:357)
  std::vector<int> env(std::max(L, 1), 0);
  for (int i = L - 1; i >= 0; --i) {
    env[i] = shifts[i] + 2 * lens[i] - 2;
    if (i + 1 < L) env[i] = std::max(env[i], env[i + 1]);
  }

  std::vector<cd> Upost((size_t)N * N, cd(0, 0)), w(N);
  for (int k = 0; k < N; ++k) Upost[(size_t)k * N + k] = 1.0;
  std::vector<M2> Tl(N + 5);
  auto rows = [N](int k, int dk, int* r0, int* r1) {   // the rows k:k+dk of an N-row array, as numpy clips them
    *r0 = std::min(k, N);
    *r1 = std::max(*r0, std::min(k + dk, N));
  };
  for (int g = 0; g < n_diag; ++g) {
    const int c0 = start[g], c1 = start[g + 1], len = c1 - c0;
    const int l = cr[c1 - 1].ind;   // the diagonal's input mode
    cd E_in = 1.0;
    int ptr_last = 0, i = 0, ind = 0, ptr = 0;
    std::fill(w.begin(), w.end(), cd(0, 0));
    for (int m = 0; m < len; ++m) {   // down the diagonal: layer ascending (configure.py:383-398)
      const Cross& c = cr[c1 - 1 - m];
      i = c.i;
      ind = c.ind;
      ptr = inds[i] + c.j;
      const int k = is_of[i + ind] ? of[i + ind] : ind;
      const int dk = (i < L - 1) ? (is_of[i + ind + 2] ? std::min(dk_max, of[i + ind + 2] - k) : dk_max) : 1;
      int r0, r1;
      rows(k, dk, &r0, &r1);
      cd num = 0, den = 0;
      for (int r = r0; r < r1; ++r) {
        num += U[(size_t)r * N + l] - w[r];
        den += E_in * Upost[(size_t)r * N + ind];
      }
      double tp[2];
      tsolve_11(num / den, s + 2 * ptr, tp);
      p[2 * ptr] = tp[0];
      if (m) p[2 * ptr_last + 1] = tp[1];
      else phi_out[ind] = tp[1];
      const M2 T = T_cross(tp, s + 2 * ptr, false);
      Tl[m] = T;
      for (int r = 0; r < N; ++r) w[r] += E_in * T.a00 * Upost[(size_t)r * N + ind];
      E_in *= T.a10;
      phi_out[ind + 1] = angle(U[(size_t)k * N + ind + 1]) - angle(Upost[(size_t)k * N + ind] * T.a01);
      ptr_last = ptr;
    }
    // the last MZI's phi (configure.py:399-403)
    const int k = (i == L - 1 || ind > env[i + 1]) ? ind + 1 : of[i + ind + 2];
    const int dk = (i < L - 1) ? (is_of[i + ind + 4] ? std::min(dk_max, of[i + ind + 4] - k) : dk_max) : 1;
    int r0, r1;
    rows(k, dk, &r0, &r1);
    cd num = 0, den = 0;
    for (int r = r0; r < r1; ++r) {
      num += U[(size_t)r * N + l] - w[r];
      den += E_in * Upost[(size_t)r * N + ind + 1];
    }
    const double phi = angle(num) - angle(den);
    p[2 * ptr + 1] = phi;
    const cd e(std::cos(phi), std::sin(phi));
    for (int r = 0; r < N; ++r) Upost[(size_t)r * N + ind + 1] *= e;
    for (int m = len - 1; m >= 0; --m)   // Upost <- Upost T for the diagonal's MZIs, layer descending
      cols2(Upost.data(), N, cr[c1 - 1 - m].ind, Tl[m]);
  }
  return MG_OK;
}
