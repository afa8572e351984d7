"""CPU oracle for the mesh-propagation hot path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.  The CUDA product path in
``meshes_gb300`` never routes through it and fails loudly when its extension is missing.

It restates, in complex128 numpy, the reference's CPU algorithm for propagating batches of fields
through layered MZI meshes:

* crossing matrices T(p, s) and their derivatives
    - ``mzi``  : ``crossing.py:216-221`` (T) and ``crossing.py:223-231`` (dT/dp)
    - ``sym``  : ``crossing.py:377-381`` (T); dT/dp from the same closed form (the reference CPU class
                 has no dT; its GPU counterpart is ``gpu/crossing.cu:90-126``)
    - ``orth`` : ``gpu/crossing.cu:132-148`` and the dense restatement in ``gpu/test.py:70-72``
* nearest-neighbour layers (lens / shifts): ``c/dot.cpp:146-238`` / ``mesh.py:44-60``; slot layout
  ``mesh.py:513-536`` (grid_phase / grid_splitter) and ``gpu/gmem.cu:236-238`` (cond_gen)
* FFT (stride) layers: ``gpu/fwdprop.cu:52-93`` and the oracle in ``gpu/test.py:74-76``
* forward-mode differentiation: ``c/dot.cpp:180-203`` (mode 1)
* back-propagation from the outputs (inverting each unitary layer by T^H and accumulating
  dJ/dT_ij = conj(g_i) x_j): ``c/dot.cpp:70-80, 240-288`` (mode 2) and ``crossing.py:146-163`` for the
  contraction dJ/dp = Re sum_ij dT_ij/dp dJ/dT_ij
* geometries: Clements ``clements.py:56-57``, Reck ``reck.py:47-48``, butterfly ``butterfly.py:47-51``
  (re-expressed as FFT strides)

Parity of this restatement is pinned against the reference itself: ``tests/golden/make_golden.py``
runs the reference's own ``StructuredMeshNetwork.dot`` / ``dot_vjp`` (its ``c/dot.cpp`` compiled from
source into ``oracle/_ref``) on seeded cases and commits the results as fixtures, and
``tests/test_oracle.py`` checks this module against them.

Field layout follows the reference GPU API: a batch of B vectors of N modes, stored (B, N) row-major
(the reference's (N, B) Fortran-order arrays, ``gpu/mesh.py:150-156``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

# (n_p, n_s): gpu/mesh.py:72-73; the lossy generic MZI has 14 splitter entries (crossing.py:448-452)
CROSSINGS = {"mzi": (2, 2), "sym": (2, 1), "orth": (1, 0), "mzi_generic": (2, 14),
             # the reference's other parameterisations (crossing.py:292-357, 384-442, 493-611)
             "mzi_balanced": (2, 2), "mzi_outphase": (2, 2), "mzi3": (2, 3), "mzi3_outphase": (2, 3),
             "mzi_generic_outphase": (2, 14), "cartesian": (2, 2), "bell": (2, 2)}


# ----------------------------------------------------------------------------------------------
# geometries
# ----------------------------------------------------------------------------------------------
def clements_geometry(N: int):
    """lens/shifts of a Clements mesh with N layers (clements.py:56-57)."""
    lens = [(N - n % 2) // 2 for n in range(N)]
    shifts = [n % 2 for n in range(N)]
    return lens, shifts


def reck_geometry(N: int):
    """lens/shifts of a Reck triangle with 2N-3 layers (reck.py:47-48)."""
    shifts = list(range(N - 2, 0, -1)) + list(range(0, N - 1))
    lens = [(N - s) // 2 for s in shifts]
    return lens, shifts


def butterfly_strides(N: int):
    """Stride exponents equivalent to the reference ButterflyNetwork (butterfly.py:47-51).

    The reference sandwiches odd layers i between permutations that bring modes (2sj+k, 2sj+k+s)
    next to each other (s = lowest set bit of i+1); the stride form applies the same MZIs in place.
    """
    assert N == 1 << int(math.log2(N))
    out = []
    for i in range(N - 1):
        if i % 2 == 0:
            out.append(0)
        else:
            x = i + 1
            out.append((x & -x).bit_length() - 1)
    return out


def fft_strides(N: int):
    """Stride exponents 0..log2(N)-1: the classic log-depth FFT mesh."""
    return list(range(int(math.log2(N))))


# ----------------------------------------------------------------------------------------------
# crossings
# ----------------------------------------------------------------------------------------------
def T_mzi(p, s=None):
    """(2, 2, k) complex128; crossing.py:216-221. p (k, 2) = (theta, phi), s (k, 2) = (alpha, beta)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    th, ph = p[:, 0], p[:, 1]
    if s is None:
        a = b = np.zeros_like(th)
    else:
        s = np.asarray(s, dtype=np.float64).reshape(-1, 2)
        a, b = s[:, 0], s[:, 1]
    Cp, Cm, C = np.cos(a + b), np.cos(a - b), np.cos(th / 2)
    Sp, Sm, S = np.sin(a + b), np.sin(a - b), np.sin(th / 2)
    return np.exp(1j * th / 2) * np.array([[np.exp(1j * ph) * (1j * S * Cm - C * Sp), 1j * C * Cp - S * Sm],
                                           [np.exp(1j * ph) * (1j * C * Cp + S * Sm), -1j * S * Cm - C * Sp]])


def dT_mzi(p, s=None):
    """(2, 2, 2, k): d T / d(theta, phi); crossing.py:223-231."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    th, ph = p[:, 0], p[:, 1]
    if s is None:
        a = b = np.zeros_like(th)
    else:
        s = np.asarray(s, dtype=np.float64).reshape(-1, 2)
        a, b = s[:, 0], s[:, 1]
    Cp, Cm, C = np.cos(a + b), np.cos(a - b), np.cos(th / 2)
    Sp, Sm, S = np.sin(a + b), np.sin(a - b), np.sin(th / 2)
    z = 0 * S
    ph_ = np.exp(1j * np.array([[[ph + th / 2, th / 2]]]))
    return ph_ * np.array([[[0.5j * (1j * S * Cm - C * Sp) + 0.5 * (1j * C * Cm + S * Sp),
                             0.5j * (1j * C * Cp - S * Sm) + 0.5 * (-1j * S * Cp - C * Sm)],
                            [0.5j * (1j * C * Cp + S * Sm) + 0.5 * (-1j * S * Cp + C * Sm),
                             0.5j * (-1j * S * Cm - C * Sp) + 0.5 * (-1j * C * Cm + S * Sp)]],
                           [[1j * (1j * S * Cm - C * Sp), z],
                            [1j * (1j * C * Cp + S * Sm), z]]])


def T_sym(p, s=None):
    """(2, 2, k); crossing.py:377-381 (symmetric crossing, one splitter error alpha)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    th, ph = p[:, 0], p[:, 1]
    al = np.zeros_like(th) if s is None else np.asarray(s, dtype=np.float64).reshape(-1)
    C, S, C2a, S2a = np.cos(th / 2), np.sin(th / 2), np.cos(2 * al), np.sin(2 * al)
    return np.array([[np.exp(1j * ph) * (S + 1j * C * S2a), 1j * C * C2a],
                     [1j * C * C2a, np.exp(-1j * ph) * (S - 1j * C * S2a)]])


def dT_sym(p, s=None):
    """(2, 2, 2, k): derivative of T_sym with respect to (theta, phi), from its closed form."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    th, ph = p[:, 0], p[:, 1]
    al = np.zeros_like(th) if s is None else np.asarray(s, dtype=np.float64).reshape(-1)
    C, S, C2a, S2a = np.cos(th / 2), np.sin(th / 2), np.cos(2 * al), np.sin(2 * al)
    z = 0 * S
    e, em = np.exp(1j * ph), np.exp(-1j * ph)
    d_th = 0.5 * np.array([[e * (C - 1j * S * S2a), -1j * S * C2a],
                           [-1j * S * C2a, em * (C + 1j * S * S2a)]])
    d_ph = np.array([[1j * e * (S + 1j * C * S2a), z + 0j],
                     [z + 0j, -1j * em * (S - 1j * C * S2a)]])
    return np.array([d_th, d_ph])


def T_orth(p, s=None):
    """(2, 2, k) real; gpu/crossing.cu:132-148: [[sin th/2, -cos th/2], [cos th/2, sin th/2]]."""
    th = np.asarray(p, dtype=np.float64).reshape(-1)
    C, S = np.cos(th / 2), np.sin(th / 2)
    return np.array([[S, -C], [C, S]])


def dT_orth(p, s=None):
    th = np.asarray(p, dtype=np.float64).reshape(-1)
    C, S = np.cos(th / 2), np.sin(th / 2)
    return 0.5 * np.array([[[C, S], [-S, C]]])


def T_mzi_generic(p, s=None):
    """(2, 2, k) complex128: lossy MZI with phase and gain errors; crossing.py:466-488 (out_phase False).

    p (k, 2) = (theta, phi); s (k, 14) = (alpha, beta, fab phase errors e11, e21, e12, e22, crosstalk
    phase errors x11, x21, x12, x22, log-gains g11, g21, g12, g22).  T = S(beta) D2 S(alpha) D1 with
    D1 = diag(exp(i(phi + e11 + x11) + g11/2), exp(i(e21 + x21) + g21/2)),
    D2 = diag(exp(i(theta + e12 + x12) + g12/2), exp(i(e22 + x22) + g22/2)),
    S(a) = [[cos(pi/4 + a), i sin(pi/4 + a)], [i sin(pi/4 + a), cos(pi/4 + a)]].
    """
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    k = p.shape[0]
    s = np.zeros((k, 14)) if s is None else np.asarray(s, dtype=np.float64).reshape(-1, 14)
    th, ph = p[:, 0], p[:, 1]
    a, b = s[:, 0], s[:, 1]
    e11, e21, e12, e22 = s[:, 2], s[:, 3], s[:, 4], s[:, 5]
    x11, x21, x12, x22 = s[:, 6], s[:, 7], s[:, 8], s[:, 9]
    g11, g21, g12, g22 = s[:, 10], s[:, 11], s[:, 12], s[:, 13]
    d1 = (np.exp(1j * (ph + e11 + x11) + g11 / 2), np.exp(1j * (e21 + x21) + g21 / 2))
    d2 = (np.exp(1j * (th + e12 + x12) + g12 / 2), np.exp(1j * (e22 + x22) + g22 / 2))

    def split(al):
        c, sn = np.cos(np.pi / 4 + al), np.sin(np.pi / 4 + al)
        return np.array([[c, 1j * sn], [1j * sn, c]])

    T = split(a) * np.array([d1[0], d1[1]])[None, :, :]                 # S(alpha) D1
    T = np.array([d2[0], d2[1]])[:, None, :] * T                         # D2 S(alpha) D1
    return np.einsum("ijk,jlk->ilk", split(b), T)                        # S(beta) D2 S(alpha) D1


def dT_mzi_generic(p, s=None):
    """(2, 2, 2, k): derivative of T_mzi_generic with respect to (theta, phi).

    theta enters D2 and phi enters D1 through exp(i.) on their first diagonal entries, so
    dT/dtheta = S(beta) diag(i, 0) D2 S(alpha) D1 and dT/dphi = T diag(i, 0).
    """
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    T = T_mzi_generic(p, s)
    dph = T.copy()
    dph[:, 0] *= 1j
    dph[:, 1] = 0
    # S(beta)^-1 T = D2 S(alpha) D1; scale its first row by i, multiply back by S(beta)
    k = p.shape[0]
    ss = np.zeros((k, 14)) if s is None else np.asarray(s, dtype=np.float64).reshape(-1, 14)
    c, sn = np.cos(np.pi / 4 + ss[:, 1]), np.sin(np.pi / 4 + ss[:, 1])
    Sb = np.array([[c, 1j * sn], [1j * sn, c]])
    Sb_inv = np.array([[c, -1j * sn], [-1j * sn, c]])                   # S(b)^H = S(b)^-1 (real angle)
    inner = np.einsum("ijk,jlk->ilk", Sb_inv, T)
    inner[1] = 0
    inner[0] *= 1j
    dth = np.einsum("ijk,jlk->ilk", Sb, inner)
    return np.array([dth, dph])


def _splits(s, k, n):
    return np.zeros((k, n)) if s is None else np.asarray(s, dtype=np.float64).reshape(k, n)


def _coupler(eta):
    """(2, 2, k) [[cos eta, i sin eta], [i sin eta, cos eta]]."""
    c, sn = np.cos(eta), np.sin(eta)
    return np.array([[c, 1j * sn], [1j * sn, c]])


def _mm(A, B):
    return np.einsum("ijk,jlk->ilk", A, B)


def T_mzi_balanced(p, s=None):
    """crossing.py:301-305: the MZI with +-theta/2 in the arms, T_mzi exp(-i theta/2)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    return T_mzi(p, s) * np.exp(-0.5j * p[:, 0])


def T_mzi_outphase(p, s=None):
    """crossing.py:329-337: phase shifters on the outputs.  T(theta, phi, a, b) is the input-phase MZI with
    splitters (b + pi/2, a - pi/2), both indices reversed and transposed: T[i][j] = T_in[1-j][1-i]."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    ab = _splits(s, p.shape[0], 2)
    Ti = T_mzi(p, np.stack([ab[:, 1] + np.pi / 2, ab[:, 0] - np.pi / 2], 1))
    return Ti[::-1, ::-1].transpose(1, 0, 2)


def T_mzi3(p, s=None):
    """crossing.py:397-416: an extra coupler eta before the MZI, T = T_mzi(a, b) C(eta); s = (a, b, eta)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    sp = _splits(s, p.shape[0], 3)
    return _mm(T_mzi(p, sp[:, :2]), _coupler(sp[:, 2]))


def T_mzi3_outphase(p, s=None):
    """crossing.py:397-406, 425-442: the output-phase MZI followed by the coupler, C(eta) T_out(a, b)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    sp = _splits(s, p.shape[0], 3)
    return _mm(_coupler(sp[:, 2]), T_mzi_outphase(p, sp[:, :2]))


def T_mzi_generic_outphase(p, s=None):
    """crossing.py:476-481 (out_phase True): the generic MZI flipped, T = R(D1) S(alpha) R(D2) S(beta) with
    R(D) the diagonal D with its entries swapped (same parameters as T_mzi_generic)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    k = p.shape[0]
    sp = _splits(s, k, 14)
    th, ph = p[:, 0], p[:, 1]
    d1 = (np.exp(1j * (ph + sp[:, 2] + sp[:, 6]) + sp[:, 10] / 2), np.exp(1j * (sp[:, 3] + sp[:, 7]) + sp[:, 11] / 2))
    d2 = (np.exp(1j * (th + sp[:, 4] + sp[:, 8]) + sp[:, 12] / 2), np.exp(1j * (sp[:, 5] + sp[:, 9]) + sp[:, 13] / 2))
    z = np.zeros(k)
    R1 = np.array([[d1[1], z], [z, d1[0]]])
    R2 = np.array([[d2[1], z], [z, d2[0]]])
    return _mm(R1, _mm(_coupler(np.pi / 4 + sp[:, 0]), _mm(R2, _coupler(np.pi / 4 + sp[:, 1]))))


def T_cartesian(p, s=None):
    """crossing.py:540-544: p = (x, y) in the unit disk around (2, 0) (s = x + iy - 2, T = [[s, i r],
    [i r, s*]]) or around (-2, 0) (t = x + iy + 2, T = [[i r, t], [t*, i r]]), r = sqrt(1 - |.|^2)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    x, y = p[:, 0], p[:, 1]
    right = x > 0
    z = (x + 1j * y) - np.where(right, 2.0, -2.0)
    ir = 1j * np.sqrt(1 - np.abs(z) ** 2)
    return np.array([[np.where(right, z, ir), np.where(right, ir, z)],
                     [np.where(right, ir, z.conj()), np.where(right, z.conj(), ir)]])


def T_bell(p, s=None):
    """crossing.py:590-594: the compressed MZI (phases theta, phi in the two arms between the splitters),
    T = exp(i(theta + phi)/2) [[-C Sp + i Cm S, -Sm S + i Cp C], [Sm S + i Cp C, -C Sp - i Cm S]] with
    C, S = cos, sin((theta - phi)/2), Cp, Sp = cos, sin(a + b), Cm, Sm = cos, sin(a - b)."""
    p = np.asarray(p, dtype=np.float64).reshape(-1, 2)
    th, ph = p[:, 0], p[:, 1]
    ab = _splits(s, p.shape[0], 2)
    a, b = ab[:, 0], ab[:, 1]
    Cp, Cm, C = np.cos(a + b), np.cos(a - b), np.cos((th - ph) / 2)
    Sp, Sm, S = np.sin(a + b), np.sin(a - b), np.sin((th - ph) / 2)
    return np.exp(0.5j * (th + ph)) * np.array([[-C * Sp + 1j * Cm * S, -Sm * S + 1j * Cp * C],
                                                 [Sm * S + 1j * Cp * C, -C * Sp - 1j * Cm * S]])


T_FN = {"mzi": T_mzi, "sym": T_sym, "orth": T_orth, "mzi_generic": T_mzi_generic,
        "mzi_balanced": T_mzi_balanced, "mzi_outphase": T_mzi_outphase, "mzi3": T_mzi3,
        "mzi3_outphase": T_mzi3_outphase, "mzi_generic_outphase": T_mzi_generic_outphase,
        "cartesian": T_cartesian, "bell": T_bell}
DT_FN = {"mzi": dT_mzi, "sym": dT_sym, "orth": dT_orth, "mzi_generic": dT_mzi_generic}


# ----------------------------------------------------------------------------------------------
# mesh description (the reference GPU grid layout: p (L, N/2, n_p), s (L, N/2, n_s))
# ----------------------------------------------------------------------------------------------
@dataclass
class OracleMesh:
    N: int
    L: int
    crossing: str = "mzi"
    lens: Optional[Sequence[int]] = None       # nearest-neighbour geometry
    shifts: Optional[Sequence[int]] = None
    strides: Optional[Sequence[int]] = None    # FFT geometry (stride exponents)
    p: np.ndarray = field(default=None)        # (L, N//2, n_p)
    s: Optional[np.ndarray] = None             # (L, N//2, n_s) or None
    T_override: Optional[np.ndarray] = None    # (L, N//2, 2, 2) complex: generic crossing
    perm: Optional[np.ndarray] = None          # (L+1, N) gather rows between layers (mesh.py:238-277)

    @property
    def fft(self) -> bool:
        return self.strides is not None

    def slots(self, n: int):
        """Active slots of layer n as (q, mode_a, mode_b)."""
        N = self.N
        out = []
        if self.fft:
            st = 1 << int(self.strides[n])
            for q in range(N // 2):
                j, k = divmod(q, st)
                out.append((q, 2 * st * j + k, 2 * st * j + k + st))
        else:
            sh, ln = int(self.shifts[n]), int(self.lens[n])
            for k in range(ln):
                q = sh // 2 + k
                out.append((q, sh + 2 * k, sh + 2 * k + 1))
        return out

    def active_mask(self) -> np.ndarray:
        m = np.zeros((self.L, self.N // 2), dtype=bool)
        for n in range(self.L):
            for q, _, _ in self.slots(n):
                m[n, q] = True
        return m

    def T_grid(self, p=None) -> np.ndarray:
        """(L, N//2, 2, 2) complex128 transfer matrices of every slot."""
        if self.T_override is not None:
            return np.asarray(self.T_override, dtype=np.complex128)
        p = self.p if p is None else p
        n_p, n_s = CROSSINGS[self.crossing]
        pp = np.asarray(p, dtype=np.float64).reshape(-1, n_p)
        ss = None if (self.s is None or n_s == 0) else np.asarray(self.s, dtype=np.float64).reshape(-1, n_s)
        T = T_FN[self.crossing](pp, ss)                     # (2, 2, k)
        return np.moveaxis(T, -1, 0).reshape(self.L, self.N // 2, 2, 2).astype(np.complex128)

    def dT_grid(self, p=None) -> np.ndarray:
        """(L, N//2, n_p, 2, 2): dT/dp for every slot."""
        p = self.p if p is None else p
        n_p, n_s = CROSSINGS[self.crossing]
        pp = np.asarray(p, dtype=np.float64).reshape(-1, n_p)
        ss = None if (self.s is None or n_s == 0) else np.asarray(self.s, dtype=np.float64).reshape(-1, n_s)
        D = DT_FN[self.crossing](pp, ss)                    # (n_p, 2, 2, k)
        return np.moveaxis(D, -1, 0).reshape(self.L, self.N // 2, n_p, 2, 2).astype(np.complex128)


# ----------------------------------------------------------------------------------------------
# propagation (complex128)
# ----------------------------------------------------------------------------------------------
def _layer_index(mesh: OracleMesh, n: int):
    """(q, a, b) index arrays of the active slots of layer n (cached on the mesh)."""
    cache = mesh.__dict__.setdefault("_idx_cache", {})
    if n not in cache:
        sl = mesh.slots(n)
        if sl:
            q, a, b = (np.array(x, dtype=np.int64) for x in zip(*sl))
        else:
            q = a = b = np.zeros(0, dtype=np.int64)
        cache[n] = (q, a, b)
    return cache[n]


def _gather(mesh: OracleMesh, k: int, *fields, inverse=False):
    """Fields (N, B) <- rows permuted by perm[k] (c/dot.cpp:29-40: new[q] = old[perm[q]]), or by its
    inverse argsort(perm[k]) (the reference's perms_bk, mesh.py:382)."""
    if mesh.perm is None:
        return
    row = np.asarray(mesh.perm[k])
    if inverse:
        row = np.argsort(row)
    for f in fields:
        f[:] = f[row]


def _apply_layer(mesh: OracleMesh, n: int, T: np.ndarray, u: np.ndarray, conj_transpose=False):
    """u <- T_n u for every active slot of layer n (vectorised over the slots of the layer)."""
    q, a, b = _layer_index(mesh, n)
    if q.size == 0:
        return
    t = T[n, q][:, :, :, None]                      # (k, 2, 2, 1) broadcast over the batch
    if conj_transpose:
        t = np.conj(np.swapaxes(t, 1, 2))
    ua, ub = u[a], u[b]                             # u is (N, B): rows are modes
    u[a] = t[:, 0, 0] * ua + t[:, 0, 1] * ub
    u[b] = t[:, 1, 0] * ua + t[:, 1, 1] * ub


def propagate(mesh: OracleMesh, x: np.ndarray, p=None) -> np.ndarray:
    """y = U x for a batch x (B, N); c/dot.cpp:146-238 (mode 0)."""
    T = mesh.T_grid(p)
    dt = np.float64 if mesh.crossing == "orth" and mesh.T_override is None else np.complex128
    u = np.array(x, dtype=dt if np.isrealobj(x) and dt == np.float64 else np.complex128)
    if u.dtype == np.float64:
        T = T.real
    u = np.ascontiguousarray(u.T)
    for n in range(mesh.L):
        _gather(mesh, n, u)                 # c/dot.cpp:150-153
        _apply_layer(mesh, n, T, u)
    _gather(mesh, mesh.L, u)                # c/dot.cpp:289-292
    return np.ascontiguousarray(u.T)


def propagate_activations(mesh: OracleMesh, x: np.ndarray, p=None):
    """Input of every layer (after the permutation before it) and the output: list of L+1 arrays."""
    T = mesh.T_grid(p)
    u = np.array(x, dtype=np.float64 if np.isrealobj(x) else np.complex128)
    if u.dtype == np.float64:
        T = T.real
    u = np.ascontiguousarray(u.T)
    acts = []
    for n in range(mesh.L):
        _gather(mesh, n, u)
        acts.append(u.T.copy())
        _apply_layer(mesh, n, T, u)
    _gather(mesh, mesh.L, u)
    acts.append(u.T.copy())
    return acts


def fwddiff(mesh: OracleMesh, x: np.ndarray, dp: np.ndarray, dx: Optional[np.ndarray] = None, p=None):
    """Forward-mode derivative along dp: returns (y, dy); c/dot.cpp:180-203 (mode 1)."""
    T = mesh.T_grid(p)
    D = mesh.dT_grid(p)                                     # (L, Q, n_p, 2, 2)
    n_p = D.shape[2]
    dT = np.einsum("lqkij,lqk->lqij", D, np.asarray(dp, np.float64).reshape(mesh.L, mesh.N // 2, n_p))
    real = np.isrealobj(x) and mesh.crossing == "orth"
    dt = np.float64 if real else np.complex128
    u = np.array(x, dtype=dt)
    du = np.zeros_like(u) if dx is None else np.array(dx, dtype=dt)
    if real:
        T, dT = T.real, dT.real
    u, du = np.ascontiguousarray(u.T), np.ascontiguousarray(du.T)
    for n in range(mesh.L):
        _gather(mesh, n, u, du)
        q, a, b = _layer_index(mesh, n)
        if q.size == 0:
            continue
        t, d = T[n, q][:, :, :, None], dT[n, q][:, :, :, None]
        ua, ub, dua, dub = u[a], u[b], du[a], du[b]
        du[a] = t[:, 0, 0] * dua + t[:, 0, 1] * dub + d[:, 0, 0] * ua + d[:, 0, 1] * ub
        du[b] = t[:, 1, 0] * dua + t[:, 1, 1] * dub + d[:, 1, 0] * ua + d[:, 1, 1] * ub
        u[a] = t[:, 0, 0] * ua + t[:, 0, 1] * ub
        u[b] = t[:, 1, 0] * ua + t[:, 1, 1] * ub
    _gather(mesh, mesh.L, u, du)
    return np.ascontiguousarray(u.T), np.ascontiguousarray(du.T)


def vjp_unitary(mesh: OracleMesh, y: np.ndarray, g: np.ndarray, p=None):
    """Back-propagation from the OUTPUTS (y, g = dJ/dy*·2) by inverting each layer with T^H.

    Returns (G, x, g_in): G (L, N//2, 2, 2) the per-slot dJ/dT_ij = sum_b conj(g_i) x_j, the
    reconstructed input x and the input gradient g_in = U^H g.  Valid for unitary crossings only,
    exactly as the reference (c/dot.cpp:70-80, 240-288; gpu/backdiff.cu).
    """
    T = mesh.T_grid(p)
    real = np.isrealobj(y) and mesh.crossing == "orth"
    dt = np.float64 if real else np.complex128
    if real:
        T = T.real
    u = np.array(y, dtype=dt)
    gg = np.array(g, dtype=dt)
    G = np.zeros((mesh.L, mesh.N // 2, 2, 2), dtype=dt)
    u, gg = np.ascontiguousarray(u.T), np.ascontiguousarray(gg.T)
    for n in range(mesh.L - 1, -1, -1):
        _gather(mesh, n + 1, u, gg, inverse=True)          # c/dot.cpp:150-153 with perms_bk
        q, a, b = _layer_index(mesh, n)
        if q.size == 0:
            continue
        th = np.conj(np.swapaxes(T[n, q], -1, -2))[:, :, :, None]
        ua, ub = u[a], u[b]
        xa = th[:, 0, 0] * ua + th[:, 0, 1] * ub
        xb = th[:, 1, 0] * ua + th[:, 1, 1] * ub
        u[a], u[b] = xa, xb
        ga, gb = gg[a], gg[b]
        G[n, q, 0, 0] = np.sum(ga.conj() * xa, axis=1)
        G[n, q, 0, 1] = np.sum(ga.conj() * xb, axis=1)
        G[n, q, 1, 0] = np.sum(gb.conj() * xa, axis=1)
        G[n, q, 1, 1] = np.sum(gb.conj() * xb, axis=1)
        gg[a] = th[:, 0, 0] * ga + th[:, 0, 1] * gb
        gg[b] = th[:, 1, 0] * ga + th[:, 1, 1] * gb
    _gather(mesh, 0, u, gg, inverse=True)
    return G, np.ascontiguousarray(u.T), np.ascontiguousarray(gg.T)


def vjp_stored(mesh: OracleMesh, x: np.ndarray, g: np.ndarray, p=None):
    """Adjoint with stored activations (valid for lossy, non-unitary T too).

    Returns (G, g_in) with G_ij = sum_b conj(g_i) x_j taken at each layer's input and g_in = U^H g.
    """
    T = mesh.T_grid(p)
    acts = propagate_activations(mesh, x, p)
    real = np.isrealobj(x) and mesh.crossing == "orth"
    if real:
        T = T.real
    gg = np.array(g, dtype=np.float64 if real else np.complex128)
    G = np.zeros((mesh.L, mesh.N // 2, 2, 2), dtype=gg.dtype)
    gg = np.ascontiguousarray(gg.T)
    for n in range(mesh.L - 1, -1, -1):
        _gather(mesh, n + 1, gg, inverse=True)
        q, a, b = _layer_index(mesh, n)
        if q.size == 0:
            continue
        xin = acts[n].T
        th = np.conj(np.swapaxes(T[n, q], -1, -2))[:, :, :, None]
        ga, gb = gg[a], gg[b]
        xa, xb = xin[a], xin[b]
        G[n, q, 0, 0] = np.sum(ga.conj() * xa, axis=1)
        G[n, q, 0, 1] = np.sum(ga.conj() * xb, axis=1)
        G[n, q, 1, 0] = np.sum(gb.conj() * xa, axis=1)
        G[n, q, 1, 1] = np.sum(gb.conj() * xb, axis=1)
        gg[a] = th[:, 0, 0] * ga + th[:, 0, 1] * gb
        gg[b] = th[:, 1, 0] * ga + th[:, 1, 1] * gb
    _gather(mesh, 0, gg, inverse=True)
    return G, np.ascontiguousarray(gg.T)


# ----------------------------------------------------------------------------------------------
# phase screen (is_phase / phi_pos; the screen step of c/dot.cpp:97-143): y = D U x for pos "out",
# y = U D x for pos "in", D = diag(exp(i ph)) over the N modes
# ----------------------------------------------------------------------------------------------
def screen(v: np.ndarray, ph, sign: int = 1) -> np.ndarray:
    """v (B, N) times exp(i sign ph) per mode."""
    return np.asarray(v, dtype=np.complex128) * np.exp(1j * sign * np.asarray(ph, dtype=np.float64))[None, :]


def propagate_screened(mesh: OracleMesh, x: np.ndarray, ph, pos: str, p=None) -> np.ndarray:
    if pos == "in":
        return propagate(mesh, screen(x, ph), p)
    return screen(propagate(mesh, x, p), ph)


def fwddiff_screened(mesh: OracleMesh, x, ph, pos: str, dp, dph, dx=None, p=None):
    """(y, dy) along (dp, dph): the screen contributes d(exp(i ph) u) = exp(i ph) du + i dph exp(i ph) u."""
    dph = np.asarray(dph, dtype=np.float64)
    dx = np.zeros_like(np.asarray(x, dtype=np.complex128)) if dx is None else np.asarray(dx, np.complex128)
    if pos == "in":
        u = screen(x, ph)
        du = screen(dx, ph) + 1j * dph[None, :] * u
        return fwddiff(mesh, u, dp, du, p)
    y, dy = fwddiff(mesh, x, dp, dx, p)
    y2 = screen(y, ph)
    return y2, screen(dy, ph) + 1j * dph[None, :] * y2


def grad_screened(mesh: OracleMesh, y, g, ph, pos: str, p=None):
    """From the outputs (y, g = 2 dJ/dy*): (dJ/dp grid, dJ/dph, g_in), unitary mesh.
    dJ/dph_k = sum_b Re(conj(g_k) i u_k) with (u, g) taken just after the screen."""
    def dph_of(u, gg):
        return np.real(np.sum(np.conj(gg) * 1j * u, axis=0))
    if pos == "out":
        dph = dph_of(y, g)
        G, _, gin = vjp_unitary(mesh, screen(y, ph, -1), screen(g, ph, -1), p)
        return contract_dp(mesh, G, p), dph, gin
    G, u, gin_m = vjp_unitary(mesh, y, g, p)
    return contract_dp(mesh, G, p), dph_of(u, gin_m), screen(gin_m, ph, -1)


def contract_dp(mesh: OracleMesh, G: np.ndarray, p=None) -> np.ndarray:
    """dJ/dp (L, N//2, n_p) = Re sum_ij dT_ij/dp G_ij; crossing.py:146-163.  Inactive slots are 0."""
    D = mesh.dT_grid(p)
    dp = np.real(np.einsum("lqkij,lqij->lqk", D, G))
    dp[~mesh.active_mask()] = 0.0
    return dp


def grad(mesh: OracleMesh, x: np.ndarray, g_of_y, p=None, unitary=True):
    """Convenience: forward, gradient callback on y, backward. Returns (y, dp, g_in)."""
    y = propagate(mesh, x, p)
    g = g_of_y(y)
    if unitary:
        G, _, g_in = vjp_unitary(mesh, y, g, p)
    else:
        G, g_in = vjp_stored(mesh, x, g, p)
    return y, contract_dp(mesh, G, p), g_in


def central_difference(loss_of_p, p: np.ndarray, idx, h=1e-6):
    """complex128 central differences of a scalar loss at flat parameter indices idx."""
    p = np.array(p, dtype=np.float64)
    flat = p.reshape(-1)
    out = []
    for i in idx:
        old = flat[i]
        flat[i] = old + h
        jp = loss_of_p(p)
        flat[i] = old - h
        jm = loss_of_p(p)
        flat[i] = old
        out.append((jp - jm) / (2 * h))
    return np.array(out)


def matrix(mesh: OracleMesh, p=None) -> np.ndarray:
    """Transfer matrix U (N, N) with y = U x."""
    eye = np.eye(mesh.N, dtype=np.float64 if mesh.crossing == "orth" else np.complex128)
    return propagate(mesh, eye, p).T


def unitarity_error(mesh: OracleMesh, p=None) -> float:
    U = matrix(mesh, p)
    return float(np.linalg.norm(U @ U.conj().T - np.eye(mesh.N)))


def rel_err(a, b) -> float:
    """Relative Frobenius error ||a - b|| / ||b||."""
    a = np.asarray(a)
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


# ----------------------------------------------------------------------------------------------
# conversions between the reference's flat CPU parameters and the GPU grid
# ----------------------------------------------------------------------------------------------
def flat_to_grid(flat: np.ndarray, lens, shifts, N: int, n: int) -> np.ndarray:
    """p_crossing (n_cr, n) -> grid (L, N//2, n) with zeros in inactive slots (mesh.py:513-536 with
    NaN -> 0 as in mesh.py:575-576)."""
    L = len(lens)
    flat = np.asarray(flat).reshape(-1, n)
    out = np.zeros((L, N // 2, n), dtype=flat.dtype)
    ind = 0
    for l, (ln, sh) in enumerate(zip(lens, shifts)):
        out[l, sh // 2: sh // 2 + ln] = flat[ind: ind + ln]
        ind += ln
    return out


def grid_to_flat(grid: np.ndarray, lens, shifts) -> np.ndarray:
    rows = []
    for l, (ln, sh) in enumerate(zip(lens, shifts)):
        rows.append(grid[l, sh // 2: sh // 2 + ln])
    return np.concatenate(rows, 0)


# ----------------------------------------------------------------------------------------------
# seeded synthetic inputs (seed = 1000 + config index)
# ----------------------------------------------------------------------------------------------
def unit_columns(rng, N, B, real=False):
    """(B, N): each vector iid N(0,1) (complex: real and imaginary parts) normalised to unit norm."""
    x = rng.standard_normal((B, N))
    if not real:
        x = x + 1j * rng.standard_normal((B, N))
    return x / np.linalg.norm(x, axis=1, keepdims=True)


def random_mesh(rng, N, geometry="clements", crossing="mzi", splitter_sigma=0.0, dtype=np.float32):
    if geometry == "clements":
        lens, shifts = clements_geometry(N)
        strides = None
    elif geometry == "reck":
        lens, shifts = reck_geometry(N)
        strides = None
    elif geometry == "butterfly":
        lens = shifts = None
        strides = butterfly_strides(N)
    elif geometry == "fft":
        lens = shifts = None
        strides = fft_strides(N)
    else:
        raise ValueError(geometry)
    L = len(strides) if strides is not None else len(lens)
    n_p, n_s = CROSSINGS[crossing]
    p = rng.uniform(0, 2 * np.pi, (L, N // 2, n_p)).astype(dtype)
    s = rng.normal(0, splitter_sigma, (L, N // 2, n_s)).astype(dtype) if (splitter_sigma and n_s) else None
    m = OracleMesh(N=N, L=L, crossing=crossing, lens=lens, shifts=shifts, strides=strides, p=p, s=s)
    if strides is None:
        mask = m.active_mask()
        p[~mask] = 0
        if s is not None:
            s[~mask] = 0
    return m


def haar_unitary(rng, N):
    """Haar-random unitary: QR of a complex Gaussian with the R-diagonal phase correction."""
    Z = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))) / math.sqrt(2)
    Q, R = np.linalg.qr(Z)
    d = np.diag(R)
    return Q * (d / np.abs(d))
