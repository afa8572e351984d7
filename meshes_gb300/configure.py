"""Self-configuration of MZI meshes by matrix diagonalisation (reference configure.py:187-330, ``diag``).

``diag(m1, m2, phi_diag, U, nm, nn, ijxyp, improved)`` programs a left mesh m1 and a right mesh m2 (either may
be None) and a diagonal phase screen so that they realise the target U, with the reference's arguments:
``nm`` groups of ``nn(m)`` nulling steps, ``ijxyp(m, n)`` giving the matrix element (i, j) that step n of
group m zeroes, the MZI at layer x and top mode y that does it and the mesh p (0: m1, 1: m2), and
``improved`` selecting the reference's improved update (``diag*``).  The meshes are ``MeshNetworkGPU``
objects with MZI crossings (nearest-neighbour layers); their phases are written in place.

Work split:
  * the meshes' matrices at their random starting phases are evaluated on the GPU by the propagation
    kernels (the columns of the running product Z propagated through each mesh: ``Z = m.dot(Z)``);
  * the nulling pass itself - one MZI at a time, each step a 10-iteration line search on a 2x2 problem and an
    update of two rows of N x N matrices - is sequential and O(N) per step, and runs natively on the host in
    double precision (``mg_diag_configure`` in libmeshes_gb300, the counterpart of the reference's
    JIT-compiled helper).

Random draws follow the reference's order on NumPy's global generator (``np.random.rand`` for each mesh's
starting phi, ``np.random.randint`` for the line-search starting points, ``np.random.randn`` for the
programming noise ``sigp``), so a seeded call reproduces the reference's programmed phases.

``reck(U, ...)`` and ``diag_reck(mesh, U, improved)`` are the Reck entry points (reference reck.py:68-72,
146-164, ``ReckNetwork(M=U, method='diag' | 'diag*')``); ``square(M, ...)`` programs a SquareNet
(square.py:77-101, ``SquareNetwork(M=M, method='diag')``) into a clipped mesh.

The direct method (reference configure.py:333-410, ``direct``) programs a mesh of output-phase MZIs with its
phase screen at the input diagonal by diagonal from the target's columns, in closed form; it needs no
propagation, so it runs entirely in the native host pass ``mg_direct_configure``, and the programmed mesh
(a ``GenericMeshGPU`` of ``mzi_outphase`` crossings) propagates on the GPU.  ``reck(U, method='direct')`` and
``square(M, method='direct')`` are its entry points (reck.py:69-74, square.py:65-66,103-113).
"""
from __future__ import annotations

import ctypes
from typing import Callable, Optional

import numpy as np
import torch

from . import geometry as geom
from ._lib import check, load
from .mesh import MeshNetworkGPU

# line-search starting points of the MZI crossings (configure.py:176-182): (pi/2, 0) or (-pi/2, 0)
INIT_P, INIT_M = np.array([np.pi / 2, 0.0]), np.array([-np.pi / 2, 0.0])
_c_double_p = ctypes.POINTER(ctypes.c_double)


def _flat_layout(lens, shifts):
    """(layer, slot) of every MZI in the reference's flat order (layer by layer, top to bottom)."""
    lay = np.concatenate([np.full(ln, l) for l, ln in enumerate(lens)]).astype(np.int64) if sum(lens) else np.zeros(0, np.int64)
    slot = np.concatenate([sh // 2 + np.arange(ln) for ln, sh in zip(lens, shifts)]).astype(np.int64) if sum(lens) else lay
    return lay, slot


def diag_steps(geo1, geo2, nm: int, nn: Callable, ijxyp: Callable):
    """The steps (i, j, ind, p) of the nulling pass (configure.py:221-225); geo = (lens, shifts) of m1 and m2
    (empty for a missing mesh).  Returns ijzp (K, 4) int32 and the layer/mode arrays x, y."""
    i, j, x, y, r = np.concatenate([np.array(ijxyp(np.repeat(m, nn(m)), np.arange(nn(m)))) for m in range(nm)], 1)
    i1, s1 = np.cumsum([0] + list(geo1[0])), np.array(geo1[1], dtype=np.int64)
    i2, s2 = np.cumsum([0] + list(geo2[0])), np.array(geo2[1], dtype=np.int64)
    L2 = len(geo2[0])
    w1, w2 = np.where(1 - r)[0], np.where(r)[0]
    x1, y1, x2, y2 = x[w1], y[w1], x[w2] + L2 - 1, y[w2]
    ind = x * 0
    ind[w1] = i1[x1] + (y1 - s1[x1]) // 2
    ind[w2] = i2[x2] + (y2 - s2[x2]) // 2
    return np.ascontiguousarray(np.array([i, j, ind, r]).T, dtype=np.int32), x, y


def diag_init(init, x, y, K: int) -> np.ndarray:
    """Line-search starting points per step (configure.py:227-232): init is 'rand', 'uniform' or a callable
    of (x, y) giving 1 (start at +pi/2) or 0 (start at -pi/2) per step."""
    if callable(init):
        init = init(x, y)
    elif isinstance(init, str) and init == "rand":
        init = np.random.randint(0, 2, K)
    elif isinstance(init, str) and init == "uniform":
        init = np.ones(K, dtype=int)
    else:
        raise ValueError(init)
    init = np.asarray(init)
    if init.ndim == 1:
        init = np.outer(init, INIT_P) + np.outer(1 - init, INIT_M)
    return np.ascontiguousarray(init, dtype=np.float64)


def diag_core(U, Z, s1, c1, s2, c2, ijzp, init, noise, improved: bool, type1: int = 0, type2: int = 1):
    """The nulling pass on the host (mg_diag_configure) from the starting product Z of the meshes' matrices.
    c1, c2 ((n, 2) float64 (theta, phi) in the reference's flat order) are updated in place; returns
    (U, VdV, WWd) as the pass leaves them and the diagonal phases phi_diag (configure.py:246)."""
    N = U.shape[0]
    Ub = np.array(U, dtype=np.complex128, order="C")
    Zb = np.array(Z, dtype=np.complex128, order="C")
    VdV = np.eye(N, dtype=np.complex128)
    WWd = np.eye(N, dtype=np.complex128)
    s1 = np.ascontiguousarray(s1, dtype=np.float64).reshape(-1, 2)
    s2 = np.ascontiguousarray(s2, dtype=np.float64).reshape(-1, 2)
    assert c1.dtype == np.float64 and c1.flags.c_contiguous and c2.dtype == np.float64 and c2.flags.c_contiguous
    assert len(s1) == len(c1) and len(s2) == len(c2)
    ijzp = np.ascontiguousarray(ijzp, dtype=np.int32)
    init = np.ascontiguousarray(init, dtype=np.float64)
    noise_p = None if noise is None else np.ascontiguousarray(noise, dtype=np.float64)
    lib = load()
    ptr = lambda a: None if a is None else a.ctypes.data
    check(lib.mg_diag_configure(N, len(ijzp), ptr(Ub), ptr(Zb), ptr(VdV), ptr(WWd), len(c1), ptr(s1), ptr(c1), type1,
                                len(c2), ptr(s2), ptr(c2), type2, ptr(ijzp), ptr(init), ptr(noise_p), int(improved)),
          "mg_diag_configure")
    phi_diag = np.angle(np.diag(Ub)) - np.angle(np.sum(VdV * WWd.T, axis=1))
    return Ub, VdV, WWd, phi_diag


def _mesh_state(m: Optional[MeshNetworkGPU]):
    """(lens, shifts), flat layout and flat splitters (n, 2) float64 of a mesh (empty for None)."""
    if m is None:
        return ([], []), (np.zeros(0, np.int64), np.zeros(0, np.int64)), np.zeros((0, 2))
    if m.X != "mzi" or m.geometry != geom_nn():
        raise ValueError("self-configuration programs nearest-neighbour meshes of MZI crossings")
    if m.perm_table is not None:
        raise ValueError("self-configuration takes meshes without permutations")
    lay, slot = _flat_layout(m.lens_h, m.shifts_h)
    sp = m.p_splitter
    s = (sp.detach().double().cpu().numpy()[lay, slot] if sp.numel() else np.zeros((len(lay), 2)))
    return (m.lens_h, m.shifts_h), (lay, slot), s


def geom_nn():
    from ._lib import GEO_NN
    return GEO_NN


def _set_phases(m: MeshNetworkGPU, layout, c: np.ndarray):
    """Write flat (theta, phi) into the mesh's grid (zeros in inactive slots); a phase screen is set to 0."""
    lay, slot = layout
    grid = np.zeros((m.L, m.N // 2, 2))
    grid[lay, slot] = c
    new = np.concatenate([grid.reshape(-1), np.zeros(m.N if m.is_phase else 0)])
    m.p_phase.copy_(torch.as_tensor(new, dtype=torch.float32))


def _set_screen(m: MeshNetworkGPU, phi):
    m.p_phase[m.L * (m.N // 2) * 2:].copy_(torch.as_tensor(np.asarray(phi), dtype=torch.float32))


def diag(m1: Optional[MeshNetworkGPU], m2: Optional[MeshNetworkGPU], phi_diag, U, nm: int, nn: Callable,
         ijxyp: Callable, improved: bool, sigp: float = 0.0, init="rand"):
    """Program m1 (left), m2 (right) and the diagonal phases phi_diag (written in place) to realise U; the
    reference's diag (configure.py:187-246), see the module docstring."""
    assert m1 is not None or m2 is not None
    U = np.asarray(U, dtype=np.complex128)
    N = (m1 or m2).N
    assert U.shape == (N, N)
    geo1, lay1, s1 = _mesh_state(m1)
    geo2, lay2, s2 = _mesh_state(m2)
    dev = (m1 or m2).device
    # starting point: theta = 0, phi uniform random, no screen; Z = M2 M1 evaluated on the GPU
    c = []
    Zd = torch.eye(N, dtype=torch.complex64, device=dev)
    for m, lay in ((m1, lay1), (m2, lay2)):
        n = len(lay[0])
        cm = np.zeros((n, 2))
        cm[:, 1] = 2 * np.pi * np.random.rand(n)
        c.append(cm)
        if m is not None:
            _set_phases(m, lay, cm)
            Zd = m.dot(Zd)
    Z = Zd.cpu().numpy().astype(np.complex128)
    ijzp, x, y = diag_steps(geo1, geo2, nm, nn, ijxyp)
    init_arr = diag_init(init, x, y, len(ijzp))
    noise = np.random.randn(len(ijzp), 2) * sigp          # drawn as the reference draws it, one pair per step
    _, _, _, ph = diag_core(U, Z, s1, c[0], s2, c[1], ijzp, init_arr, noise if sigp else None, improved)
    for m, lay, cm in ((m1, lay1, c[0]), (m2, lay2, c[1])):
        if m is not None:
            _set_phases(m, lay, cm)
    if isinstance(phi_diag, torch.Tensor):
        phi_diag.copy_(torch.as_tensor(ph, dtype=phi_diag.dtype))
    else:
        phi_diag[:] = ph
    return ph


def reck_steps(N: int):
    """nn and ijxyp of the Reck mesh with its screen at the output (reference reck.py:155-160)."""
    def nn(m):
        return N - 1 - m

    def ijxyp(m, n):
        return [m, N - 1 - n, m * 2 + n, N - 2 - n, m * 0]
    return nn, ijxyp


def diag_reck(mesh: MeshNetworkGPU, U, improved: bool = True, sigp: float = 0.0, init="rand"):
    """Program a Reck MeshNetworkGPU (screen at the output) to realise U (reference diagReck, reck.py:146-160):
    its crossing phases and its phase screen are written in place."""
    N = mesh.N
    if not (mesh.is_phase and mesh.phi_pos == "out"):
        raise ValueError("the Reck diagonalisation programs a mesh with its phase screen at the output")
    nn, ijxyp = reck_steps(N)
    phi = np.zeros(N)
    diag(mesh, None, phi, U, N - 1, nn, ijxyp, improved, sigp, init)
    _set_screen(mesh, phi)
    return mesh


def reck(U, p_splitter=0.0, improved: bool = True, sigp: float = 0.0, init="rand", device=None,
         method: Optional[str] = None):
    """A Reck mesh realising U (reference ReckNetwork(M=U, p_splitter=..., method=...), reck.py:68-74):
    p_splitter is a scalar or (N(N-1)/2, 2) splitting errors in the reference's flat order.  method 'diag*'
    (or improved=True) and 'diag' return a MeshNetworkGPU with its screen at the output; 'direct' returns the
    reference's phi_pos='in' mesh of output-phase MZIs as a GenericMeshGPU."""
    if method is not None:
        if method not in ("diag", "diag*", "direct"):
            raise ValueError("method must be 'diag', 'diag*' or 'direct'")
        if method == "direct":
            return reck_direct(U, p_splitter, device)
        improved = method == "diag*"
    U = np.asarray(U, dtype=np.complex128)
    N = U.shape[0]
    lens, shifts = geom.reck(N)
    lay = _flat_layout(lens, shifts)
    s = np.zeros((len(lay[0]), 2)) + np.asarray(p_splitter, dtype=np.float64)
    grid = np.zeros((len(lens), N // 2, 2))
    grid[lay[0], lay[1]] = s
    m = MeshNetworkGPU(N, len(lens), lens, shifts, np.zeros(len(lens) * (N // 2) * 2 + N), grid.astype(np.float32),
                       "mzi", phi_pos="out", is_phase=True, device=device)
    return diag_reck(m, U, improved, sigp, init)


def square(M, p_splitter=0.0, eig: Optional[float] = None, improved: bool = False, init="rand", device=None,
           method: str = "diag"):
    """A SquareNet (square.py:22-101, SquareNetwork(M=M, method='diag'), screen at the output) realising the
    (m, n) matrix M, returned as a ClippedMeshGPU over its (m + n)-mode diamond mesh, and the scale factor the
    reference applies to M first (1, or sqrt(eig / max eigenvalue of M M^H) when eig is given).  method='direct'
    is SquareNetwork(M=M, method='direct', phi_pos='in') (square.py:103-113): the full mesh is then a
    GenericMeshGPU of output-phase MZIs with its screen at the input."""
    from scipy.linalg import eigvalsh

    from .clipped import ClippedMeshGPU
    if method == "direct":
        return square_direct(M, p_splitter, eig, device)
    if method not in ("diag", "diag*"):
        raise ValueError("method must be 'diag', 'diag*' or 'direct'")
    improved = improved or method == "diag*"
    M11 = np.array(M, dtype=np.complex128)
    m_out, n_in = M11.shape
    Nf = m_out + n_in
    shifts = np.abs(np.arange(-n_in + 1, m_out))
    lens = (Nf - shifts - shifts[::-1]) // 2
    MMt = M11 @ M11.conj().T
    fact = np.sqrt(eig / eigvalsh(MMt, subset_by_index=[m_out - 1, m_out - 1])[0]) if eig else 1.0
    MMt = MMt * fact ** 2
    M11 = M11 * fact
    M12 = np.linalg.cholesky(np.eye(m_out) - MMt)
    U = np.zeros((Nf, Nf), dtype=np.complex128)
    U[:m_out, :n_in] = M11
    U[:m_out, n_in:] = M12
    lay = _flat_layout(lens.tolist(), shifts.tolist())
    s = np.zeros((len(lay[0]), 2)) + np.asarray(p_splitter, dtype=np.float64)
    grid = np.zeros((len(lens), Nf // 2, 2))
    grid[lay[0], lay[1]] = s
    full = MeshNetworkGPU(Nf, len(lens), lens, shifts, np.zeros(len(lens) * (Nf // 2) * 2 + Nf),
                          grid.astype(np.float32), "mzi", phi_pos="out", is_phase=True, device=device)

    def nn(m):
        return n_in

    def ijxyp(m, n):
        return [m, n_in + m - n, m + n, n_in - 1 + m - n, m * 0]

    phi = np.zeros(Nf)
    diag(full, None, phi, U, m_out, nn, ijxyp, improved, 0.0, init)
    _set_screen(full, phi)
    return ClippedMeshGPU(full, slice(n_in), slice(m_out)), fact


# ---- the direct method

def direct_core(N: int, lens, shifts, U, s_flat, p_flat=None, dk_max: int = 1):
    """The direct method's host pass (mg_direct_configure): (theta, phi) of every crossing (n_cr, 2) in the
    reference's flat order and the input screen (N,), for a nearest-neighbour mesh (lens, shifts) of output-phase
    MZIs with splitting errors s_flat (n_cr, 2); p_flat holds the starting phases (zeros if None), kept for the
    crossings no diagonal reaches."""
    lens = np.ascontiguousarray(lens, dtype=np.int32)
    shifts = np.ascontiguousarray(shifts, dtype=np.int32)
    n_cr = int(lens.sum())
    Ub = np.ascontiguousarray(np.asarray(U, dtype=np.complex128))
    if Ub.shape != (N, N):
        raise ValueError("U must be %d x %d" % (N, N))
    s = np.ascontiguousarray(np.broadcast_to(np.asarray(s_flat, dtype=np.float64), (n_cr, 2)))
    p = np.zeros((n_cr, 2)) if p_flat is None else np.array(p_flat, dtype=np.float64).reshape(n_cr, 2)
    phi = np.zeros(N)

    def ptr(a):
        return a.ctypes.data_as(ctypes.c_void_p)
    check(load().mg_direct_configure(N, len(lens), ptr(lens), ptr(shifts), ptr(Ub), ptr(s), ptr(p), ptr(phi),
                                     int(dk_max)), "mg_direct_configure")
    return p, phi


def direct(mesh, U, diag: str = "down", dk_max: int = 1):
    """Program mesh (a GenericMeshGPU of 'mzi_outphase' crossings, nearest-neighbour, phase screen at the input) to
    realise U by the direct method (reference configure.py:333-368, direct(m, U, 'down', dk_max)); its crossing
    phases and screen are written in place.  The reference's 'up' form flips an output-screen mesh and programs
    the flipped one; no caller of the reference uses it, and it is not provided."""
    from .lossy import GenericMeshGPU
    if diag != "down":
        raise NotImplementedError("only the 'down' diagonals (the form Reck and SquareNet meshes use)")
    if not isinstance(mesh, GenericMeshGPU) or mesh.X != "mzi_outphase" or not mesh.is_phase or mesh.phi_pos != "in":
        raise ValueError("the direct method programs a GenericMeshGPU of 'mzi_outphase' crossings with its phase "
                         "screen at the input")
    lm = mesh.mesh
    if lm.geometry != geom_nn():
        raise ValueError("the direct method programs nearest-neighbour meshes")
    N, L = mesh.N, mesh.L
    lay, slot = _flat_layout(lm.lens_h, lm.shifts_h)
    n_cr = len(lay)
    s = (mesh.p_splitter.detach().cpu().numpy()[lay, slot] if mesh.p_splitter is not None else np.zeros((n_cr, 2)))
    grid = mesh.p_phase[:L * (N // 2) * 2].detach().cpu().numpy().reshape(L, N // 2, 2)
    p, phi = direct_core(N, lm.lens_h, lm.shifts_h, U, s, grid[lay, slot], dk_max)
    grid = np.zeros((L, N // 2, 2))
    grid[lay, slot] = p
    mesh.p_phase.copy_(torch.as_tensor(np.concatenate([grid.reshape(-1), phi]), dtype=mesh.p_phase.dtype))
    return mesh


def _outphase_mesh(N, lens, shifts, p_splitter, device):
    from .lossy import GenericMeshGPU
    lay = _flat_layout(list(lens), list(shifts))
    s = np.zeros((len(lay[0]), 2)) + np.asarray(p_splitter, dtype=np.float64)
    grid = np.zeros((len(lens), N // 2, 2))
    grid[lay[0], lay[1]] = s
    return GenericMeshGPU(N, len(lens), list(lens), list(shifts), np.zeros(len(lens) * (N // 2) * 2 + N), grid,
                          X="mzi_outphase", phi_pos="in", is_phase=True, device=device)


def reck_direct(U, p_splitter=0.0, device=None):
    """ReckNetwork(M=U, p_splitter=..., method='direct', phi_pos='in') (reck.py:69-74): a GenericMeshGPU of
    output-phase MZIs with its screen at the input, programmed by the direct method.  The GPU kernels take an
    even number of modes (as the reference's GPU path, gpu/mesh.py:67): for odd N the mesh is built on N + 1
    modes, the last one untouched by any MZI and unscreened, and returned as a ClippedMeshGPU on the first N."""
    U = np.asarray(U, dtype=np.complex128)
    N = U.shape[0]
    lens, shifts = geom.reck(N)
    if N % 2 == 0:
        return direct(_outphase_mesh(N, lens, shifts, p_splitter, device), U)
    from .clipped import ClippedMeshGPU
    n_cr = sum(lens)
    s = np.zeros((n_cr, 2)) + np.asarray(p_splitter, dtype=np.float64)
    p, phi = direct_core(N, lens, shifts, U, s)
    full = _outphase_mesh(N + 1, lens, shifts, p_splitter, device)
    lay, slot = _flat_layout(lens, shifts)
    grid = np.zeros((full.L, (N + 1) // 2, 2))
    grid[lay, slot] = p
    full.p_phase.copy_(torch.as_tensor(np.concatenate([grid.reshape(-1), phi, [0.0]]), dtype=full.p_phase.dtype))
    return ClippedMeshGPU(full, slice(N), slice(N))


def square_direct(M, p_splitter=0.0, eig: Optional[float] = None, device=None):
    """SquareNetwork(M=M, method='direct', phi_pos='in') (square.py:103-113): the (m + n)-mode diamond mesh of
    output-phase MZIs, screen at the input, programmed by the direct method to [[fact M, 0], [0, 0]]; returned
    as a ClippedMeshGPU (inputs 0..n-1, outputs 0..m-1) and the scale factor fact."""
    from scipy.linalg import eigvalsh

    from .clipped import ClippedMeshGPU
    M11 = np.array(M, dtype=np.complex128)
    m_out, n_in = M11.shape
    Nf = m_out + n_in
    shifts = np.abs(np.arange(-n_in + 1, m_out))
    lens = (Nf - shifts - shifts[::-1]) // 2
    fact = np.sqrt(eig / eigvalsh(M11 @ M11.conj().T, subset_by_index=[m_out - 1, m_out - 1])[0]) if eig else 1.0
    U = np.zeros((Nf, Nf), dtype=np.complex128)
    U[:m_out, :n_in] = M11 * fact
    full = direct(_outphase_mesh(Nf, lens.tolist(), shifts.tolist(), p_splitter, device), U)
    return ClippedMeshGPU(full, slice(n_in), slice(m_out)), fact


# ---- local error correction

def _mzi_T(p, s) -> np.ndarray:
    """(2, 2, n) transfer matrices of MZI crossings, p (n, 2) = (theta, phi), s (n, 2) = (alpha, beta): the
    reference's MZICrossing.T (crossing.py:216-221)."""
    th, ph = p[:, 0], p[:, 1]
    a, b = s[:, 0], s[:, 1]
    Cp, Cm, C = np.cos(a + b), np.cos(a - b), np.cos(th / 2)
    Sp, Sm, S = np.sin(a + b), np.sin(a - b), np.sin(th / 2)
    f = np.exp(1j * ph)
    return np.exp(1j * th / 2) * np.array([[f * (1j * S * Cm - C * Sp), 1j * C * Cp - S * Sm],
                                           [f * (1j * C * Cp + S * Sm), -1j * S * Cm - C * Sp]])


def _solve_row0(t0, t1, s) -> np.ndarray:
    """(theta, phi) per MZI (n, 2) whose first row is proportional to (t0, t1), for splitting errors s (n, 2):
    the reference's MZICrossing.Tsolve(..., 'T1:') (crossing.py:246-251); unreachable ratios clip to the
    nearest splitting ratio."""
    a, b = s[:, 0], s[:, 1]
    Cp, Cm, Sp, Sm = np.cos(a + b), np.cos(a - b), np.sin(a + b), np.sin(a - b)
    R2 = np.abs(t1) ** 2 / (np.abs(t0) ** 2 + 1e-30)
    with np.errstate(invalid="ignore", divide="ignore"):
        S2 = (Cp ** 2 - R2 * Sp ** 2) / ((Cp ** 2 - Sm ** 2) + R2 * (Cm ** 2 - Sp ** 2))
        h = np.nan_to_num(np.arcsin(np.sqrt(np.clip(S2, 0, 1))), nan=0.0, posinf=0.0, neginf=0.0)
    C, S = np.cos(h), np.sin(h)
    phi = np.angle(1j * C * Cp - S * Sm) - np.angle(1j * Cm * S - C * Sp) + np.angle(t0) - np.angle(t1)
    return np.stack([2 * h, phi], axis=1)


def errcorr_core(N: int, lens, shifts, p0, s0, s1, perm_rows=None):
    """Local error correction (reference configure.py:412-433, errcorr_local; S. Bandyopadhyay et al.,
    arXiv:2103.04993) on flat arrays: a nearest-neighbour MZI mesh of N modes (lens, shifts) with phases p0 (n_cr, 2) realises
    its matrix with splitting errors s0; returns the phases p1 (n_cr, 2) that, with splitting errors s1, match each
    MZI's first row up to output phases, and the phases (N,) those leave at the output, which the caller adds to the
    output screen.  perm_rows: (L + 1, N) gather rows between layers (row i before layer i, row L after the last),
    or None.  Host code: one vectorised solve per layer."""
    lens = [int(v) for v in lens]
    shifts = [int(v) for v in shifts]
    p0 = np.asarray(p0, dtype=np.float64).reshape(-1, 2)
    n_cr = p0.shape[0]
    s0 = np.broadcast_to(np.asarray(s0, dtype=np.float64), (n_cr, 2))
    s1 = np.broadcast_to(np.asarray(s1, dtype=np.float64), (n_cr, 2))
    phase = np.zeros(int(N))
    p1 = np.zeros((n_cr, 2))
    ind = 0
    for i, (ln, sh) in enumerate(zip(lens, shifts)):
        if perm_rows is not None:
            phase = phase[np.asarray(perm_rows[i])]
        sl = slice(ind, ind + ln)
        psi = phase[sh:sh + 2 * ln]
        T0 = _mzi_T(p0[sl], s0[sl])
        T0[:, 0, :] *= np.exp(1j * psi[::2])
        T0[:, 1, :] *= np.exp(1j * psi[1::2])
        p1[sl] = _solve_row0(T0[0, 0], T0[0, 1], s1[sl])
        with np.errstate(invalid="ignore", divide="ignore"):
            phase[sh:sh + 2 * ln] = np.angle(T0 / _mzi_T(p1[sl], s1[sl]))[:, 0, :].T.reshape(-1)
        ind += ln
    if perm_rows is not None:
        phase = phase[np.asarray(perm_rows[len(lens)])]
    return p1, phase


def errcorr_local(mesh: MeshNetworkGPU, p_splitter) -> MeshNetworkGPU:
    """A copy of mesh (nearest-neighbour MZI crossings, phase screen at the output or none) reprogrammed for the
    splitting errors p_splitter (scalar or (n_cr, 2) in the reference's flat order) by local error correction
    (reference configure.py:412-433): each MZI's first row is matched up to phases, which are carried forward and
    added to the output screen.  The result has an output screen."""
    if mesh.X != "mzi" or mesh.geometry != geom_nn():
        raise ValueError("local error correction takes nearest-neighbour meshes of MZI crossings")
    if mesh.is_phase and mesh.phi_pos != "out":
        raise ValueError("local error correction adds its phases to an output screen")
    N, L = mesh.N, mesh.L
    lay, slot = _flat_layout(mesh.lens_h, mesh.shifts_h)
    n_grid = L * (N // 2) * 2
    grid = mesh.p_phase[:n_grid].detach().double().cpu().numpy().reshape(L, N // 2, 2)
    sp = mesh.p_splitter
    s0 = sp.detach().double().cpu().numpy()[lay, slot] if sp.numel() else np.zeros((len(lay), 2))
    s1 = np.broadcast_to(np.asarray(p_splitter, dtype=np.float64), (len(lay), 2))
    perm = None if mesh.perm_table is None else np.asarray(mesh.perm_h)
    p1, phase = errcorr_core(N, mesh.lens_h, mesh.shifts_h, grid[lay, slot], s0, s1, perm)
    screen = mesh.p_phase[n_grid:].detach().double().cpu().numpy() if mesh.is_phase else np.zeros(N)
    g1 = np.zeros((L, N // 2, 2))
    g1[lay, slot] = p1
    gs = np.zeros((L, N // 2, 2))
    gs[lay, slot] = s1
    return MeshNetworkGPU(N, L, mesh.lens_h, mesh.shifts_h, np.concatenate([g1.reshape(-1), screen + phase]),
                          gs.astype(np.float32), "mzi", phi_pos="out", is_phase=True, device=mesh.device,
                          perm=None if perm is None else [row for row in perm])
