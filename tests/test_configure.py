"""Self-configuration by matrix diagonalisation (reference configure.py:187-330) against the reference's own
results (tests/golden/configure_*.npz, written by make_golden.py from ReckNetwork(M=U, method='diag*' | 'diag')
and SquareNetwork(M=M, method='diag') after a recorded np.random seed).

CPU: the native nulling pass (mg_diag_configure), started from the complex128 matrix of the seeded random
start, reproduces the reference's programmed phases and screen to 1e-9.  GPU: the whole method, with the
starting matrix evaluated by the propagation kernels in complex64, reproduces the programmed phases and
screen to 1e-5 rad and the programmed mesh's matrix to 1e-5 relative error.

The direct method (configure.py:333-410) against ReckNetwork(M=U, method='direct', phi_pos='in') and
SquareNetwork(M=M, method='direct', phi_pos='in') (configure_*_direct_*.npz): the native pass
(mg_direct_configure) reproduces the programmed phases and input screen to 1e-9 on the CPU; on the GPU the
programmed output-phase mesh's matrix equals the reference's to 1e-5."""
import os

import numpy as np
import pytest

from oracle import meshes_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RECK = ["reck_diagstar_N8", "reck_diag_N8"]
DIRECT_RECK = ["reck_direct_N8", "reck_direct_N5", "reck_direct_N16"]
DIRECT_SQUARE = ["square_direct_N3", "square_direct_4x2"]


def load(name):
    return np.load(os.path.join(GOLDEN, "configure_%s.npz" % name))


def _wrap(a):
    """angles to (-pi, pi]"""
    return np.angle(np.exp(1j * np.asarray(a)))


def _square_problem(z):
    """The reference's SquareNet embedding (square.py:85-92): U = [[M, M12]] with M12 = chol(I - M M^H)."""
    M = z["M"]
    m, n = M.shape
    U = np.zeros((m + n, m + n), dtype=complex)
    U[:m, :n] = M
    U[:m, n:] = np.linalg.cholesky(np.eye(m) - M @ M.conj().T)
    return U, m, n


@pytest.mark.parametrize("name", RECK + ["square_diag_N3"])
def test_nulling_pass_matches_reference(name):
    from meshes_gb300 import configure as C
    z = load(name)
    lens, shifts = z["lens"].tolist(), z["shifts"].tolist()
    N = len(z["phi_out"])
    n_cr = sum(lens)
    if name.startswith("reck"):
        U = z["U"]
        s = z["p_splitter"]
        nm, (nn, ijxyp) = N - 1, C.reck_steps(N)
    else:
        U, m, n = _square_problem(z)
        s = np.zeros((n_cr, 2))
        nm = m
        nn = lambda k: n                                               # noqa: E731
        ijxyp = lambda k, j: [k, n + k - j, k + j, n - 1 + k - j, k * 0]   # noqa: E731
    np.random.seed(int(z["seed"]))
    c1 = np.zeros((n_cr, 2))
    c1[:, 1] = 2 * np.pi * np.random.rand(n_cr)
    np.random.rand(0)
    om = O.OracleMesh(N=N, L=len(lens), crossing="mzi", lens=lens, shifts=shifts,
                      p=O.flat_to_grid(c1, lens, shifts, N, 2), s=O.flat_to_grid(s, lens, shifts, N, 2))
    Z = O.matrix(om)
    ijzp, x, y = C.diag_steps((lens, shifts), ([], []), nm, nn, ijxyp)
    init = C.diag_init("rand", x, y, len(ijzp))
    _, _, _, phi = C.diag_core(U, Z, s, c1, np.zeros((0, 2)), np.zeros((0, 2)), ijzp, init, None,
                               str(z["method"]) == "diag*")
    assert np.max(np.abs(_wrap(c1 - z["p_crossing"]))) < 1e-9
    assert np.max(np.abs(_wrap(phi - z["phi_out"]))) < 1e-9


def test_nulling_pass_rejects_bad_steps():
    from meshes_gb300 import _lib
    lib = _lib.load()
    N = 4
    U = np.eye(N, dtype=complex)
    bufs = [U.copy() for _ in range(4)]
    c = np.zeros((3, 2))
    s = np.zeros((3, 2))
    ijzp = np.array([[0, 3, 5, 0]], np.int32)        # MZI 5 of a 3-MZI mesh
    init = np.zeros((1, 2))
    rc = lib.mg_diag_configure(N, 1, *[b.ctypes.data for b in bufs], 3, s.ctypes.data, c.ctypes.data, 0, 0, None,
                               None, 1, ijzp.ctypes.data, init.ctypes.data, None, 1)
    assert rc == -1 and "out of range" in _lib.last_error()
    assert np.array_equal(bufs[0], np.eye(N))


@pytest.mark.gpu
@pytest.mark.parametrize("name", RECK)
def test_reck_programmed_on_gpu_matches_reference(name):
    from meshes_gb300 import configure as C
    z = load(name)
    N = int(z["N"])
    np.random.seed(int(z["seed"]))
    m = C.reck(z["U"], p_splitter=z["p_splitter"], improved=str(z["method"]) == "diag*", device="cuda")
    lay, slot = C._flat_layout(m.lens_h, m.shifts_h)
    n_grid = m.L * (N // 2) * 2
    p = m.p_phase[:n_grid].reshape(m.L, N // 2, 2).double().cpu().numpy()[lay, slot]
    assert np.max(np.abs(_wrap(p - z["p_crossing"]))) < 1e-5
    assert np.max(np.abs(_wrap(m.p_phase[n_grid:].double().cpu().numpy() - z["phi_out"]))) < 1e-5
    U = m.matrix().cpu().numpy()
    assert O.rel_err(U, z["matrix"]) < 1e-5
    assert m.status() == 0


@pytest.mark.gpu
def test_square_programmed_on_gpu_matches_reference():
    from meshes_gb300 import configure as C
    z = load("square_diag_N3")
    np.random.seed(int(z["seed"]))
    cm, fact = C.square(z["M"], device="cuda")
    assert fact == 1.0
    full = cm.full
    lay, slot = C._flat_layout(full.lens_h, full.shifts_h)
    n_grid = full.L * (full.N // 2) * 2
    p = full.p_phase[:n_grid].reshape(full.L, full.N // 2, 2).double().cpu().numpy()[lay, slot]
    assert np.max(np.abs(_wrap(p - z["p_crossing"]))) < 1e-5
    assert np.max(np.abs(_wrap(full.p_phase[n_grid:].double().cpu().numpy() - z["phi_out"]))) < 1e-5
    assert O.rel_err(cm.matrix().cpu().numpy(), z["matrix"]) < 1e-5


def _direct_problem(name, z):
    N = len(z["phi_out"])
    if name.startswith("reck"):
        return N, z["U"], z["p_splitter"]
    M = z["M"] * float(z["fact"])
    U = np.zeros((N, N), dtype=complex)
    U[:M.shape[0], :M.shape[1]] = M
    return N, U, np.zeros((int(z["lens"].sum()), 2))


@pytest.mark.parametrize("name", DIRECT_RECK + DIRECT_SQUARE)
def test_direct_pass_matches_reference(name):
    from meshes_gb300 import configure as C
    z = load(name)
    assert str(z["X"]) == "MZICrossingOutPhase"
    N, U, s = _direct_problem(name, z)
    p, phi = C.direct_core(N, z["lens"], z["shifts"], U, s)
    assert np.max(np.abs(_wrap(p - z["p_crossing"]))) < 1e-9
    assert np.max(np.abs(_wrap(phi - z["phi_out"]))) < 1e-9


def test_direct_pass_geometry_checks():
    """A Clements layout (two diagonals driven through input 0) is refused with MG_E_ARG; a mesh of one
    diagonal (N = 2) keeps its phases and gets a zero screen, as the reference's diagonal split leaves it."""
    from meshes_gb300 import _lib
    from meshes_gb300 import configure as C
    with pytest.raises(_lib.MeshLibraryError, match="share an input mode"):
        C.direct_core(4, [2, 1, 2, 1], [0, 1, 0, 1], np.eye(4), np.zeros((6, 2)))
    with pytest.raises(_lib.MeshLibraryError, match="outside N"):
        C.direct_core(4, [2, 2], [0, 1], np.eye(4), np.zeros((4, 2)))
    p0 = np.array([[0.3, -0.2]])
    p, phi = C.direct_core(2, [1], [0], np.eye(2), np.zeros((1, 2)), p0)
    assert np.array_equal(p, p0) and np.array_equal(phi, np.zeros(2))


@pytest.mark.gpu
@pytest.mark.parametrize("name", DIRECT_RECK)
def test_reck_direct_on_gpu_matches_reference(name):
    from meshes_gb300 import configure as C
    z = load(name)
    N = int(z["N"])
    m = C.reck(z["U"], p_splitter=z["p_splitter"], method="direct", device="cuda")
    full = m.full if N % 2 else m                      # odd N: an (N + 1)-mode mesh clipped to N ports
    Nf = full.N
    lay, slot = C._flat_layout(full.mesh.lens_h, full.mesh.shifts_h)
    n_grid = full.L * (Nf // 2) * 2
    p = full.p_phase[:n_grid].reshape(full.L, Nf // 2, 2).cpu().numpy()[lay, slot]
    assert np.max(np.abs(_wrap(p - z["p_crossing"]))) < 1e-9
    assert np.max(np.abs(_wrap(full.p_phase[n_grid:n_grid + N].cpu().numpy() - z["phi_out"]))) < 1e-9
    U = m.matrix().cpu().numpy()
    assert U.shape == (N, N)
    assert O.rel_err(U, z["matrix"]) < 1e-5
    assert O.rel_err(U, z["U"]) < 1e-5
    assert full.status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", DIRECT_SQUARE)
def test_square_direct_on_gpu_matches_reference(name):
    from meshes_gb300 import configure as C
    z = load(name)
    eig = float(z["eig"])
    cm, fact = C.square(z["M"], eig=None if eig < 0 else eig, device="cuda", method="direct")
    assert abs(fact - float(z["fact"])) < 1e-12
    assert O.rel_err(cm.matrix().cpu().numpy(), z["matrix"]) < 1e-5
    assert O.rel_err(cm.matrix().cpu().numpy(), fact * z["M"]) < 1e-5


ERRCORR = ["clements_N8", "perm_N8"]


def _errcorr(name):
    z = np.load(os.path.join(GOLDEN, "errcorr_%s.npz" % name))
    perm = None if z["perm_none"].all() else z["perm_rows"]
    return z, perm


@pytest.mark.parametrize("name", ERRCORR)
def test_errcorr_core_matches_reference(name):
    """Local error correction (configure.py:412-433) on the host: the corrected phases and the phases added to
    the output screen equal the reference's errcorr_local (to 1e-9; a Clements mesh and a permuted mesh)."""
    from meshes_gb300 import configure as C
    z, perm = _errcorr(name)
    p1, phase = C.errcorr_core(int(z["N"]), z["lens"], z["shifts"], z["p_crossing0"], z["p_splitter0"],
                               z["p_splitter"], perm)
    assert np.max(np.abs(_wrap(p1 - z["p_crossing"]))) < 1e-9
    assert np.max(np.abs(_wrap(z["phi_out0"] + phase - z["phi_out"]))) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", ERRCORR)
def test_errcorr_on_gpu_matches_reference(name):
    """errcorr_local on a MeshNetworkGPU: the corrected mesh (new splitting errors) propagates on the GPU to the
    reference's corrected matrix within 1e-5, and the uncorrected mesh to the reference's target matrix."""
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300 import configure as C
    z, perm = _errcorr(name)
    N = int(z["N"])
    lens, shifts = z["lens"].tolist(), z["shifts"].tolist()
    L = len(lens)
    lay, slot = C._flat_layout(lens, shifts)
    grid = np.zeros((L, N // 2, 2))
    grid[lay, slot] = z["p_crossing0"]
    sgrid = np.zeros((L, N // 2, 2))
    sgrid[lay, slot] = z["p_splitter0"]
    rows = None if perm is None else [None if none else row for row, none in zip(perm, z["perm_none"])]
    m = MeshNetworkGPU(N, L, lens, shifts, np.concatenate([grid.reshape(-1), z["phi_out0"]]), sgrid.astype(np.float32),
                       "mzi", phi_pos="out", is_phase=True, device="cuda", perm=rows)
    assert O.rel_err(m.matrix().cpu().numpy(), z["matrix0"]) < 1e-5
    m1 = C.errcorr_local(m, z["p_splitter"])
    assert O.rel_err(m1.matrix().cpu().numpy(), z["matrix"]) < 1e-5
    assert m1.status() == 0
