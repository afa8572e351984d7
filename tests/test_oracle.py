"""CPU tests: the oracle pinned to the reference's own outputs, the C++ port pinned to the reference's
compiled c/dot.cpp, geometry helpers, and the C ABI library's exports (no GPU calls)."""
import os
import re

import numpy as np
import pytest

from oracle import meshes_oracle as O
from oracle import port as P

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def fixtures():
    """Fixtures of the plain meshes (the phase-screen and lossy fixtures have their own tests)."""
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz") and "_screen_" not in f and "lossy" not in f
                  and not f.startswith(("clipped_", "perm_", "piloss_", "xmesh_", "crossings_", "converter_", "configure_", "errcorr_")))


def load(name):
    z = np.load(os.path.join(GOLDEN, name))
    kw = dict(lens=z["lens"].tolist(), shifts=z["shifts"].tolist()) if "lens" in z else dict(strides=z["strides"].tolist())
    return z, O.OracleMesh(N=int(z["N"]), L=int(z["L"]), crossing=str(z["crossing"]), p=z["p"],
                           s=z["s"] if "s" in z else None, **kw)


@pytest.mark.parametrize("name", fixtures())
def test_oracle_matches_reference_fixtures(name):
    z, om = load(name)
    assert O.rel_err(O.propagate(om, z["x"]), z["y"]) < 1e-12
    if "dy" in z:
        y, dy = O.fwddiff(om, z["x"], z["dp_dir"])
        assert O.rel_err(dy, z["dy"]) < 1e-12
    if "dJdp" in z:
        G, xr, gin = O.vjp_unitary(om, z["y"], z["g"])
        assert O.rel_err(O.contract_dp(om, G), z["dJdp"]) < 1e-12
        assert O.rel_err(gin, z["g_in"]) < 1e-12
        assert O.rel_err(xr, z["x"]) < 1e-12
        G2, gin2 = O.vjp_stored(om, z["x"], z["g"])
        assert O.rel_err(O.contract_dp(om, G2), z["dJdp"]) < 1e-12


@pytest.mark.parametrize("name", [f for f in fixtures() if "y_c64" in np.load(os.path.join(GOLDEN, f))])
def test_port_matches_reference_fixtures(name):
    """The C++ port against the reference's complex128 dot and its complex64 meshdot_helper32."""
    z, om = load(name)
    fns = P.port_lib()
    y64 = P.forward(fns, om, z["x"], dtype=np.complex128)
    assert O.rel_err(y64, z["y"]) < 1e-12
    y32 = P.forward(fns, om, z["x"], dtype=np.complex64)
    assert O.rel_err(y32, z["y_c64"]) < 1e-6
    G, gin = P.vjp(fns, om, z["y"], z["g"], dtype=np.complex128)
    assert O.rel_err(O.contract_dp(om, G), z["dJdp"]) < 1e-12
    assert O.rel_err(gin, z["g_in"]) < 1e-12


def _random_flat_case(rng, N, B, perm=False, pos=-1):
    lens, shifts = O.clements_geometry(N)
    om = O.random_mesh(rng, N, "clements", "mzi", 0.05)
    T, inds = P.packed_T(om)
    nT = T.shape[2]
    dT = (rng.standard_normal(T.shape) + 1j * rng.standard_normal(T.shape))
    v = rng.standard_normal((N, B)) + 1j * rng.standard_normal((N, B))
    dv = rng.standard_normal((N, B)) + 1j * rng.standard_normal((N, B))
    ph = rng.uniform(0, 2 * np.pi, N) if pos >= 0 else np.zeros(0)
    dph = rng.standard_normal(N) if pos >= 0 else np.zeros(0)
    perms = np.array([rng.permutation(N) for _ in range(len(lens) + 1)], np.int32) if perm else np.empty((0, 0), np.int32)
    return om, T, dT, ph, dph, v, dv, inds, lens, shifts, perms, nT


@pytest.mark.skipif(P.ref_lib() is None, reason="reference c/dot.cpp not compiled here (oracle/_ref)")
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("perm,pos", [(False, -1), (True, -1), (False, 1), (True, 0)])
def test_port_matches_reference_binary(mode, perm, pos):
    """Port vs the reference's own compiled c/dot.cpp on random inputs, phase screens and permutations
    included (mode 2 with one thread: the reference's threaded reduction races)."""
    rng = np.random.default_rng(100 + mode + 10 * perm + 3 * pos)
    case = _random_flat_case(rng, 12, 19, perm, pos)
    om, T, dT, ph, dph, v, dv, inds, lens, shifts, perms, nT = case
    outs = []
    for fns in (P.port_lib(), P.ref_lib()):
        T_, dT_ = T.copy(), (dT.copy() if mode == 1 else np.zeros_like(dT))
        ph_, dph_ = ph.copy(), (dph.copy() if mode == 1 else np.zeros_like(dph))
        v_, dv_ = v.copy(), dv.copy()
        P.call(fns, T_, dT_, ph_, dph_, v_, dv_, inds, lens, shifts, perms, pos, mode, 1)
        outs.append((v_, dv_, dT_, dph_))
    for a, b in zip(*outs):
        if a.size:
            assert O.rel_err(a, b) < 1e-12


def test_port_threads_race_free():
    """Mode 2 with several threads equals one thread (private accumulators, ordered sum)."""
    rng = np.random.default_rng(11)
    om = O.random_mesh(rng, 32, "clements", "mzi", 0.02)
    y = O.unit_columns(rng, 32, 200)
    g = O.unit_columns(rng, 32, 200)
    fns = P.port_lib()
    G1, g1 = P.vjp(fns, om, y, g, threads=1, dtype=np.complex128)
    G8, g8 = P.vjp(fns, om, y, g, threads=8, dtype=np.complex128)
    assert O.rel_err(G8, G1) < 1e-13 and O.rel_err(g8, g1) < 1e-14


def test_oracle_gradient_central_differences():
    rng = np.random.default_rng(12)
    for geo, cr in (("clements", "mzi"), ("reck", "sym"), ("fft", "mzi"), ("clements", "orth")):
        om = O.random_mesh(rng, 8, geo, cr, 0.02)
        real = cr == "orth"
        x = O.unit_columns(rng, 8, 5, real=real)
        t = O.unit_columns(rng, 8, 5, real=real)

        def loss(p):
            return float(np.sum(np.abs(O.propagate(om, x, p) - t) ** 2))

        y, dp, _ = O.grad(om, x, lambda y: 2 * (y - t))
        idx = np.flatnonzero(np.broadcast_to(om.active_mask()[..., None], om.p.shape))[:10]
        fd = O.central_difference(loss, om.p.astype(np.float64), idx, h=1e-6)
        assert np.allclose(dp.reshape(-1)[idx], fd, rtol=1e-6, atol=1e-8)


def test_lossy_adjoint_matches_finite_differences():
    """vjp_stored (activations kept) is exact for non-unitary crossings, vjp_unitary is not."""
    rng = np.random.default_rng(13)
    om = O.random_mesh(rng, 6, "clements", "mzi", 0.02)
    T = om.T_grid() * np.exp(rng.normal(0, 0.05, (om.L, 3, 1, 1)))   # per-slot gain
    lossy = O.OracleMesh(N=6, L=om.L, crossing="mzi", lens=om.lens, shifts=om.shifts, p=om.p, s=om.s, T_override=T)
    x = O.unit_columns(rng, 6, 4)
    g = O.unit_columns(rng, 6, 4)
    G, gin = O.vjp_stored(lossy, x, g)
    # dJ/dx* for J = Re<g, Ux>*2 is U^H g
    U = O.matrix(lossy)
    assert O.rel_err(gin, (U.conj().T @ g.T).T) < 1e-12
    Gu, _, _ = O.vjp_unitary(lossy, O.propagate(lossy, x), g)
    assert O.rel_err(Gu, G) > 1e-3


def _lossy_mesh(rng, N, gain=0.1):
    """Clements mesh of lossy generic MZIs: phase errors and log-gains g_ij ~ -|N(gain, gain/2)|."""
    om = O.random_mesh(rng, N, "clements", "mzi_generic", 0.02)
    s = np.zeros((om.L, N // 2, 14))
    s[..., :10] = rng.normal(0, 0.03, (om.L, N // 2, 10))
    s[..., 10:] = -np.abs(rng.normal(gain, gain / 2, (om.L, N // 2, 4)))
    s[~om.active_mask()] = 0
    om.s = s
    return om


def test_lossy_crossing_matches_reference_fixture():
    """T of the lossy generic MZI and the forward through a lossy Clements mesh, against the reference."""
    f = np.load(os.path.join(GOLDEN, "clements_mzigeneric_N8_lossy.npz"))
    om = O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing="mzi_generic", lens=list(f["lens"]),
                      shifts=list(f["shifts"]), p=f["p"], s=f["s"])
    mask = om.active_mask()
    assert np.abs(om.T_grid()[mask] - f["T"][mask]).max() < 1e-14
    y = O.propagate(om, f["x"])
    assert O.rel_err(y, f["y"]) < 1e-13
    assert np.linalg.norm(y) < 0.9 * np.linalg.norm(f["x"])          # the mesh loses power


def test_lossy_generic_gradient_central_differences():
    """dJ/dp of a lossy mesh from stored activations (vjp_stored + dT_mzi_generic) equals complex128
    central differences; the T^H-inversion adjoint of the unitary path does not."""
    rng = np.random.default_rng(14)
    om = _lossy_mesh(rng, 8)
    x = O.unit_columns(rng, 8, 5)
    t = O.unit_columns(rng, 8, 5)

    def loss(p):
        return float(np.sum(np.abs(O.propagate(om, x, p) - t) ** 2))

    y = O.propagate(om, x)
    G, _ = O.vjp_stored(om, x, 2 * (y - t))
    dp = O.contract_dp(om, G)
    idx = np.flatnonzero(np.broadcast_to(om.active_mask()[..., None], om.p.shape))
    fd = O.central_difference(loss, om.p.astype(np.float64), idx, h=1e-6)
    assert np.allclose(dp.reshape(-1)[idx], fd, rtol=1e-6, atol=1e-9)
    Gu, _, _ = O.vjp_unitary(om, y, 2 * (y - t))
    assert O.rel_err(O.contract_dp(om, Gu).reshape(-1)[idx], fd) > 1e-2


@pytest.mark.parametrize("pos", ["out", "in"])
def test_phase_screen_matches_reference_fixtures(pos):
    """Forward, forward-mode derivative and VJP of a Clements mesh with a phase screen (is_phase=True)."""
    f = np.load(os.path.join(GOLDEN, "clements_mzi_N8_screen_%s.npz" % pos))
    assert str(f["phi_pos"]) == pos
    om = O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing="mzi", lens=list(f["lens"]), shifts=list(f["shifts"]),
                      p=f["p"], s=f["s"])
    y = O.propagate_screened(om, f["x"], f["ph"], pos)
    assert O.rel_err(y, f["y"]) < 1e-13
    y2, dy = O.fwddiff_screened(om, f["x"], f["ph"], pos, f["dp_dir"], f["dph_dir"])
    assert O.rel_err(y2, f["y"]) < 1e-13 and O.rel_err(dy, f["dy"]) < 1e-12
    dp, dph, gin = O.grad_screened(om, f["y"], f["g"], f["ph"], pos)
    assert O.rel_err(dp, f["dJdp"]) < 1e-12
    assert O.rel_err(dph, f["dJdph"]) < 1e-12
    assert O.rel_err(gin, f["g_in"]) < 1e-12


@pytest.mark.parametrize("name", ["clipped_squarenet_N4.npz", "clipped_qrnet_N4.npz"])
def test_clipped_mesh_matches_reference_fixtures(name):
    """ClippedNetwork semantics (mesh.py:718-802): embed the inputs at idx_in, propagate the full mesh
    (phase screen on), keep idx_out; grad_L2 of ||U[idx_out] - U_t||^2."""
    f = np.load(os.path.join(GOLDEN, name))
    pos = str(f["phi_pos"])
    om = O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing="mzi", lens=list(f["lens"]), shifts=list(f["shifts"]),
                      p=f["p"], s=f["s"])
    Nf, n_in = int(f["N"]), len(f["idx_in"])
    X = np.zeros((f["x"].shape[1], Nf), complex)
    X[:, f["idx_in"]] = f["x"].T
    y = O.propagate_screened(om, X, f["ph"], pos)[:, f["idx_out"]].T
    assert O.rel_err(y, f["y"]) < 1e-13
    E = np.zeros((n_in, Nf), complex)
    E[np.arange(n_in), f["idx_in"]] = 1
    U = O.propagate_screened(om, E, f["ph"], pos)                  # rows: U[:, idx_in[k]]
    dU = U[:, f["idx_out"]].T - f["U_target"]
    assert abs(np.sum(np.abs(dU) ** 2) - float(f["J"])) < 1e-12 * float(f["J"])
    G = np.zeros_like(U)
    G[:, f["idx_out"]] = 2 * dU.T
    dp, dph, _ = O.grad_screened(om, U, G, f["ph"], pos)
    assert O.rel_err(dp, f["dJdp"]) < 1e-12 and O.rel_err(dph, f["dJdph"]) < 1e-12


def _perm_mesh(f):
    return O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing="mzi", lens=list(f["lens"]), shifts=list(f["shifts"]),
                        p=f["p"], s=f["s"], perm=f["perm"])


@pytest.mark.parametrize("name", ["perm_mzi_N8_split.npz", "perm_mzi_N8_screen_in.npz"])
def test_permuted_mesh_matches_reference_fixtures(name):
    """Permutations between layers (c/dot.cpp:29-40,150-153,289-292): forward, forward-mode derivative and
    dot_vjp (inverse permutations in reverse, mesh.py:382) of the reference, with and without a screen."""
    f = np.load(os.path.join(GOLDEN, name))
    om = _perm_mesh(f)
    if bool(f["is_phase"]):
        pos = str(f["phi_pos"])
        y = O.propagate_screened(om, f["x"], f["ph"], pos)
        _, dy = O.fwddiff_screened(om, f["x"], f["ph"], pos, f["dp_dir"], f["dph_dir"])
        dp, dph, gin = O.grad_screened(om, f["y"], f["g"], f["ph"], pos)
        assert O.rel_err(dph, f["dJdph"]) < 1e-12
    else:
        y = O.propagate(om, f["x"])
        _, dy = O.fwddiff(om, f["x"], f["dp_dir"])
        G, xr, gin = O.vjp_unitary(om, f["y"], f["g"])
        dp = O.contract_dp(om, G)
        assert O.rel_err(xr, f["x"]) < 1e-12
        G2, gin2 = O.vjp_stored(om, f["x"], f["g"])
        assert O.rel_err(O.contract_dp(om, G2), f["dJdp"]) < 1e-12 and O.rel_err(gin2, f["g_in"]) < 1e-12
    assert O.rel_err(y, f["y"]) < 1e-13
    assert O.rel_err(dy, f["dy"]) < 1e-12
    assert O.rel_err(dp, f["dJdp"]) < 1e-12
    assert O.rel_err(gin, f["g_in"]) < 1e-12


def test_piloss_matches_reference_fixture():
    """PILOSS mesh (piloss.py:18-57): a ClippedNetwork over a permuted full mesh with an output screen."""
    f = np.load(os.path.join(GOLDEN, "piloss_N4.npz"))
    pos = str(f["phi_pos"])
    om = _perm_mesh(f)
    Nf, n_in = int(f["N"]), len(f["idx_in"])
    X = np.zeros((f["x"].shape[1], Nf), complex)
    X[:, f["idx_in"]] = f["x"].T
    assert O.rel_err(O.propagate_screened(om, X, f["ph"], pos)[:, f["idx_out"]].T, f["y"]) < 1e-13
    E = np.zeros((n_in, Nf), complex)
    E[np.arange(n_in), f["idx_in"]] = 1
    U = O.propagate_screened(om, E, f["ph"], pos)
    dU = U[:, f["idx_out"]].T - f["U_target"]
    assert abs(np.sum(np.abs(dU) ** 2) - float(f["J"])) < 1e-12 * float(f["J"])
    G = np.zeros_like(U)
    G[:, f["idx_out"]] = 2 * dU.T
    dp, dph, _ = O.grad_screened(om, U, G, f["ph"], pos)
    assert O.rel_err(dp, f["dJdp"]) < 1e-12 and O.rel_err(dph, f["dJdph"]) < 1e-12


GENERIC_CROSSINGS = ["mzi_balanced", "mzi_outphase", "mzi3", "mzi3_outphase", "mzi_generic_outphase", "cartesian",
                     "bell"]


@pytest.mark.parametrize("name", GENERIC_CROSSINGS)
def test_crossing_parameterisations_match_reference(name):
    """T of the reference's other crossing classes (crossing.py:292-611): the oracle's restatement and the
    product's torch builder (on the CPU, float64) against the reference's own T."""
    import torch
    from meshes_gb300.crossings import transfer
    z = np.load(os.path.join(GOLDEN, "crossings_T.npz"))
    p, s, T = z[name + "_p"], z[name + "_s"], z[name + "_T"]
    assert O.rel_err(np.moveaxis(O.T_FN[name](p, s), -1, 0), T) < 1e-14
    Tt = transfer(name, torch.tensor(p), torch.tensor(s)).numpy()
    assert O.rel_err(Tt, T) < 1e-14


@pytest.mark.parametrize("name", GENERIC_CROSSINGS)
def test_generic_crossing_meshes_match_reference(name):
    """A Clements mesh of each class through the reference's StructuredMeshNetwork.dot, and its dot_vjp
    where the class has dT: the oracle forward, and central differences of Re sum conj(g) y(p) (whose
    gradient is the reference's dJ/dp for g = 2 dJ/dy*)."""
    f = np.load(os.path.join(GOLDEN, "xmesh_%s_N6.npz" % name))
    om = O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing=name, lens=list(f["lens"]), shifts=list(f["shifts"]),
                      p=f["p"], s=f["s"])
    assert O.rel_err(O.propagate(om, f["x"]), f["y"]) < 1e-13
    if "dJdp" not in f:
        return
    active = om.active_mask()
    idx = np.flatnonzero(np.broadcast_to(active[..., None], f["p"].shape))
    fd = O.central_difference(lambda pp: float(np.real(np.sum(np.conj(f["g"]) * O.propagate(om, f["x"], pp)))),
                              f["p"], idx)
    G, gin = O.vjp_stored(om, f["x"], f["g"])
    assert O.rel_err(gin, f["g_in"]) < 1e-12
    if name != "mzi_outphase":
        assert O.rel_err(fd, f["dJdp"].reshape(-1)[idx]) < 1e-7
        return
    # The reference's MZICrossingOutPhase.dT (crossing.py:338-340) reverses, in its vectorised branch, the
    # slot axis instead of the first matrix axis (dT_in[:, :, ::-1, ::-1] on (n_phase, 2, 2, k)), so its
    # dot_vjp gradient is not the derivative of its own T.  Pin that reading: the reference's numbers are the
    # contraction with that array, and the true derivative (central differences) differs.
    ab = f["s"][active]
    dT_in = O.dT_mzi(f["p"][active], np.stack([ab[:, 1] + np.pi / 2, ab[:, 0] - np.pi / 2], 1))
    dT_ref = dT_in[:, :, ::-1, ::-1].transpose(0, 2, 1, 3)
    dJdp_ref = np.real(np.einsum("nijk,kij->kn", dT_ref, G[active]))
    assert O.rel_err(dJdp_ref, f["dJdp"][active]) < 1e-12
    assert O.rel_err(fd, f["dJdp"].reshape(-1)[idx]) > 0.1


def test_geometry_helpers_agree():
    from meshes_gb300 import geometry as gm
    for N in (2, 4, 8, 10, 64, 256):
        assert gm.clements(N) == O.clements_geometry(N)
        if N >= 3:
            assert gm.reck(N) == O.reck_geometry(N)
    for N in (2, 8, 64, 512):
        assert gm.butterfly(N) == O.butterfly_strides(N)
        assert gm.fft(N) == O.fft_strides(N)
    with pytest.raises(ValueError):
        gm.validate_nn(8, [4], [1])
    with pytest.raises(ValueError):
        gm.validate_fft(8, [3])


def test_header_symbols_exported():
    """Every entry point declared in include/meshes_gb300.h is exported by the library and bound in
    meshes_gb300._lib (loading only; no compute call without a GPU)."""
    from meshes_gb300 import _lib
    from meshes_gb300.build import build
    build()
    hdr = open(os.path.join(ROOT, "include", "meshes_gb300.h")).read()
    declared = set(re.findall(r"\b(mg_\w+)\s*\(", hdr))
    lib = _lib.load()
    for name in declared:
        assert hasattr(lib, name), name
    assert declared == set(_lib.exported_symbols())
    assert lib.mg_version().decode().startswith("meshes_gb300")


def test_adam_step_rejects_bad_arguments():
    """mg_adam_step checks its arguments before it launches anything (no GPU needed): a negative size, a
    learning rate or betas out of range, a missing pointer."""
    from meshes_gb300 import _lib
    from meshes_gb300.build import build
    build()
    lib = _lib.load()
    ok = dict(p=8, g=8, m=8, v=8, n=4, lr=1e-2, b1=0.9, b2=0.999, eps=1e-8, state=8)

    def call(**kw):
        a = dict(ok, **kw)
        return lib.mg_adam_step(a["p"], a["g"], a["m"], a["v"], a["n"], a["lr"], a["b1"], a["b2"], a["eps"],
                                a["state"], None)
    assert call(n=-1) == -1
    assert call(lr=-1.0) == -1
    assert call(b1=1.0) == -1
    assert call(b2=-0.5) == -1
    assert call(eps=float("nan")) == -1
    assert call(p=None) == -1
    assert call(state=None) == -1
    assert call(n=0, p=None, g=None, m=None, v=None, state=None) == 0


def test_adam_wrapper_rejects_unsupported_tensors():
    """autograd.Adam takes contiguous float32 CUDA tensors only, and says so before anything touches a GPU."""
    import torch
    from meshes_gb300.autograd import Adam
    for bad in (torch.zeros(4), torch.zeros(4, dtype=torch.float64), torch.zeros(4, 2).t()):
        with pytest.raises(ValueError):
            Adam([bad])


def test_tuning_table_entries_are_valid_plans():
    """Every configuration in the committed tuning table plans (mg_plan: host-side arithmetic only) at both
    ends of its batch range, with the register tile it names; planning needs no GPU."""
    import ctypes
    import json
    from meshes_gb300 import _lib
    from meshes_gb300.build import build
    build()
    lib = _lib.load()
    table = json.load(open(os.path.join(ROOT, "meshes_gb300", "tuned_configs.json")))
    assert table
    for key, entries in table.items():
        op, crossing, geometry, N = (int(v) for v in key.split("/"))
        for e in entries:
            lo, hi = e["B"]
            assert 1 <= lo <= hi
            for B in (lo, hi):
                info = _lib.mg_plan_info()
                rc = lib.mg_plan(op, N, N, B, crossing, geometry, _lib.cfg_ptr(_lib.config(*e["cfg"])),
                                 ctypes.byref(info))
                assert rc == 0, (key, B, _lib.last_error())
                assert (info.M, info.V, info.W) == tuple(e["cfg"][:3])
                assert info.smem <= 227 * 1024 and info.grid >= 1
