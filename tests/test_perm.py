"""Permutations between layers (the reference's StructuredMeshNetwork.perm, mesh.py:238-277, applied by
c/dot.cpp:29-40,150-153,289-292): GPU parity against the reference fixtures (a permuted Clements mesh with
and without a screen, the PILOSS mesh) and against the complex128 oracle on random permuted meshes of every
geometry and crossing, through MeshNetworkGPU, the autograd function and the C ABI.

Tolerances as in test_gpu_parity.py: relative Frobenius error 1e-5.
"""
import os
import zlib

import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-5


def to_dev(x, real=False):
    dt = np.float32 if real else np.complex64
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(dt))).cuda().t()


def to_np(t):
    return t.t().contiguous().cpu().numpy()


def test_perm_rows_host_checks():
    """Host-side normalisation of the perm list (no GPU): None rows are the identity, an all-identity
    list means no permutations, a row that is not a permutation is refused."""
    from meshes_gb300.mesh import _perm_rows
    assert _perm_rows(None, 4, 2) == (None, None)
    assert _perm_rows([None, None, None], 4, 2) == (None, None)
    assert _perm_rows([np.arange(4), None, np.arange(4)], 4, 2) == (None, None)
    rows, _ = _perm_rows([None, [1, 0, 3, 2], None], 4, 2)
    assert rows.dtype == np.int32 and rows.tolist() == [[0, 1, 2, 3], [1, 0, 3, 2], [0, 1, 2, 3]]
    with pytest.raises(AssertionError):
        _perm_rows([None, [1, 1, 3, 2], None], 4, 2)
    with pytest.raises(AssertionError):
        _perm_rows([None, None], 4, 2)


def _gpu_mesh(om, ph=None, pos="out", **kw):
    from meshes_gb300 import MeshNetworkGPU
    p = np.asarray(om.p, dtype=np.float32).reshape(-1)
    if ph is not None:
        p = np.concatenate([p, np.asarray(ph, np.float32)])
    s = None if om.s is None else np.asarray(om.s, dtype=np.float32)
    geo = dict(strides=om.strides) if om.fft else {}
    return MeshNetworkGPU(om.N, om.L, None if om.fft else om.lens, None if om.fft else om.shifts, p, s, om.crossing,
                          phi_pos=pos, is_phase=ph is not None, perm=om.perm, **geo, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["perm_mzi_N8_split.npz", "perm_mzi_N8_screen_in.npz"])
def test_golden_permuted_mesh(name):
    z = np.load(os.path.join(GOLDEN, name))
    om = O.OracleMesh(N=int(z["N"]), L=int(z["L"]), crossing="mzi", lens=list(z["lens"]), shifts=list(z["shifts"]),
                      p=z["p"], s=z["s"], perm=z["perm"])
    is_phase = bool(z["is_phase"])
    m = _gpu_mesh(om, z["ph"] if is_phase else None, str(z["phi_pos"]))
    ncp = om.L * (om.N // 2) * 2
    assert O.rel_err(to_np(m.dot(to_dev(z["x"]))), z["y"]) < TOL
    dpd = z["dp_dir"].reshape(-1)
    if is_phase:
        dpd = np.concatenate([dpd, z["dph_dir"]])
    y, dy = m.dot(to_dev(z["x"]), dp=dpd.astype(np.float32))
    assert O.rel_err(to_np(y), z["y"]) < TOL and O.rel_err(to_np(dy), z["dy"]) < TOL
    dp, gin = m.grad_phi(to_dev(z["y"]), to_dev(z["g"]), vpos="out")
    dp = dp.cpu().numpy()
    assert O.rel_err(dp[:ncp].reshape(om.L, om.N // 2, 2), z["dJdp"]) < TOL
    if is_phase:
        assert O.rel_err(dp[ncp:], z["dJdph"]) < TOL
    assert O.rel_err(to_np(gin), z["g_in"]) < TOL
    assert m.status() == 0


@pytest.mark.gpu
def test_golden_piloss():
    """The PILOSS mesh (piloss.py:18-57) as a ClippedMeshGPU over a permuted full mesh with an output screen,
    against the reference's ClippedNetwork.dot and grad_L2."""
    from meshes_gb300.clipped import ClippedMeshGPU
    z = np.load(os.path.join(GOLDEN, "piloss_N4.npz"))
    om = O.OracleMesh(N=int(z["N"]), L=int(z["L"]), crossing="mzi", lens=list(z["lens"]), shifts=list(z["shifts"]),
                      p=z["p"], s=z["s"], perm=z["perm"])
    full = _gpu_mesh(om, z["ph"], str(z["phi_pos"]))
    m = ClippedMeshGPU(full, z["idx_in"], z["idx_out"])
    y = m.dot(torch.tensor(z["x"].astype(np.complex64), device="cuda")).cpu().numpy()
    assert O.rel_err(y, z["y"]) < TOL
    J, dp = m.grad_L2(z["U_target"])
    assert abs(J - float(z["J"])) < 1e-5 * float(z["J"])
    ncp = om.L * (om.N // 2) * 2
    dp = dp.cpu().numpy()
    assert O.rel_err(dp[:ncp].reshape(om.L, om.N // 2, 2), z["dJdp"]) < TOL
    assert O.rel_err(dp[ncp:], z["dJdph"]) < TOL
    assert full.status() == 0


CASES = [
    # (geometry, crossing, N, B, which layers carry a permutation: "all" (PILOSS-like) or "some")
    ("clements", "mzi", 256, 300, "all"), ("clements", "mzi", 256, 4096, "some"), ("clements", "mzi", 10, 7, "all"),
    ("clements", "mzi", 512, 6, "some"), ("reck", "sym", 32, 9, "some"), ("clements", "orth", 64, 40, "all"),
    ("fft", "mzi", 64, 21, "all"), ("fft", "orth", 128, 5, "some"), ("clements", "mzi", 2, 3, "all"),
]


def _perm_case(geo, cr, N, B, which, seed):
    rng = np.random.default_rng(seed)
    om = O.random_mesh(rng, N, geo, cr, 0.0 if cr == "orth" else 0.02)
    rows = np.array([rng.permutation(N) for _ in range(om.L + 1)])
    if which == "some":
        keep = rng.random(om.L + 1) < 0.3
        keep[[0, -1]] = True
        rows[~keep] = np.arange(N)
    om.perm = rows
    real = cr == "orth"
    return rng, om, real, O.unit_columns(rng, N, B, real=real), O.unit_columns(rng, N, B, real=real)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%s-N%d-B%d-%s" % c)
def test_random_permuted_mesh(case):
    rng, om, real, x, t = _perm_case(*case, seed=zlib.crc32(repr(case).encode()))
    m = _gpu_mesh(om)
    assert O.rel_err(to_np(m.dot(to_dev(x, real))), O.propagate(om, x)) < TOL
    n_p = O.CROSSINGS[om.crossing][0]
    dpd = rng.standard_normal((om.L, om.N // 2, n_p)).astype(np.float32)
    dx = O.unit_columns(rng, om.N, x.shape[0], real=real)
    y_ref, dy_ref = O.fwddiff(om, x, dpd, dx)
    y, dy = m.dot(to_dev(x, real), dp=dpd.reshape(-1), dv=to_dev(dx, real))
    assert O.rel_err(to_np(y), y_ref) < TOL and O.rel_err(to_np(dy), dy_ref) < TOL
    g = 2 * (y_ref - t)
    G, _, gin_ref = O.vjp_unitary(om, y_ref, g)
    dp, gin = m.grad_phi(to_dev(y_ref, real), to_dev(g, real), vpos="out")
    assert O.rel_err(dp.cpu().numpy().reshape(om.L, om.N // 2, n_p), O.contract_dp(om, G)) < TOL
    assert O.rel_err(to_np(gin), gin_ref) < TOL
    assert m.status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("cr,N,B", [("mzi", 128, 77), ("orth", 64, 40)])
def test_autograd_permuted_mesh(cr, N, B):
    """mesh_apply on a permuted mesh: the forward kernel on back-propagation tiles and the backward kernel
    share one workspace and its permutation tables."""
    from meshes_gb300.autograd import mesh_apply
    rng, om, real, x, t = _perm_case("clements", cr, N, B, "all", seed=zlib.crc32(("ag%s%d" % (cr, N)).encode()))
    m = _gpu_mesh(om)
    dt = torch.float32 if real else torch.complex64
    xd = torch.tensor(x, dtype=dt, device="cuda", requires_grad=True)
    p = torch.tensor(np.asarray(om.p, np.float32), device="cuda", requires_grad=True)
    y = mesh_apply(m, xd, p)
    y_ref = O.propagate(om, x)
    assert O.rel_err(y.detach().cpu().numpy(), y_ref) < TOL
    tt = torch.tensor(t, dtype=dt, device="cuda")
    loss = (y - tt).abs().pow(2).sum()
    loss.backward()
    G, _, gin_ref = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
    assert O.rel_err(p.grad.cpu().numpy(), O.contract_dp(om, G)) < TOL
    assert O.rel_err(xd.grad.cpu().numpy(), gin_ref) < TOL


@pytest.mark.gpu
def test_invalid_permutation_row_reports_status():
    """A table row that is not a permutation (written through the C ABI, bypassing the host checks) records
    bad geometry and acts as the identity; the valid rows still apply."""
    from meshes_gb300 import _lib
    rng, om, real, x, t = _perm_case("clements", "mzi", 16, 9, "all", seed=5)
    m = _gpu_mesh(om)
    bad = np.array(om.perm, dtype=np.int32)
    bad[2] = 0                                   # every entry 0: not a permutation
    om_ref = O.OracleMesh(N=om.N, L=om.L, crossing="mzi", lens=om.lens, shifts=om.shifts, p=om.p, s=om.s,
                          perm=np.where(np.arange(om.L + 1)[:, None] == 2, np.arange(om.N)[None, :], om.perm))
    lib = _lib.load()
    B = x.shape[0]
    xd = to_dev(x)
    yd = torch.empty_like(xd.t()).t()
    p = m.p_phase
    s = m.p_splitter
    nb = lib.mg_workspace_bytes(0, om.N, om.L, B, 0, m.geo_code, None)
    ws = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    table = torch.tensor(bad, device="cuda")
    _lib.check(lib.mg_build_tiles(0, om.N, om.L, m.geo_code, m.lens.data_ptr(), m.shifts.data_ptr(), None, 0,
                                  p.data_ptr(), om.N, s.data_ptr(), om.N, None, None, None, B, None, ws.data_ptr(), nb,
                                  st), "mg_build_tiles")
    _lib.check(lib.mg_build_perms(0, om.N, om.L, B, 0, m.geo_code, table.data_ptr(), None, ws.data_ptr(), nb, st),
               "mg_build_perms")
    _lib.check(lib.mg_propagate(0, om.N, om.L, B, 0, m.geo_code, xd.data_ptr(), None, yd.data_ptr(), None, om.N, None,
                                0, 0, None, ws.data_ptr(), nb, st), "mg_propagate")
    assert lib.mg_read_status(ws.data_ptr(), 1, st) == 2
    assert O.rel_err(to_np(yd), O.propagate(om_ref, x)) < TOL
    # a plan without MG_GEO_PERM refuses the tables
    assert lib.mg_build_perms(0, om.N, om.L, B, 0, 0, table.data_ptr(), None, ws.data_ptr(), nb, st) != 0


@pytest.mark.gpu
def test_permuted_batch_is_rejected_by_batched_engine():
    from meshes_gb300.batched import kernel_class
    rng, om, real, x, t = _perm_case("clements", "mzi", 16, 3, "some", seed=9)
    with pytest.raises(ValueError):
        kernel_class(_gpu_mesh(om))
