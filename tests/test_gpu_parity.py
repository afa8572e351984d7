"""GPU parity: the sm_103a kernels (through the C ABI, via MeshNetworkGPU) against the complex128
oracle and the reference-generated golden fixtures.

Tolerances (relative Frobenius error ||gpu - ref|| / ||ref||):
  * forward fields, forward derivatives, input gradients, reconstructed inputs: 1e-5
  * parameter gradients dJ/dp: 1e-5 against the exact complex128 adjoint; 2e-4 against central
    differences (their own truncation/rounding error at h=1e-6 dominates there)
"""
import os
import zlib

import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-5


def gpu_mesh(om: "O.OracleMesh", **kw):
    from meshes_gb300 import MeshNetworkGPU
    p = np.asarray(om.p, dtype=np.float32).reshape(-1)
    s = None if om.s is None else np.asarray(om.s, dtype=np.float32)
    if om.fft:
        return MeshNetworkGPU(om.N, om.L, None, None, p, s, om.crossing, is_phase=False, strides=om.strides, **kw)
    return MeshNetworkGPU(om.N, om.L, om.lens, om.shifts, p, s, om.crossing, is_phase=False, **kw)


def to_dev(x, real=False):
    """(B, N) numpy -> (N, B) device tensor with contiguous columns (the reference layout)."""
    dt = np.float32 if real else np.complex64
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(dt))).cuda().t()


def to_np(t):
    return t.t().contiguous().cpu().numpy()


def fixtures():
    """Fixtures of the plain meshes (the phase-screen and lossy fixtures have their own tests)."""
    return sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz") and "_screen_" not in f and "lossy" not in f
                  and not f.startswith(("clipped_", "perm_", "piloss_", "xmesh_", "crossings_", "converter_", "configure_", "errcorr_")))


def load_fixture(name):
    z = np.load(os.path.join(GOLDEN, name))
    kw = dict(lens=z["lens"].tolist(), shifts=z["shifts"].tolist()) if "lens" in z else dict(strides=z["strides"].tolist())
    om = O.OracleMesh(N=int(z["N"]), L=int(z["L"]), crossing=str(z["crossing"]), p=z["p"],
                      s=z["s"] if "s" in z else None, **kw)
    return z, om


@pytest.mark.parametrize("name", fixtures())
def test_golden_forward(name):
    z, om = load_fixture(name)
    m = gpu_mesh(om)
    y = to_np(m.dot(to_dev(z["x"])))
    assert O.rel_err(y, z["y"]) < TOL
    assert m.status() == 0


@pytest.mark.parametrize("name", [f for f in fixtures() if "sym" not in f])
def test_golden_backward(name):
    z, om = load_fixture(name)
    m = gpu_mesh(om)
    dp, gin = m.grad_phi(to_dev(z["y"]), to_dev(z["g"]), vpos="out")
    dp = dp.cpu().numpy().reshape(om.L, om.N // 2, 2)
    assert O.rel_err(dp, z["dJdp"]) < TOL
    assert O.rel_err(to_np(gin), z["g_in"]) < TOL


@pytest.mark.parametrize("name", [f for f in fixtures() if "dy" in np.load(os.path.join(GOLDEN, f))])
def test_golden_fwddiff(name):
    z, om = load_fixture(name)
    m = gpu_mesh(om)
    y, dy = m.dot(to_dev(z["x"]), dp=z["dp_dir"].astype(np.float32).reshape(-1))
    assert O.rel_err(to_np(y), z["y"]) < TOL
    assert O.rel_err(to_np(dy), z["dy"]) < TOL


CASES = [
    # (geometry, crossing, N, B, splitter sigma)
    ("clements", "mzi", 2, 3, 0.02), ("clements", "mzi", 4, 5, 0.0), ("clements", "mzi", 6, 1, 0.02),
    ("clements", "mzi", 8, 33, 0.02), ("clements", "mzi", 10, 7, 0.02), ("clements", "mzi", 30, 17, 0.02),
    ("clements", "mzi", 64, 65, 0.02), ("clements", "mzi", 100, 9, 0.02), ("clements", "mzi", 128, 40, 0.02),
    ("clements", "mzi", 200, 5, 0.01), ("clements", "mzi", 256, 37, 0.02), ("clements", "mzi", 512, 6, 0.02),
    ("reck", "mzi", 8, 9, 0.02), ("reck", "mzi", 64, 31, 0.02), ("reck", "mzi", 130, 3, 0.0),
    ("clements", "sym", 16, 11, 0.02), ("clements", "sym", 96, 10, 0.02), ("reck", "sym", 32, 4, 0.0),
    ("clements", "orth", 8, 13, 0.0), ("clements", "orth", 64, 50, 0.0), ("reck", "orth", 34, 8, 0.0),
    ("clements", "orth", 256, 9, 0.0),
    ("fft", "mzi", 8, 5, 0.02), ("fft", "mzi", 64, 21, 0.02), ("fft", "mzi", 256, 9, 0.02),
    ("fft", "mzi", 512, 4, 0.02), ("butterfly", "mzi", 16, 7, 0.02), ("butterfly", "mzi", 64, 12, 0.02),
    ("fft", "sym", 128, 6, 0.02), ("fft", "orth", 32, 10, 0.0), ("fft", "orth", 256, 3, 0.0),
    ("butterfly", "orth", 32, 5, 0.0),
    # wide nearest-neighbour meshes (512 < N <= 640, 20 modes per lane)
    ("clements", "mzi", 640, 9, 0.02), ("reck", "mzi", 600, 4, 0.02), ("clements", "sym", 520, 6, 0.02),
    ("clements", "orth", 640, 5, 0.0), ("clements", "mzi", 514, 3, 0.0),
]


def _case(geo, cr, N, B, sig, seed):
    rng = np.random.default_rng(seed)
    om = O.random_mesh(rng, N, geo, cr, sig)
    real = cr == "orth"
    x = O.unit_columns(rng, N, B, real=real)
    t = O.unit_columns(rng, N, B, real=real)
    return rng, om, real, x, t


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%s-N%d-B%d" % c[:4])
def test_random_forward(case):
    rng, om, real, x, t = _case(*case, seed=zlib.crc32(repr(case).encode()))
    m = gpu_mesh(om)
    y = to_np(m.dot(to_dev(x, real)))
    ref = O.propagate(om, x)
    assert O.rel_err(y, ref) < TOL
    assert m.status() == 0


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%s-N%d-B%d" % c[:4])
def test_random_backward(case):
    rng, om, real, x, t = _case(*case, seed=zlib.crc32(repr(case).encode()) + 1)
    m = gpu_mesh(om)
    y = O.propagate(om, x)
    g = 2 * (y - t)
    G, xrec, g_in = O.vjp_unitary(om, y, g)
    dp_ref = O.contract_dp(om, G)
    dp, gin = m.grad_phi(to_dev(y, real), to_dev(g, real), vpos="out")
    n_p = O.CROSSINGS[om.crossing][0]
    dp = dp.cpu().numpy().reshape(om.L, om.N // 2, n_p)
    assert O.rel_err(dp, dp_ref) < TOL
    assert O.rel_err(to_np(gin), g_in) < TOL
    assert m.status() == 0


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%s-N%d-B%d" % c[:4])
def test_random_fwddiff(case):
    rng, om, real, x, t = _case(*case, seed=zlib.crc32(repr(case).encode()) + 2)
    m = gpu_mesh(om)
    n_p = O.CROSSINGS[om.crossing][0]
    dpdir = rng.standard_normal((om.L, om.N // 2, n_p)).astype(np.float32)
    dx = O.unit_columns(rng, om.N, x.shape[0], real=real)
    y_ref, dy_ref = O.fwddiff(om, x, dpdir, dx)
    y, dy = m.dot(to_dev(x, real), dp=dpdir.reshape(-1), dv=to_dev(dx, real))
    assert O.rel_err(to_np(y), y_ref) < TOL
    assert O.rel_err(to_np(dy), dy_ref) < TOL


def test_random_nn_layouts():
    """Random shifts and lens per layer, odd shifts included (reference gpu/test.py:32-42)."""
    rng = np.random.default_rng(7)
    for N in (16, 128, 254):
        L = 13
        shifts = rng.integers(0, N - 1, L)
        lens = np.array([rng.integers(0, (N - s) // 2 + 1) for s in shifts])
        p = rng.uniform(0, 2 * np.pi, (L, N // 2, 2)).astype(np.float32)
        s = rng.normal(0, 0.1, (L, N // 2, 2)).astype(np.float32)
        om = O.OracleMesh(N=N, L=L, crossing="mzi", lens=lens.tolist(), shifts=shifts.tolist(), p=p, s=s)
        x = O.unit_columns(rng, N, 19)
        m = gpu_mesh(om)
        assert O.rel_err(to_np(m.dot(to_dev(x))), O.propagate(om, x)) < TOL
        y = O.propagate(om, x)
        g = rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape)
        G, _, gin_ref = O.vjp_unitary(om, y, g)
        dp, gin = m.grad_phi(to_dev(y), to_dev(g), vpos="out")
        assert O.rel_err(dp.cpu().numpy().reshape(L, N // 2, 2), O.contract_dp(om, G)) < TOL
        assert O.rel_err(to_np(gin), gin_ref) < TOL


def test_plain_forward_full_size():
    """Plain forward at the full N=64, L=64, B=1024 Clements shape (seed 1000)."""
    rng = np.random.default_rng(1000)
    om = O.random_mesh(rng, 64, "clements", "mzi", 0.0)
    x = O.unit_columns(rng, 64, 1024)
    m = gpu_mesh(om)
    y = to_np(m.dot(to_dev(x)))
    ref = O.propagate(om, x)
    err = O.rel_err(y, ref)
    U = to_np(m.matrix())
    unit = np.linalg.norm(U.conj().T @ U - np.eye(64))
    print("rel err %.2e  ||UU^H - I|| %.2e" % (err, unit))
    assert err < TOL
    assert unit < 1e-4


def test_determinism_and_inplace():
    rng = np.random.default_rng(3)
    om = O.random_mesh(rng, 128, "clements", "mzi", 0.02)
    x = O.unit_columns(rng, 128, 300)
    m = gpu_mesh(om)
    v = to_dev(x)
    y1 = m.dot(v)
    g = to_dev(rng.standard_normal(x.shape) + 1j * rng.standard_normal(x.shape))
    dp1, gi1 = m.grad_phi(y1, g, vpos="out")
    dp2, gi2 = m.grad_phi(y1, g, vpos="out")
    assert torch.equal(dp1, dp2) and torch.equal(gi1, gi2)
    v2 = v.clone()
    m.dot(v2, out=v2)             # in place
    assert torch.equal(v2, y1)


def test_edge_sizes():
    from meshes_gb300 import MeshNetworkGPU
    rng = np.random.default_rng(5)
    om = O.random_mesh(rng, 16, "clements", "mzi", 0.0)
    m = gpu_mesh(om)
    v0 = torch.zeros((16, 0), dtype=torch.complex64, device="cuda")
    assert m.dot(v0).shape == (16, 0)
    # L = 0 is the identity
    m0 = MeshNetworkGPU(16, 0, [], [], np.zeros(0, np.float32), None, "mzi", is_phase=False)
    x = O.unit_columns(rng, 16, 4)
    assert np.allclose(to_np(m0.dot(to_dev(x))), x)
    # accumulate semantics of grad_phi(out_dp=...)
    y = O.propagate(om, x)
    g = 2 * y
    dp_a, _ = m.grad_phi(to_dev(y), to_dev(g), vpos="out")
    acc = torch.ones_like(dp_a)
    m.grad_phi(to_dev(y), to_dev(g), vpos="out", out_dp=acc)
    assert torch.allclose(acc, dp_a + 1, atol=1e-6)


def test_bad_geometry_reports_status():
    """Malformed device geometry (shift + 2*len > N) is caught by the kernel, not a fault."""
    from meshes_gb300 import _lib
    lib = _lib.load()
    N, L, B = 8, 2, 4
    lens = torch.tensor([4, 4], dtype=torch.int32, device="cuda")
    shifts = torch.tensor([0, 1], dtype=torch.int32, device="cuda")   # layer 1: 1 + 8 > 8
    p = torch.zeros(L * N // 2 * 2, device="cuda")
    u = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    out = torch.empty_like(u)
    nb = lib.mg_workspace_bytes(0, N, L, B, 0, 0, None)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mg_workspace_init(ws.data_ptr(), nb, st) == 0
    assert lib.mg_fwdprop(N, L, B, lens.data_ptr(), shifts.data_ptr(), p.data_ptr(), N, None, 0, u.data_ptr(),
                          out.data_ptr(), N, 0, ws.data_ptr(), nb, st) == 0
    assert lib.mg_read_status(ws.data_ptr(), 1, st) == 2
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0


def test_width_limits():
    """N up to 640 (the reference's limit, gpu/mesh.py:83) for nearest-neighbour meshes; beyond, or a
    butterfly above 512, is refused before any launch."""
    from meshes_gb300 import _lib
    lib = _lib.load()
    assert lib.mg_workspace_bytes(0, 640, 640, 8, 0, 0, None) > 0
    assert lib.mg_workspace_bytes(2, 600, 10, 8, 2, 0, None) > 0
    assert lib.mg_workspace_bytes(0, 642, 640, 8, 0, 0, None) == 0
    assert "640" in _lib.last_error()
    assert lib.mg_workspace_bytes(0, 1024, 10, 8, 0, 1, None) == 0


def test_argument_errors():
    from meshes_gb300 import _lib
    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    assert lib.mg_fwdprop(7, 1, 1, None, None, None, 0, None, 0, None, None, 7, 0, None, 0, st) == -1
    assert "even" in _lib.last_error()
    assert lib.mg_fwdprop(1024, 1, 1, None, None, None, 0, None, 0, None, None, 1024, 0, None, 0, st) == -1
    assert lib.mg_fwdprop(8, 1, 1, None, None, None, 0, None, 0, None, None, 8, 0, None, 0, st) == -2


@pytest.mark.parametrize("cr,N,B", [("mzi", 128, 77), ("orth", 64, 40), ("sym", 32, 9), ("mzi", 512, 5)])
def test_shared_tiles_and_fused_l2_target(cr, N, B):
    """One coefficient pass (back-propagation tiles) serves the forward kernel (op 3); the L2 gradient
    2 (y - t) is formed inside the backward kernel (mg_propagate_l2)."""
    from meshes_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(N + B)
    om = O.random_mesh(rng, N, "clements", cr, 0.02)
    real = cr == "orth"
    x = O.unit_columns(rng, N, B, real=real)
    t = O.unit_columns(rng, N, B, real=real)
    m = gpu_mesh(om)
    dt = torch.float32 if real else torch.complex64
    xd = torch.tensor(x, dtype=dt, device="cuda")
    td = torch.tensor(t, dtype=dt, device="cuda")
    y = torch.empty_like(xd)
    gx = torch.empty_like(xd)
    dp = torch.empty(m.p_phase.numel(), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    nb = lib.mg_workspace_bytes(2, N, om.L, B, m.crossing, 0, None)
    ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
    assert lib.mg_workspace_init(ws.data_ptr(), nb, st) == 0
    s = m.p_splitter
    ldp, lds = N // 2 * m.X_np, N // 2 * m.X_ns
    assert lib.mg_build_tiles(2, N, om.L, 0, m.lens.data_ptr(), m.shifts.data_ptr(), None, m.crossing,
                              m.p_phase.data_ptr(), ldp, s.data_ptr() if s.numel() else None, lds, None, None, None,
                              B, None, ws.data_ptr(), nb, st) == 0
    assert lib.mg_propagate(3, N, om.L, B, m.crossing, 0, xd.data_ptr(), None, y.data_ptr(), None, N, None, 0, 0,
                            None, ws.data_ptr(), nb, st) == 0, _lib.last_error()
    assert lib.mg_propagate_l2(N, om.L, B, m.crossing, 0, y.data_ptr(), td.data_ptr(), None, gx.data_ptr(), N,
                               dp.data_ptr(), ldp, 0, None, ws.data_ptr(), nb, st) == 0, _lib.last_error()
    y_ref = O.propagate(om, x)
    G, _, gin = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
    n_p = O.CROSSINGS[cr][0]
    assert O.rel_err(y.cpu().numpy(), y_ref) < TOL
    assert O.rel_err(gx.cpu().numpy(), gin) < TOL
    assert O.rel_err(dp.cpu().numpy().reshape(om.L, N // 2, n_p), O.contract_dp(om, G)) < TOL
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0


@pytest.mark.parametrize("pos", ["out", "in"])
def test_golden_phase_screen(pos):
    """is_phase=True (forbidden by the reference GPU API, defined by its CPU path) against the reference's
    own dot / fwd-diff / dot_vjp with a nonzero phase screen."""
    from meshes_gb300 import MeshNetworkGPU
    z = np.load(os.path.join(GOLDEN, "clements_mzi_N8_screen_%s.npz" % pos))
    N, L = int(z["N"]), int(z["L"])
    ncp = L * (N // 2) * 2
    p_full = np.concatenate([z["p"].reshape(-1), z["ph"]]).astype(np.float32)
    m = MeshNetworkGPU(N, L, z["lens"], z["shifts"], p_full, z["s"].astype(np.float32), "mzi", phi_pos=pos,
                       is_phase=True)
    assert O.rel_err(to_np(m.dot(to_dev(z["x"]))), z["y"]) < TOL
    y, dy = m.dot(to_dev(z["x"]), dp=np.concatenate([z["dp_dir"].reshape(-1), z["dph_dir"]]).astype(np.float32))
    assert O.rel_err(to_np(y), z["y"]) < TOL and O.rel_err(to_np(dy), z["dy"]) < TOL
    dp, gin = m.grad_phi(to_dev(z["y"]), to_dev(z["g"]), vpos="out")
    dp = dp.cpu().numpy()
    assert O.rel_err(dp[:ncp].reshape(L, N // 2, 2), z["dJdp"]) < TOL
    assert O.rel_err(dp[ncp:], z["dJdph"]) < TOL
    assert O.rel_err(to_np(gin), z["g_in"]) < TOL


@pytest.mark.parametrize("pos", ["out", "in"])
@pytest.mark.parametrize("geo,N,B", [("clements", 64, 33), ("fft", 128, 20), ("reck", 30, 7)])
def test_random_phase_screen(pos, geo, N, B):
    from meshes_gb300 import MeshNetworkGPU
    rng = np.random.default_rng(zlib.crc32(("%s%s%d" % (pos, geo, N)).encode()))
    om = O.random_mesh(rng, N, geo, "mzi", 0.02)
    ph = rng.uniform(0, 2 * np.pi, N).astype(np.float32)
    p_full = np.concatenate([np.asarray(om.p, np.float32).reshape(-1), ph])
    kw = dict(strides=om.strides) if om.fft else {}
    m = MeshNetworkGPU(N, om.L, None if om.fft else om.lens, None if om.fft else om.shifts, p_full,
                       np.asarray(om.s, np.float32), "mzi", phi_pos=pos, is_phase=True, **kw)
    x = O.unit_columns(rng, N, B).astype(np.complex64)
    t = O.unit_columns(rng, N, B).astype(np.complex64)
    y_ref = O.propagate_screened(om, x, ph, pos)
    assert O.rel_err(to_np(m.dot(to_dev(x))), y_ref) < TOL
    # forward-mode derivative along a random direction of all phases, screen included
    dpd = rng.standard_normal(p_full.size).astype(np.float32)
    dpd[: om.p.size][~np.broadcast_to(om.active_mask()[..., None], om.p.shape).reshape(-1)] = 0
    _, dy = m.dot(to_dev(x), dp=dpd)
    _, dy_ref = O.fwddiff_screened(om, x, ph, pos, dpd[: om.p.size], dpd[om.p.size:])
    assert O.rel_err(to_np(dy), dy_ref) < TOL
    # gradient from the input (vpos "in") with a callable objective, then accumulated into out_dp
    tt = to_dev(t)
    dp, gin = m.grad_phi(to_dev(x), lambda yy: 2 * (yy - tt))
    dp_ref, dph_ref, gin_ref = O.grad_screened(om, y_ref, 2 * (y_ref - t), ph, pos)
    dp = dp.cpu().numpy()
    assert O.rel_err(dp[: om.p.size].reshape(om.p.shape), dp_ref) < TOL
    assert O.rel_err(dp[om.p.size:], dph_ref) < TOL
    assert O.rel_err(to_np(gin), gin_ref) < TOL
    acc = torch.ones(p_full.size, dtype=torch.float32, device="cuda")
    m.grad_phi(to_dev(x), lambda yy: 2 * (yy - tt), out_dp=acc)
    assert O.rel_err(acc.cpu().numpy() - 1.0, dp) < 1e-6


@pytest.mark.parametrize("cr,N,B", [("mzi", 256, 4096), ("mzi", 256, 2500), ("mzi", 512, 3000), ("orth", 256, 3000)])
def test_split_launch_parity(cr, N, B):
    """Split launches (two CTA kinds per SM, V and V-1 vectors per lane group) against the oracle, forward
    and back-propagation, and bit-identical to themselves on a second run."""
    from meshes_gb300 import _lib
    import ctypes
    lib = _lib.load()
    rng = np.random.default_rng(N * 7 + B)
    om = O.random_mesh(rng, N, "clements", cr, 0.02 if cr == "mzi" else 0.0)
    real = cr == "orth"
    x = O.unit_columns(rng, N, B, real=real)
    g = O.unit_columns(rng, N, B, real=real)
    m = gpu_mesh(om)
    dt = torch.float32 if real else torch.complex64
    xd, gd = torch.tensor(x, dtype=dt, device="cuda"), torch.tensor(g, dtype=dt, device="cuda")
    y, gx = torch.empty_like(xd), torch.empty_like(xd)
    dp = torch.empty(m.p_phase.numel(), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    s = m.p_splitter
    ldp, lds = N // 2 * m.X_np, N // 2 * m.X_ns
    outs = []
    for op in (0, 2):
        cfg = _lib.config(split=1)
        info = _lib.mg_plan_info()
        assert lib.mg_plan(op, N, om.L, B, m.crossing, 0, _lib.cfg_ptr(cfg), ctypes.byref(info)) == 0
        assert info.nA > 0 and info.grid > info.nA                # really split
        nb = info.total
        ws = torch.zeros(nb, dtype=torch.uint8, device="cuda")
        assert lib.mg_build_tiles(op, N, om.L, 0, m.lens.data_ptr(), m.shifts.data_ptr(), None, m.crossing,
                                  m.p_phase.data_ptr(), ldp, s.data_ptr() if s.numel() else None, lds, None, None,
                                  None, B, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st) == 0, _lib.last_error()
        for rep in range(2):
            if op == 0:
                assert lib.mg_propagate(0, N, om.L, B, m.crossing, 0, xd.data_ptr(), None, y.data_ptr(), None, N,
                                        None, 0, 0, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st) == 0, _lib.last_error()
                outs.append(y.clone())
            else:
                assert lib.mg_propagate(2, N, om.L, B, m.crossing, 0, y.data_ptr(), gd.data_ptr(), None,
                                        gx.data_ptr(), N, dp.data_ptr(), ldp, 0, _lib.cfg_ptr(cfg), ws.data_ptr(),
                                        nb, st) == 0, _lib.last_error()
                outs.append((gx.clone(), dp.clone()))
        assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
    assert torch.equal(outs[0], outs[1])
    assert torch.equal(outs[2][0], outs[3][0]) and torch.equal(outs[2][1], outs[3][1])
    y_ref = O.propagate(om, x)
    G, _, gin = O.vjp_unitary(om, y_ref, g)
    n_p = O.CROSSINGS[cr][0]
    assert O.rel_err(outs[0].cpu().numpy(), y_ref) < TOL
    assert O.rel_err(outs[2][0].cpu().numpy(), gin) < TOL
    assert O.rel_err(outs[2][1].cpu().numpy().reshape(om.L, N // 2, n_p), O.contract_dp(om, G)) < TOL


@pytest.mark.parametrize("N,M", [(256, 8), (128, 4)])
@pytest.mark.parametrize("V", [2, 4])
def test_packed_crossing_tiles(N, M, V):
    """Explicit full-warp tiles whose forward, forward-mode derivative and back-propagation take the vectors
    two at a time (packed f32x2 crossings), on a ragged batch, against the oracle."""
    from meshes_gb300 import _lib
    import ctypes
    lib = _lib.load()
    B = 301
    rng = np.random.default_rng(N * 31 + V)
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    x = O.unit_columns(rng, N, B)
    dx = O.unit_columns(rng, N, B)
    g = O.unit_columns(rng, N, B)
    dpdir = rng.standard_normal((om.L, N // 2, 2)).astype(np.float32)
    m = gpu_mesh(om)
    xd, dxd, gd = (torch.tensor(a, dtype=torch.complex64, device="cuda") for a in (x, dx, g))
    y, dy, gx = torch.empty_like(xd), torch.empty_like(xd), torch.empty_like(xd)
    dpd = torch.tensor(dpdir.reshape(-1), device="cuda")
    dp = torch.empty(m.p_phase.numel(), device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    s = m.p_splitter
    ldp, lds = N // 2 * m.X_np, N // 2 * m.X_ns
    for op in (0, 1, 2):
        cfg = _lib.config(M, V, 8, 0, 2, 2)
        info = _lib.mg_plan_info()
        assert lib.mg_plan(op, N, om.L, B, m.crossing, 0, _lib.cfg_ptr(cfg), ctypes.byref(info)) == 0
        assert (info.M, info.V, info.G) == (M, V, 32)
        nb = info.total
        ws = torch.zeros(nb, dtype=torch.uint8, device="cuda")
        assert lib.mg_build_tiles(op, N, om.L, 0, m.lens.data_ptr(), m.shifts.data_ptr(), None, m.crossing,
                                  m.p_phase.data_ptr(), ldp, s.data_ptr() if s.numel() else None, lds,
                                  dpd.data_ptr() if op == 1 else None, None, None, B, _lib.cfg_ptr(cfg),
                                  ws.data_ptr(), nb, st) == 0, _lib.last_error()
        if op == 0:
            rc = lib.mg_propagate(0, N, om.L, B, m.crossing, 0, xd.data_ptr(), None, y.data_ptr(), None, N, None, 0,
                                  0, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st)
        elif op == 1:
            rc = lib.mg_propagate(1, N, om.L, B, m.crossing, 0, xd.data_ptr(), dxd.data_ptr(), y.data_ptr(),
                                  dy.data_ptr(), N, None, 0, 0, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st)
        else:
            rc = lib.mg_propagate(2, N, om.L, B, m.crossing, 0, y.data_ptr(), gd.data_ptr(), None, gx.data_ptr(), N,
                                  dp.data_ptr(), ldp, 0, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st)
        assert rc == 0, _lib.last_error()
        assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
        if op == 1:
            y_ref, dy_ref = O.fwddiff(om, x, dpdir, dx)
            assert O.rel_err(y.cpu().numpy(), y_ref) < TOL
            assert O.rel_err(dy.cpu().numpy(), dy_ref) < TOL
    y_ref = O.propagate(om, x)
    G, _, gin = O.vjp_unitary(om, y.cpu().numpy().astype(np.complex128), g)
    assert O.rel_err(y.cpu().numpy(), y_ref) < TOL
    assert O.rel_err(gx.cpu().numpy(), gin) < TOL
    assert O.rel_err(dp.cpu().numpy().reshape(om.L, N // 2, 2), O.contract_dp(om, G)) < TOL


def test_coefficient_trigonometry_matches_library():
    """The coefficient precompute's own double sin/cos (Cody-Waite reduction + Taylor series) agrees with
    the CUDA library's to a few units in the last place, over phase-like, small and large arguments; its
    tile-precision version (values rounded to float32 afterwards) and its small-angle version for splitting
    errors (|x| < 1/8 by series, other arguments through the tile version, NaN passed through) to 1e-13."""
    from meshes_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(77)
    x = np.concatenate([rng.uniform(0, 2 * np.pi, 20000), rng.uniform(-20, 20, 20000),
                        rng.normal(0, 0.02, 20000), rng.uniform(-1e5, 1e5, 5000),
                        rng.uniform(-0.125, 0.125, 20000), np.nextafter(0.125, 0) * np.array([1.0, -1.0]),
                        np.arange(-64, 65) * np.pi / 4, [0.0, 1e-30, -1e-30, 0.125, -0.125, 2.0 ** 20, 3e7]])
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    out = torch.empty(6 * x.size, dtype=torch.float64, device="cuda")
    assert lib.mg_trig_check(xd.data_ptr(), out.data_ptr(), x.size, torch.cuda.current_stream().cuda_stream) == 0
    out = out.view(-1, 6).abs()
    assert out[:, :2].max().item() < 1e-15
    assert out[:, 2:].max().item() < 1e-13
    # NaN takes the library path of every version and comes back as NaN
    xn = torch.tensor([float("nan")], dtype=torch.float64, device="cuda")
    on = torch.empty(6, dtype=torch.float64, device="cuda")
    assert lib.mg_trig_check(xn.data_ptr(), on.data_ptr(), 1, torch.cuda.current_stream().cuda_stream) == 0
    assert torch.isnan(on).all().item()


@pytest.mark.parametrize("name", ["clipped_squarenet_N4.npz", "clipped_qrnet_N4.npz"])
def test_golden_clipped_mesh(name):
    """SquareNet and QR meshes (ClippedNetwork, reference mesh.py:718-802) against the reference's own dot
    and grad_L2 with the phase screen on."""
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300.clipped import ClippedMeshGPU
    z = np.load(os.path.join(GOLDEN, name))
    N, L = int(z["N"]), int(z["L"])
    full = MeshNetworkGPU(N, L, z["lens"], z["shifts"], np.concatenate([z["p"].reshape(-1), z["ph"]]).astype(np.float32),
                          z["s"].astype(np.float32), "mzi", phi_pos=str(z["phi_pos"]), is_phase=True)
    m = ClippedMeshGPU(full, z["idx_in"], z["idx_out"])
    y = m.dot(torch.tensor(z["x"].astype(np.complex64), device="cuda")).cpu().numpy()
    assert O.rel_err(y, z["y"]) < TOL
    J, dp = m.grad_L2(z["U_target"])
    assert abs(J - float(z["J"])) < 1e-5 * float(z["J"])
    ncp = L * (N // 2) * 2
    dp = dp.cpu().numpy()
    assert O.rel_err(dp[:ncp].reshape(L, N // 2, 2), z["dJdp"]) < TOL
    assert O.rel_err(dp[ncp:], z["dJdph"]) < TOL


def test_conjugated_and_negated_views():
    """Inputs that are lazily conjugated or negated views (torch's conj/neg bits) give the results of their
    materialised values: the library reads raw memory, so such views are resolved before a call."""
    rng = np.random.default_rng(77)
    om = O.random_mesh(rng, 16, "clements", "mzi", 0.02)
    m = gpu_mesh(om)
    U = torch.tensor(O.haar_unitary(rng, 16).astype(np.complex64), device="cuda")
    v = U.t().conj()
    assert v.is_conj()
    ref = m.dot(v.resolve_conj())
    assert torch.equal(m.dot(v), ref)
    y = O.propagate(om, U.t().conj().t().cpu().numpy())
    assert O.rel_err(to_np(m.dot(v)), y) < TOL
    g = torch.tensor(O.unit_columns(rng, 16, 16).astype(np.complex64), device="cuda").t()
    dp1, g1 = m.grad_phi(v, g.conj())
    dp2, g2 = m.grad_phi(v.resolve_conj(), g.conj().resolve_conj())
    assert torch.equal(dp1, dp2) and torch.equal(g1, g2)


@pytest.mark.parametrize("geo", ["clements", "reck"])
@pytest.mark.parametrize("N,V,W", [(128, 1, 4), (128, 2, 4), (96, 1, 1), (112, 2, 2)])
def test_small_mesh_backprop_tiles(geo, N, V, W):
    """The small-mesh nearest-neighbour back-propagation tiles (4 modes and 1 or 2 vectors per lane, a vector over
    the whole warp) with the fused L2 gradient, on ragged batches, against the complex128 adjoint; the plan reports
    the requested tile."""
    from meshes_gb300 import _lib
    import ctypes
    lib = _lib.load()
    rng = np.random.default_rng(N * 5 + V * 3 + W)
    for sig, B in ((0.0, 128), (0.02, 77)):
        om = O.random_mesh(rng, N, geo, "mzi", sig)
        x = O.unit_columns(rng, N, B)
        t = O.unit_columns(rng, N, B)
        m = gpu_mesh(om)
        xd = torch.tensor(x, dtype=torch.complex64, device="cuda")
        td = torch.tensor(t, dtype=torch.complex64, device="cuda")
        y, gx = torch.empty_like(xd), torch.empty_like(xd)
        dp = torch.empty(m.p_phase.numel(), device="cuda")
        st = torch.cuda.current_stream().cuda_stream
        s = m.p_splitter
        cfg = _lib.config(4, V, W, 0, 0, 2)
        info = _lib.mg_plan_info()
        assert lib.mg_plan(2, N, om.L, B, m.crossing, 0, _lib.cfg_ptr(cfg), ctypes.byref(info)) == 0, _lib.last_error()
        assert (info.M, info.V, info.G) == (4, V, 32)
        ws = torch.zeros(info.total, dtype=torch.uint8, device="cuda")
        assert lib.mg_build_tiles(2, N, om.L, 0, m.lens.data_ptr(), m.shifts.data_ptr(), None, m.crossing,
                                  m.p_phase.data_ptr(), N, s.data_ptr() if s.numel() else None, N, None, None, None,
                                  B, _lib.cfg_ptr(cfg), ws.data_ptr(), info.total, st) == 0, _lib.last_error()
        assert lib.mg_propagate(3, N, om.L, B, m.crossing, 0, xd.data_ptr(), None, y.data_ptr(), None, N, None, 0, 0,
                                _lib.cfg_ptr(cfg), ws.data_ptr(), info.total, st) == 0, _lib.last_error()
        assert lib.mg_propagate_l2(N, om.L, B, m.crossing, 0, y.data_ptr(), td.data_ptr(), None, gx.data_ptr(), N,
                                   dp.data_ptr(), N, 0, _lib.cfg_ptr(cfg), ws.data_ptr(), info.total, st) == 0, \
            _lib.last_error()
        assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
        assert O.rel_err(y.cpu().numpy(), y_ref) < TOL
        assert O.rel_err(gx.cpu().numpy(), gin) < TOL
        assert O.rel_err(dp.cpu().numpy().reshape(om.L, N // 2, 2), O.contract_dp(om, G)) < TOL


@pytest.mark.parametrize("geo", ["clements", "reck"])
@pytest.mark.parametrize("N,M,V", [(64, 2, 1), (64, 2, 2), (64, 2, 4), (40, 2, 2), (128, 4, 1), (96, 4, 2)])
def test_small_mesh_forward_tiles(geo, N, M, V):
    """The small-mesh nearest-neighbour forward tiles (2 or 4 modes and 1 to 4 vectors per lane, a vector over the
    whole warp) on ragged batches, with and without splitter errors, against the oracle; the plan reports the
    requested tile."""
    from meshes_gb300 import _lib
    import ctypes
    lib = _lib.load()
    rng = np.random.default_rng(N * 7 + M * 3 + V)
    for sig, B in ((0.0, 1024), (0.02, 77)):
        om = O.random_mesh(rng, N, geo, "mzi", sig)
        x = O.unit_columns(rng, N, B)
        m = gpu_mesh(om)
        xd = torch.tensor(x, dtype=torch.complex64, device="cuda")
        y = torch.empty_like(xd)
        st = torch.cuda.current_stream().cuda_stream
        s = m.p_splitter
        cfg = _lib.config(M, V, 0, 0, 0, 2)
        info = _lib.mg_plan_info()
        assert lib.mg_plan(0, N, om.L, B, m.crossing, 0, _lib.cfg_ptr(cfg), ctypes.byref(info)) == 0, _lib.last_error()
        assert (info.M, info.V, info.G) == (M, V, 32)
        ws = torch.zeros(info.total, dtype=torch.uint8, device="cuda")
        assert lib.mg_build_tiles(0, N, om.L, 0, m.lens.data_ptr(), m.shifts.data_ptr(), None, m.crossing,
                                  m.p_phase.data_ptr(), N, s.data_ptr() if s.numel() else None, N, None, None, None,
                                  B, _lib.cfg_ptr(cfg), ws.data_ptr(), info.total, st) == 0, _lib.last_error()
        assert lib.mg_propagate(0, N, om.L, B, m.crossing, 0, xd.data_ptr(), None, y.data_ptr(), None, N, None, 0, 0,
                                _lib.cfg_ptr(cfg), ws.data_ptr(), info.total, st) == 0, _lib.last_error()
        assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
        assert O.rel_err(y.cpu().numpy(), O.propagate(om, x)) < TOL
