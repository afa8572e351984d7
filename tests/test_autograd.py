"""torch.autograd through the kernels (meshes_gb300.autograd), checked against the complex128 oracle.

Tolerances: relative Frobenius error 1e-5 for outputs and gradients against the exact complex128
adjoint; central differences (h = 1e-6, complex128) agree with the float32 GPU gradient to 1e-4
relative per checked component (the central differences carry their own O(h^2) and rounding error,
and a single component of the float32 gradient is not averaged like a Frobenius norm).
"""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu


def gpu_mesh(om):
    from meshes_gb300 import MeshNetworkGPU
    p = np.asarray(om.p, np.float32).reshape(-1)
    s = None if om.s is None else np.asarray(om.s, np.float32)
    if om.fft:
        return MeshNetworkGPU(om.N, om.L, None, None, p, s, om.crossing, is_phase=False, strides=om.strides)
    return MeshNetworkGPU(om.N, om.L, om.lens, om.shifts, p, s, om.crossing, is_phase=False)


@pytest.mark.parametrize("geo,cr,N,B", [("clements", "mzi", 64, 37), ("reck", "mzi", 32, 9), ("fft", "mzi", 128, 20),
                                        ("clements", "sym", 16, 5), ("clements", "orth", 64, 33),
                                        ("butterfly", "orth", 16, 7)])
def test_autograd_matches_oracle(geo, cr, N, B):
    from meshes_gb300.autograd import mesh_apply
    rng = np.random.default_rng(N + B)
    om = O.random_mesh(rng, N, geo, cr, 0.02)
    real = cr == "orth"
    x = O.unit_columns(rng, N, B, real=real)
    t = O.unit_columns(rng, N, B, real=real)
    m = gpu_mesh(om)
    dt = torch.float32 if real else torch.complex64
    xd = torch.tensor(x, dtype=dt, device="cuda", requires_grad=True)
    pd = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
    y = mesh_apply(m, xd, pd)
    loss = ((y - torch.tensor(t, dtype=dt, device="cuda")).abs() ** 2).sum()
    loss.backward()
    y_ref = O.propagate(om, x)
    G, _, gin = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
    assert O.rel_err(y.detach().cpu().numpy(), y_ref) < 1e-5
    assert O.rel_err(pd.grad.cpu().numpy(), O.contract_dp(om, G)) < 1e-5
    assert O.rel_err(xd.grad.cpu().numpy(), gin) < 1e-5


@pytest.mark.parametrize("geo,cr,N,B", [("clements", "mzi", 64, 37), ("reck", "mzi", 32, 9), ("fft", "mzi", 128, 20),
                                        ("clements", "orth", 64, 33)])
def test_l2_loss_matches_oracle(geo, cr, N, B):
    """mesh_l2_loss: J = sum |U x - t|^2 with the loss gradient formed inside the back-propagation kernel;
    J, dJ/dp, dJ/dx and dJ/dt against the complex128 adjoint, scaled by a grad_output of 0.5."""
    from meshes_gb300.autograd import mesh_l2_loss
    rng = np.random.default_rng(7 * N + B)
    om = O.random_mesh(rng, N, geo, cr, 0.02)
    real = cr == "orth"
    x = O.unit_columns(rng, N, B, real=real)
    t = O.unit_columns(rng, N, B, real=real)
    m = gpu_mesh(om)
    dt = torch.float32 if real else torch.complex64
    xd = torch.tensor(x, dtype=dt, device="cuda", requires_grad=True)
    td = torch.tensor(t, dtype=dt, device="cuda", requires_grad=True)
    pd = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
    J = mesh_l2_loss(m, xd, td, pd)
    (0.5 * J).backward()
    y_ref = O.propagate(om, x)
    J_ref = float(np.sum(np.abs(y_ref - t) ** 2))
    G, _, gin = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
    assert abs(float(J.detach()) - J_ref) < 1e-5 * J_ref
    assert O.rel_err(pd.grad.cpu().numpy(), 0.5 * O.contract_dp(om, G)) < 1e-5
    assert O.rel_err(xd.grad.cpu().numpy(), 0.5 * gin) < 1e-5
    assert O.rel_err(td.grad.cpu().numpy(), -(y_ref - t)) < 1e-5
    assert m.status() == 0


def test_l2_loss_equals_mesh_apply_form():
    """mesh_l2_loss gives bitwise the loss and gradients of sum(view_as_real(y - t)^2) through mesh_apply: the
    kernel's 2 (y - t) is torch's gradient of that sum, and both reach the same back-propagation kernel."""
    from meshes_gb300.autograd import mesh_apply, mesh_l2_loss
    rng = np.random.default_rng(4242)
    N, B = 128, 128
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    m = gpu_mesh(om)
    x = torch.tensor(O.unit_columns(rng, N, B), dtype=torch.complex64, device="cuda")
    t = torch.tensor(O.unit_columns(rng, N, B), dtype=torch.complex64, device="cuda")
    grads = []
    for fused in (True, False):
        xd = x.clone().requires_grad_(True)
        pd = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
        J = mesh_l2_loss(m, xd, t, pd) if fused else torch.view_as_real(mesh_apply(m, xd, pd) - t).square().sum()
        J.backward()
        grads.append((J.detach(), pd.grad, xd.grad))
    for a, b in zip(*grads):
        assert torch.equal(a, b)


def test_fused_adam_matches_torch_adam():
    """autograd.Adam (one mg_adam_step launch per tensor) against torch.optim.Adam on the same 30 seeded
    gradients: parameters and both moments within float32 rounding (1e-5 absolute on parameters in [0, 2 pi], a
    thousandth of one lr = 1e-2 step; 1e-5 relative on the moments); the device step count advances by one per
    step."""
    from meshes_gb300.autograd import Adam
    rng = np.random.default_rng(77)
    p0 = rng.uniform(0, 2 * np.pi, (65, 32, 2)).astype(np.float32)
    pa = torch.tensor(p0, device="cuda", requires_grad=True)
    pt = torch.tensor(p0, device="cuda", requires_grad=True)
    oa = Adam([pa], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    ot = torch.optim.Adam([pt], lr=1e-2, betas=(0.9, 0.999), eps=1e-8, foreach=False)
    for k in range(30):
        g = torch.tensor(rng.standard_normal(p0.shape).astype(np.float32) * (10.0 ** rng.uniform(-3, 1)), device="cuda")
        pa.grad, pt.grad = g.clone(), g.clone()
        oa.step()
        ot.step()
        assert float((pa - pt).abs().max()) < 1e-5, k
    st = ot.state[pt]
    assert float((oa.exp_avg[0] - st["exp_avg"]).abs().max()) <= 1e-5 * float(st["exp_avg"].abs().max())
    assert float((oa.exp_avg_sq[0] - st["exp_avg_sq"]).abs().max()) <= 1e-5 * float(st["exp_avg_sq"].abs().max())
    assert oa.state[0].tolist() == [30, 0]


@pytest.mark.parametrize("pos", ["out", "in"])
def test_autograd_with_phase_screen(pos):
    """mesh_apply on a mesh with a phase screen: the screen phases get their gradient too."""
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300.autograd import mesh_apply
    rng = np.random.default_rng(91 if pos == "out" else 92)
    N, B = 64, 21
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    ph = rng.uniform(0, 2 * np.pi, N)
    m = MeshNetworkGPU(N, om.L, om.lens, om.shifts, np.concatenate([np.asarray(om.p, np.float32).reshape(-1),
                                                                   ph.astype(np.float32)]),
                       np.asarray(om.s, np.float32), "mzi", phi_pos=pos, is_phase=True)
    x = O.unit_columns(rng, N, B)
    t = O.unit_columns(rng, N, B)
    xd = torch.tensor(x, dtype=torch.complex64, device="cuda", requires_grad=True)
    pd = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
    phd = torch.tensor(ph, dtype=torch.float32, device="cuda", requires_grad=True)
    y = mesh_apply(m, xd, pd, phd)
    loss = ((y - torch.tensor(t, dtype=torch.complex64, device="cuda")).abs() ** 2).sum()
    loss.backward()
    y_ref = O.propagate_screened(om, x, ph.astype(np.float32), pos)
    dp_ref, dph_ref, gin_ref = O.grad_screened(om, y_ref, 2 * (y_ref - t), ph.astype(np.float32), pos)
    assert O.rel_err(y.detach().cpu().numpy(), y_ref) < 1e-5
    assert O.rel_err(pd.grad.cpu().numpy(), dp_ref) < 1e-5
    assert O.rel_err(phd.grad.cpu().numpy(), dph_ref) < 1e-5
    assert O.rel_err(xd.grad.cpu().numpy(), gin_ref) < 1e-5


def _loss_from_layer(om, acts, l, T, t):
    """sum |y - t|^2 propagating from the input of layer l with transfer matrices T (complex128)."""
    u = np.ascontiguousarray(acts[l].T).copy()
    for n in range(l, om.L):
        O._apply_layer(om, n, T, u)
    return float(np.sum(np.abs(u.T - t) ** 2))


def test_differentiated_imperfect_clements_full_size():
    """Clements mzi, N=256, L=256 (32640 MZIs), splitting errors N(0, 0.02), B=4096 unit-norm inputs,
    loss sum |y - y_t|^2: forward + autograd backward against the exact complex128 adjoint on the whole
    batch, and against complex128 central differences (h=1e-6) on 64 random MZIs (theta and phi)."""
    from meshes_gb300.autograd import mesh_apply
    rng = np.random.default_rng(1002)
    N, B = 256, 4096
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    x = O.unit_columns(rng, N, B)
    t = O.unit_columns(rng, N, B)
    m = gpu_mesh(om)
    xd = torch.tensor(x, dtype=torch.complex64, device="cuda")
    pd = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
    y = mesh_apply(m, xd, pd)
    loss = ((y - torch.tensor(t, dtype=torch.complex64, device="cuda")).abs() ** 2).sum()
    loss.backward()
    y_ref = O.propagate(om, x)
    G, _, _ = O.vjp_unitary(om, y_ref, 2 * (y_ref - t))
    dp_ref = O.contract_dp(om, G)
    e_y = O.rel_err(y.detach().cpu().numpy(), y_ref)
    e_dp = O.rel_err(pd.grad.cpu().numpy(), dp_ref)
    print("N=256 L=256 B=4096: rel err y %.2e, dJ/dp %.2e" % (e_y, e_dp))
    assert e_y < 1e-5 and e_dp < 1e-5

    # central differences on a 64-vector sub-batch, 64 random active MZIs
    Bs = 64
    xs, ts = x[:Bs], t[:Bs]
    pd.grad = None
    ys = mesh_apply(m, torch.tensor(xs, dtype=torch.complex64, device="cuda"), pd)
    ((ys - torch.tensor(ts, dtype=torch.complex64, device="cuda")).abs() ** 2).sum().backward()
    g_gpu = pd.grad.cpu().numpy()
    acts = O.propagate_activations(om, xs)
    act = np.argwhere(om.active_mask())
    pick = act[rng.choice(len(act), 64, replace=False)]
    h = 1e-6
    worst = 0.0
    for (l, q) in pick:
        for k in range(2):
            vals = []
            for sgn in (1, -1):
                pp = om.p.astype(np.float64).copy()
                pp[l, q, k] += sgn * h
                T = om.T_grid(pp)
                vals.append(_loss_from_layer(om, acts, l, T, ts))
            fd = (vals[0] - vals[1]) / (2 * h)
            worst = max(worst, abs(fd - g_gpu[l, q, k]) / max(abs(fd), 1e-3))
    print("central differences: worst relative deviation %.2e" % worst)
    assert worst < 1e-4


def test_unitary_fitting_training_loop():
    """Clements mzi N=128, L=128, splitting errors N(0, 0.02); target a Haar-random unitary; x = I;
    loss ||U - U_t||_F^2; 2000 Adam steps (lr 1e-2) on theta, phi through the autograd function; the
    final fidelity |tr(U^H U_t)|^2 / N^2 is re-evaluated in complex128 by the oracle."""
    from meshes_gb300.autograd import mesh_apply
    rng = np.random.default_rng(1004)
    N = 128
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    Ut = O.haar_unitary(rng, N).astype(np.complex64)
    m = gpu_mesh(om)
    x = torch.eye(N, dtype=torch.complex64, device="cuda")          # row b = e_b -> y[b] = U[:, b]
    target = torch.tensor(Ut.T, device="cuda")                       # rows of U_t^T
    p = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
    opt = torch.optim.Adam([p], lr=1e-2)
    first = None
    for it in range(2000):
        opt.zero_grad(set_to_none=True)
        y = mesh_apply(m, x, p)
        loss = ((y - target).abs() ** 2).sum()
        loss.backward()
        opt.step()
        if first is None:
            first = loss.item()
    with torch.no_grad():
        U = mesh_apply(m, x, p).t().cpu().numpy()
    fid_gpu = abs(np.trace(U.conj().T @ Ut)) ** 2 / N ** 2
    om.p = p.detach().cpu().numpy()
    U128 = O.matrix(om)
    fid_ref = abs(np.trace(U128.conj().T @ Ut.astype(np.complex128))) ** 2 / N ** 2
    loss_ref = float(np.sum(np.abs(U128 - Ut.astype(np.complex128)) ** 2))
    with torch.no_grad():
        loss_end = float(((mesh_apply(m, x, p) - target).abs() ** 2).sum())
    print("loss %.3f -> %.4f (complex128 %.4f), fidelity %.6f (complex128 %.6f)"
          % (first, loss_end, loss_ref, fid_gpu, fid_ref))
    assert loss_end < 0.5 * first                    # the optimisation makes progress
    assert abs(fid_gpu - fid_ref) < 1e-5             # the GPU's U is the complex128 U
    assert O.rel_err(U, U128) < 1e-5
    assert abs(loss_ref - loss_end) < 1e-4 * loss_ref


@pytest.mark.parametrize("geo,N,B,fused", [("clements", 32, 16, False), ("fft", 64, 24, False), ("clements", 64, 32, True)])
def test_graphed_training_step_matches_eager(geo, N, B, fused):
    """A training step captured in a CUDA graph (GraphedStep) and replayed follows the eager steps
    exactly: same losses, bitwise the same phases after 3 warm-up and 12 replayed steps.  fused: the
    step uses mesh_l2_loss and the library's fused Adam (as the unitary-fitting benchmark does)."""
    from meshes_gb300.autograd import Adam, GraphedStep, mesh_apply, mesh_l2_loss
    rng = np.random.default_rng(2024 + N)
    om = O.random_mesh(rng, N, geo, "mzi", 0.02)
    m = gpu_mesh(om)
    x = torch.tensor(O.unit_columns(rng, N, B), dtype=torch.complex64, device="cuda")
    target = torch.tensor(O.unit_columns(rng, N, B), dtype=torch.complex64, device="cuda")

    def trainer():
        p = torch.tensor(om.p, dtype=torch.float32, device="cuda", requires_grad=True)
        opt = Adam([p], lr=1e-2) if fused else torch.optim.Adam([p], lr=1e-2, capturable=True)

        def step():
            opt.zero_grad(set_to_none=True)
            if fused:
                loss = mesh_l2_loss(m, x, target, p)
            else:
                loss = ((mesh_apply(m, x, p) - target).abs() ** 2).sum()
            loss.backward()
            opt.step()
            return loss
        return p, step

    p_e, step_e = trainer()
    eager = [float(step_e().detach()) for _ in range(15)]
    p_g, step_g = trainer()
    g = GraphedStep(step_g, warmup=3)
    graphed = [float(g().detach()) for _ in range(12)]
    assert graphed == eager[3:]
    assert torch.equal(p_g.detach(), p_e.detach())
    assert eager[-1] < eager[0]
    assert m.status() == 0
