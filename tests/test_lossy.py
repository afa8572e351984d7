"""Lossy meshes: the checkpointed stored-activation adjoint against the complex128 oracle.

The oracle's lossy crossing is pinned to the reference (tests/golden/clements_mzigeneric_N8_lossy.npz)
and its stored-activation gradient to complex128 central differences (test_oracle.py); the reference's
own VJP raises NotImplementedError for this crossing.
"""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5          # relative error of the complex64 kernels against complex128


def lossy_oracle(rng, N, geometry, gain):
    om = O.random_mesh(rng, N, geometry, "mzi_generic", 0.02)
    s = np.zeros((om.L, N // 2, 14))
    s[..., :2] = rng.normal(0, 0.02, (om.L, N // 2, 2))
    s[..., 2:10] = rng.normal(0, 0.03, (om.L, N // 2, 8))
    s[..., 10:] = -np.abs(rng.normal(gain, gain / 2, (om.L, N // 2, 4)))
    s = s.astype(np.float32).astype(np.float64)
    s[~om.active_mask()] = 0
    om.s = s
    return om


def gpu_lossy(om, segment=None):
    from meshes_gb300.lossy import LossyMesh
    if om.fft:
        return LossyMesh(om.N, strides=om.strides, segment=segment)
    return LossyMesh(om.N, om.lens, om.shifts, segment=segment)


CASES = [
    ("clements", 8, 5, None),
    ("clements", 64, 33, None),
    ("clements", 64, 33, 1),          # a checkpoint before every layer
    ("clements", 64, 33, 7),          # ragged last segment
    ("clements", 64, 33, 1000),       # one segment: all activations stored
    ("reck", 10, 7, None),
    ("fft", 32, 40, None),
    ("butterfly", 16, 9, None),
    ("clements", 256, 300, None),
    ("clements", 512, 20, None),
]


@pytest.mark.parametrize("geometry,N,B,segment", CASES)
def test_lossy_forward_and_adjoint(geometry, N, B, segment):
    rng = np.random.default_rng(N * 131 + B)
    om = lossy_oracle(rng, N, geometry, gain=min(0.1, 2.0 / N))
    mesh = gpu_lossy(om, segment)
    dev = mesh.device
    p = torch.tensor(om.p, dtype=torch.float64, device=dev, requires_grad=True)
    s = torch.tensor(om.s, dtype=torch.float64, device=dev)
    T = mesh.T(p, s)
    T.retain_grad()
    mask = om.active_mask()
    # the library's double-precision T, rounded once to complex64
    assert np.abs(T.detach().cpu().numpy()[mask] - om.T_grid()[mask]).max() < 1.5e-7
    from meshes_gb300.lossy import mzi_generic_T
    T128 = mzi_generic_T(p.detach(), s)                     # the differentiable tensor formula
    assert np.abs(T128.cpu().numpy()[mask] - om.T_grid()[mask]).max() < 1e-12
    x_np = O.unit_columns(rng, N, B)
    t_np = O.unit_columns(rng, N, B)
    x = torch.tensor(x_np.astype(np.complex64), device=dev, requires_grad=True)
    t = torch.tensor(t_np.astype(np.complex64), device=dev)
    y = mesh(x, T)
    loss = torch.sum(torch.abs(y - t) ** 2)
    loss.backward()
    assert mesh.status() == 0
    # oracle: forward, stored-activation VJP, phase gradient
    x128 = x_np.astype(np.complex64).astype(np.complex128)
    y_ref = O.propagate(om, x128)
    assert O.rel_err(y.detach().cpu().numpy(), y_ref) < TOL
    G, gin = O.vjp_stored(om, x128, 2 * (y_ref - t_np.astype(np.complex64)))
    assert O.rel_err(x.grad.cpu().numpy(), gin) < TOL
    assert O.rel_err(T.grad.cpu().numpy()[mask], np.conj(G)[mask]) < TOL
    assert np.all(T.grad.cpu().numpy()[~mask] == 0)
    assert O.rel_err(p.grad.cpu().numpy(), O.contract_dp(om, G)) < TOL


def test_lossy_gradient_is_deterministic_and_segment_independent():
    rng = np.random.default_rng(7)
    om = lossy_oracle(rng, 64, "clements", 0.03)
    grads = []
    for seg in (None, None, 5, 64):
        mesh = gpu_lossy(om, seg)
        T = torch.tensor(om.T_grid(), dtype=torch.complex64, device=mesh.device, requires_grad=True)
        x = torch.tensor(O.unit_columns(np.random.default_rng(1), 64, 77).astype(np.complex64), device=mesh.device,
                         requires_grad=True)
        y = mesh(x, T)
        (torch.sum(y.real ** 3) + torch.sum(y.imag)).backward()
        grads.append((y.detach().cpu().numpy(), x.grad.cpu().numpy(), T.grad.cpu().numpy()))
    for a, b in zip(grads[0], grads[1]):
        assert np.array_equal(a, b)                         # run to run: bit-identical
    for g in grads[2:]:                                     # other checkpoint spacings: same numbers
        for a, b in zip(grads[0], g):
            assert O.rel_err(b, a) < 1e-6


def test_lossless_generic_matches_mzi_path():
    """With no phase errors and no gains the generic crossing is the MZI: the stored-activation adjoint
    and the T^H-reconstruction kernels of MeshNetworkGPU give the same gradients."""
    from meshes_gb300 import MeshNetworkGPU
    rng = np.random.default_rng(8)
    om = O.random_mesh(rng, 128, "clements", "mzi", 0.02)
    mesh = gpu_lossy(om)
    dev = mesh.device
    s14 = np.zeros((om.L, 64, 14))
    s14[..., :2] = om.s
    p = torch.tensor(om.p, dtype=torch.float64, device=dev, requires_grad=True)
    T = mesh.T(p, torch.tensor(s14, device=dev))
    x_np = O.unit_columns(rng, 128, 50).astype(np.complex64)
    g_np = O.unit_columns(rng, 128, 50).astype(np.complex64)
    x = torch.tensor(x_np, device=dev, requires_grad=True)
    y = mesh(x, T)
    y.backward(torch.tensor(g_np, device=dev))
    ref = MeshNetworkGPU(om.N, om.L, om.lens, om.shifts, om.p.reshape(-1), om.s, "mzi", is_phase=False)
    y2 = ref.dot(x_np.T)
    dp2, gin2 = ref.grad_phi(x_np.T, g_np.T)          # v = mesh input (vpos "in")
    assert O.rel_err(y.detach().cpu().numpy(), y2.t().cpu().numpy()) < TOL
    assert O.rel_err(x.grad.cpu().numpy(), gin2.t().cpu().numpy()) < TOL
    assert O.rel_err(p.grad.cpu().numpy().reshape(-1), dp2.reshape(-1).cpu().numpy()) < TOL


def test_range_argument_errors():
    from meshes_gb300._lib import GENERIC, GEO_NN, OP_BWD_STORED, OP_FWD, OP_BWD, load
    lib = load()
    N, L, B = 8, 8, 4
    nb = lib.mg_workspace_bytes(OP_BWD_STORED, N, L, B, GENERIC, GEO_NN, None)
    ws = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    f = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    # bad range, bad op, missing activations, stored back-prop through mg_propagate
    assert lib.mg_propagate_range(OP_FWD, N, L, 3, 9, B, GENERIC, GEO_NN, f.data_ptr(), None, f.data_ptr(), None, N,
                                  None, None, 0, None, ws.data_ptr(), nb, s) < 0
    assert lib.mg_propagate_range(OP_BWD, N, L, 0, 8, B, GENERIC, GEO_NN, None, f.data_ptr(), None, f.data_ptr(), N,
                                  None, None, 0, None, ws.data_ptr(), nb, s) < 0
    assert lib.mg_propagate_range(OP_BWD_STORED, N, L, 0, 8, B, GENERIC, GEO_NN, None, f.data_ptr(), None,
                                  f.data_ptr(), N, None, None, 0, None, ws.data_ptr(), nb, s) < 0
    assert lib.mg_propagate(OP_BWD_STORED, N, L, B, GENERIC, GEO_NN, None, f.data_ptr(), None, f.data_ptr(), N, None,
                            0, 0, None, ws.data_ptr(), nb, s) < 0
    # orth has no stored-activation back-propagation
    assert lib.mg_workspace_bytes(OP_BWD_STORED, N, L, B, 2, GEO_NN, None) == 0
