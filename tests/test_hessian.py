"""Finite-difference Hessians of MeshNetworkGPU (reference gpu/mesh.py:236-288): hvp, hvp_target, hess and
hess_target against the same central differences taken of the oracle's complex128 gradient.

The reference (and this API) forms H v = (g(p + eps v) - g(p - eps v)) / (2 eps) from two GPU gradients in
float32, so its error is the float32 gradient error amplified by 1/(2 eps); the oracle takes the same
differences with the same eps of its exact complex128 gradient, so the truncation error is common to both
and the comparison bound is set by that amplification (eps = 1e-2: about 1e-6 / 2e-2 of |g|, tested at 2e-3
of |H v|).  The reference's hess() passes its arguments on to hvp_target in the wrong order
(gpu/mesh.py:275); here hess() differentiates the given objective w."""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu
EPS = 1e-2
TOL = 2e-3


def _mesh(seed, N):
    from meshes_gb300 import MeshNetworkGPU
    rng = np.random.default_rng(seed)
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    m = MeshNetworkGPU(N, om.L, om.lens, om.shifts, om.p.reshape(-1), om.s, "mzi", is_phase=False, device="cuda")
    return rng, om, m


def _oracle_grad_target(om, Ut):
    """dJ/dp of J = ||offdiag(U U_t^H - I)||^2 (the reference's L2norm with is_phase False, gpu/mesh.py:176-181):
    the input vectors are the columns of U_t^H."""
    N = om.N
    x = Ut.conj().T.T                       # rows = columns of U_t^H

    def g_of_y(y):
        V = y.T - np.eye(N)
        V[np.diag_indices(N)] = 0
        return (2 * V).T

    return lambda p: O.grad(om, x, g_of_y, p)[1]


def _oracle_grad_fields(om, x, t):
    return lambda p: O.grad(om, x, lambda y: 2 * (y - t), p)[1]


def _fd(grad, p, vec, eps=EPS):
    return (grad(p + eps * vec) - grad(p - eps * vec)) / (2 * eps)


def _direction(rng, om):
    vec = rng.standard_normal(om.p.shape) * om.active_mask()[..., None]
    return vec.astype(np.float32).astype(np.float64)


@pytest.mark.parametrize("N", [8, 16])
def test_hvp_target(N):
    rng, om, m = _mesh(41 + N, N)
    Ut = O.haar_unitary(rng, N)
    vec = _direction(rng, om)
    h = m.hvp_target(torch.tensor(vec.reshape(-1), dtype=torch.float32, device="cuda"), Ut.astype(np.complex64),
                     eps=EPS).cpu().numpy().reshape(om.p.shape)
    ref = _fd(_oracle_grad_target(om, Ut.astype(np.complex64).astype(np.complex128)), om.p.astype(np.float64), vec)
    assert O.rel_err(h, ref) < TOL
    assert m.status() == 0


def test_hvp_fields():
    """hvp with a caller-given objective gradient w(v_out) = 2 (v_out - t) (J = sum |y - t|^2)."""
    rng, om, m = _mesh(43, 8)
    x = O.unit_columns(rng, 8, 5)
    t = O.unit_columns(rng, 8, 5)
    vec = _direction(rng, om)
    tt = torch.tensor(t.T.astype(np.complex64), device="cuda")
    h = m.hvp(torch.tensor(vec.reshape(-1), dtype=torch.float32, device="cuda"),
              torch.tensor(x.T.astype(np.complex64), device="cuda"), lambda y: 2 * (y - tt), eps=EPS)
    ref = _fd(_oracle_grad_fields(om, x.astype(np.complex64).astype(np.complex128),
                                  t.astype(np.complex64).astype(np.complex128)), om.p.astype(np.float64), vec)
    assert O.rel_err(h.cpu().numpy().reshape(om.p.shape), ref) < TOL


def test_hess_target_and_hess():
    """The full Hessians (one hvp per unit vector of the phase parameters) of a 4-mode mesh: symmetric, equal
    to the oracle's, and hess() of the same objective written as w equals hess_target()."""
    rng, om, m = _mesh(47, 4)
    Ut = O.haar_unitary(rng, 4).astype(np.complex64)
    Hd = m.hess_target(Ut, eps=EPS).cpu().numpy()
    n = om.p.size
    assert Hd.shape == (n, n)
    grad = _oracle_grad_target(om, Ut.astype(np.complex128))
    p0 = om.p.astype(np.float64)
    ref = np.stack([_fd(grad, p0, e.reshape(om.p.shape)).reshape(-1) for e in np.eye(n)])
    assert O.rel_err(Hd, ref) < TOL
    assert O.rel_err(Hd, Hd.T) < TOL
    N = 4

    def w(U):
        V = U - torch.eye(N, dtype=U.dtype, device=U.device)
        return 2 * (V - torch.diag(torch.diagonal(V)))

    v = torch.tensor(Ut.conj().T, device="cuda")
    H2 = m.hess(v, w, eps=EPS).cpu().numpy()
    assert O.rel_err(H2, Hd) < 1e-6
