"""MeshOptimizer (reference gpu/opt.py): scipy fitting of a mesh to a target with GPU gradients."""
import numpy as np
import pytest

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu


def _mesh(om):
    from meshes_gb300 import MeshNetworkGPU
    return MeshNetworkGPU(om.N, om.L, om.lens, om.shifts, np.asarray(om.p, np.float32).reshape(-1),
                          np.asarray(om.s, np.float32), "mzi", is_phase=False)


def test_gradient_matches_central_differences_and_oracle():
    from meshes_gb300.opt import MeshOptimizer
    rng = np.random.default_rng(21)
    om = O.random_mesh(rng, 8, "clements", "mzi", 0.02)
    target = O.matrix(O.random_mesh(np.random.default_rng(22), 8, "clements", "mzi", 0.02))
    opt = MeshOptimizer(_mesh(om), target)
    p = opt.p.copy()
    assert p.size == 28 * 2                                   # active slots only, reference order
    g = opt.jac(p)
    # oracle: J = ||M U_t^H - I||^2 without the diagonal (reference gpu/mesh.py:176-181)
    def J_ref(pp):
        grid = np.zeros((om.L, 4, 2))
        grid[om.active_mask()] = pp.reshape(-1, 2)
        V = O.matrix(om, grid) @ target.conj().T - np.eye(8)
        V[np.diag_indices(8)] = 0
        return float(np.sum(np.abs(V) ** 2))
    assert abs(opt.f(p) - J_ref(p)) < 1e-5 * J_ref(p)
    fd = np.array([(J_ref(p + h) - J_ref(p - h)) / 2e-6 for h in np.eye(p.size) * 1e-6])
    assert O.rel_err(g, fd) < 1e-5


def test_fit_reaches_a_reachable_target():
    """Target = the same Clements mesh at other phases; start 0.3 rad away from them."""
    from meshes_gb300.opt import MeshOptimizer
    rng = np.random.default_rng(23)
    ot = O.random_mesh(rng, 16, "clements", "mzi", 0.02)
    target = O.matrix(ot)
    om = O.OracleMesh(N=16, L=ot.L, crossing="mzi", lens=ot.lens, shifts=ot.shifts, s=ot.s,
                      p=np.where(ot.active_mask()[..., None], ot.p + rng.normal(0, 0.3, ot.p.shape), 0.0))
    opt = MeshOptimizer(_mesh(om), target)
    J0 = opt.f(opt.p)
    res = opt.run("L-BFGS-B", tol=1e-14, maxiter=3000)
    assert res.fun < 1e-5 * J0
    assert len(res.yt) == len(res.t) > 0 and res.yt[-1] < res.yt[0]
