"""The reference's other crossing parameterisations (crossing.py:292-611) on the GPU through
lossy.GenericMeshGPU (T per slot from crossings.transfer, generic precomputed-T kernels, checkpointed
adjoint): against the reference's own StructuredMeshNetwork.dot / dot_vjp fixtures and against the
complex128 oracle with central differences on larger random meshes, phase screens included.

Tolerances: fields and input gradients 1e-5 relative (complex64 kernels); parameter gradients 1e-5 against
the reference's dot_vjp, 2e-4 against central differences (h = 1e-6, their own error dominates).
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
NAMES = ["mzi_balanced", "mzi_outphase", "mzi3", "mzi3_outphase", "mzi_generic_outphase", "cartesian", "bell"]


def to_dev(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).astype(np.complex64))).cuda().t()


def _mesh(om, ph=None, pos="out"):
    from meshes_gb300.lossy import GenericMeshGPU
    p = np.asarray(om.p, np.float64).reshape(-1)
    if ph is not None:
        p = np.concatenate([p, ph])
    return GenericMeshGPU(om.N, om.L, om.lens, om.shifts, p, om.s, om.crossing, phi_pos=pos, is_phase=ph is not None)


@pytest.mark.parametrize("name", NAMES)
def test_golden_generic_crossing_mesh(name):
    f = np.load(os.path.join(GOLDEN, "xmesh_%s_N6.npz" % name))
    om = O.OracleMesh(N=int(f["N"]), L=int(f["L"]), crossing=name, lens=list(f["lens"]), shifts=list(f["shifts"]),
                      p=f["p"], s=f["s"])
    m = _mesh(om)
    y = m.dot(to_dev(f["x"])).t().cpu().numpy()
    assert O.rel_err(y, f["y"]) < TOL
    if "dJdp" not in f:
        return
    dp, gin = m.grad_phi(to_dev(f["x"]), to_dev(f["g"]))
    dp = dp.cpu().numpy().reshape(om.L, om.N // 2, 2)
    act = om.active_mask()
    assert O.rel_err(gin.t().cpu().numpy(), f["g_in"]) < TOL
    if name == "mzi_outphase":
        # the reference's dot_vjp for this class contracts a slot-reversed dT (crossing.py:338-340); compare
        # with the derivative of its T instead
        idx = np.flatnonzero(np.broadcast_to(act[..., None], f["p"].shape))
        ref = O.central_difference(lambda pp: float(np.real(np.sum(np.conj(f["g"]) * O.propagate(om, f["x"], pp)))),
                                   f["p"], idx)
        assert O.rel_err(dp.reshape(-1)[idx], ref) < 2e-4
    else:
        assert O.rel_err(dp[act], f["dJdp"][act]) < TOL
    assert m.status() == 0


def _random_params(rng, name, shape_p, n_s, k_active):
    if name == "cartesian":
        rho, ang = 0.9 * np.sqrt(rng.uniform(0, 1, shape_p[:-1])), rng.uniform(0, 2 * np.pi, shape_p[:-1])
        side = np.where(rng.uniform(0, 1, shape_p[:-1]) < 0.5, 2.0, -2.0)
        p = np.stack([side + rho * np.cos(ang), rho * np.sin(ang)], -1)
    else:
        p = rng.uniform(0, 2 * np.pi, shape_p)
    s = rng.normal(0, 0.05, shape_p[:-1] + (n_s,))
    if n_s == 14:
        s[..., 10:] = -np.abs(rng.normal(0.1, 0.05, shape_p[:-1] + (4,)))
    return p, s


@pytest.mark.parametrize("name", NAMES + ["mzi", "sym", "mzi_generic"])
@pytest.mark.parametrize("pos", [None, "out", "in"])
def test_random_generic_crossing_mesh(name, pos):
    rng = np.random.default_rng(zlib.crc32(("%s%s" % (name, pos)).encode()))
    N, B = 32, 9
    lens, shifts = O.clements_geometry(N)
    L = len(lens)
    n_p, n_s = O.CROSSINGS[name]
    p, s = _random_params(rng, name, (L, N // 2, n_p), n_s, None)
    om = O.OracleMesh(N=N, L=L, crossing=name, lens=lens, shifts=shifts, p=p, s=s)
    act = om.active_mask()
    ph = rng.uniform(0, 2 * np.pi, N) if pos else None
    m = _mesh(om, ph, pos or "out")
    x = O.unit_columns(rng, N, B)
    t = O.unit_columns(rng, N, B)

    def fwd(pp, phh):
        return O.propagate_screened(om, x, phh, pos, pp) if pos else O.propagate(om, x, pp)

    with np.errstate(invalid="ignore"):
        y_ref = fwd(p, ph)
    assert O.rel_err(m.dot(to_dev(x)).t().cpu().numpy(), y_ref) < TOL
    tt = to_dev(t)
    dp, gin = m.grad_phi(to_dev(x), lambda yy: 2 * (yy - tt))
    dp = dp.cpu().numpy()
    # central differences of J = sum |y - t|^2 on random active crossing parameters and screen phases
    flat = np.flatnonzero(np.broadcast_to(act[..., None], p.shape))
    idx = rng.choice(flat, 10, replace=False)

    def J(pp):
        with np.errstate(invalid="ignore"):
            return float(np.sum(np.abs(fwd(pp, ph) - t) ** 2))
    fd = O.central_difference(J, p, idx)
    assert O.rel_err(dp[: p.size][idx], fd) < 2e-4
    if pos:
        def Jph(phh):
            with np.errstate(invalid="ignore"):
                return float(np.sum(np.abs(fwd(p, phh) - t) ** 2))
        fdph = O.central_difference(Jph, ph, np.arange(0, N, 5))
        assert O.rel_err(dp[p.size:][np.arange(0, N, 5)], fdph) < 2e-4
    assert m.status() == 0
