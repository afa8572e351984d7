"""The converter from a reference network (StructuredMeshNetwork.gpu(), reference mesh.py:568-579) on objects
rebuilt from fixtures that the reference itself produced (tests/golden/converter_*.npz, written by
make_golden.py from ClementsNetwork, ReckNetwork, ButterflyNetwork, a permuted StructuredMeshNetwork, an
MZICrossingOutPhase mesh and a SquareNetwork): every attribute the converter reads is stored, and the
converted GPU mesh must reproduce the reference's own dot and dot_vjp (ClippedNetwork.dot and grad_L2 for
the clipped mesh)."""
import os

import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-5
CASES = ["clements_mzi_N8_screen", "reck_mzi_N6_screen", "butterfly_mzi_N8", "perm_mzi_N8", "outphase_N6"]


def _named(name):
    """An instance of an empty class called `name` (the converter dispatches on class names)."""
    return type(str(name), (), {})()


def rebuild(z, prefix=""):
    """A stand-in for the reference network with the attributes StructuredMeshNetwork.gpu() reads."""
    net = _named(z[prefix + "net_class"])
    net.N, net.L = int(z[prefix + "N"]), int(z[prefix + "L"])
    net.lens, net.shifts = z[prefix + "lens"].tolist(), z[prefix + "shifts"].tolist()
    net.grid_phase, net.grid_splitter = z[prefix + "grid_phase"], z[prefix + "grid_splitter"]
    net.X = _named(z[prefix + "X"])
    net.perm = [None if none else row for row, none in zip(z[prefix + "perm_rows"], z[prefix + "perm_none"])]
    net.is_phase = bool(z[prefix + "is_phase"])
    net.phi_out = z[prefix + "phi_out"]
    net.phi_pos = str(z[prefix + "phi_pos"])
    return net


def load(name):
    return np.load(os.path.join(GOLDEN, "converter_%s.npz" % name))


def test_converter_fixtures_rebuild():
    """CPU: every fixture rebuilds into a stand-in whose grids hold the reference's parameters (the NaN slots
    the reference leaves outside each layer's MZIs included)."""
    for name in CASES:
        z = load(name)
        net = rebuild(z)
        n_cr = int(np.sum(net.lens))
        flat = O.grid_to_flat(np.nan_to_num(net.grid_phase), net.lens, net.shifts)
        assert flat.shape[0] == n_cr
        assert np.array_equal(flat.reshape(-1), z["p_phase"][:flat.size])
        assert len(net.perm) == net.L + 1
    z = load("squarenet_N3")
    full = rebuild(z, "full_")
    assert full.is_phase and len(z["idx_in"]) == 3 and len(z["idx_out"]) == 3


def _to_gpu_dp(z, dJdp):
    """The reference's flat dJ/dp (crossings in layer order, then the phase screen) in the GPU layout (the
    reference GPU grid (L, N/2, n_p), then the screen)."""
    N, lens, shifts = int(z["N"]), z["lens"].tolist(), z["shifts"].tolist()
    n_cr = int(np.sum(lens))
    grid = O.flat_to_grid(dJdp[:2 * n_cr].reshape(n_cr, 2), lens, shifts, N, 2)
    return np.concatenate([grid.reshape(-1), dJdp[2 * n_cr:]])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_from_structured_matches_reference(name):
    from meshes_gb300 import from_structured
    z = load(name)
    m = from_structured(rebuild(z), device="cuda")
    x = torch.tensor(z["x"].astype(np.complex64), device="cuda")
    y = m.dot(x)
    assert O.rel_err(y.cpu().numpy(), z["y"]) < TOL
    g = torch.tensor(z["g"].astype(np.complex64), device="cuda")
    if name == "outphase_N6":
        # generic crossings back-propagate from the input fields; only dJ/dv is compared: the reference's
        # MZICrossingOutPhase.dT reverses the wrong axis (crossing.py:338-340), so its dJ/dp is not the
        # gradient of its own dot (pinned separately against central differences in test_crossings.py)
        dp, gin = m.grad_phi(x, g)
        assert O.rel_err(gin.cpu().numpy(), z["g_in"]) < TOL
        return
    dp, gin = m.grad_phi(torch.tensor(z["y"].astype(np.complex64), device="cuda"), g, vpos="out")
    assert O.rel_err(gin.cpu().numpy(), z["g_in"]) < TOL
    assert O.rel_err(dp.cpu().numpy().reshape(-1), _to_gpu_dp(z, z["dJdp"])) < TOL
    assert m.status() == 0


@pytest.mark.gpu
def test_from_structured_clipped_matches_reference():
    from meshes_gb300 import from_structured
    z = load("squarenet_N3")
    net = _named("SquareNetwork")
    net.full, net.idx_in, net.idx_out = rebuild(z, "full_"), z["idx_in"], z["idx_out"]
    m = from_structured(net, device="cuda")
    y = m.dot(torch.tensor(z["x"].astype(np.complex64), device="cuda")).cpu().numpy()
    assert O.rel_err(y, z["y"]) < TOL
    J, dp = m.grad_L2(z["U_target"])
    assert abs(J - float(z["J"])) < TOL * float(z["J"])
    zf = {k[len("full_"):]: z[k] for k in z.files if k.startswith("full_")}
    assert O.rel_err(dp.cpu().numpy().reshape(-1), _to_gpu_dp(zf, z["dJdp"])) < TOL
