"""Batched meshes (one persistent launch over a (mesh, batch-tile) work queue) against the oracle."""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5


def gpu_mesh(om):
    from meshes_gb300 import MeshNetworkGPU
    p = np.asarray(om.p, np.float32).reshape(-1)
    s = None if om.s is None else np.asarray(om.s, np.float32)
    if om.fft:
        return MeshNetworkGPU(om.N, om.L, None, None, p, s, om.crossing, is_phase=False, strides=om.strides)
    return MeshNetworkGPU(om.N, om.L, om.lens, om.shifts, p, s, om.crossing, is_phase=False)


def _mix(rng):
    specs = [("clements", "mzi", 8, 700), ("reck", "mzi", 16, 5), ("clements", "orth", 32, 130),
             ("clements", "mzi", 64, 33), ("reck", "mzi", 64, 1), ("clements", "orth", 8, 1500),
             ("clements", "mzi", 256, 70), ("clements", "mzi", 512, 9), ("fft", "mzi", 128, 40),
             ("clements", "orth", 256, 17), ("reck", "orth", 16, 64), ("clements", "mzi", 10, 3)]
    oms, xs = [], []
    for geo, cr, N, B in specs:
        om = O.random_mesh(rng, N, geo, cr, 0.01 if cr == "mzi" else 0.0)
        oms.append(om)
        xs.append(O.unit_columns(rng, N, B, real=cr == "orth"))
    return oms, xs


def test_batched_forward_backward_and_graph():
    from meshes_gb300.batched import BatchedMeshes
    rng = np.random.default_rng(31)
    oms, xs = _mix(rng)
    meshes = [gpu_mesh(om) for om in oms]
    bm = BatchedMeshes(meshes, [x.shape[0] for x in xs])
    gys = []
    for st, x, om in zip(bm.states, xs, oms):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
        g = O.unit_columns(rng, om.N, x.shape[0], real=om.crossing == "orth")
        gys.append(g)
    bm.forward()
    for st, g in zip(bm.states, gys):
        st.gy.copy_(torch.tensor(g, dtype=st.gy.dtype))
    bm.backward()
    assert bm.check_status() == 0
    for om, st, x, g in zip(oms, bm.states, xs, gys):
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(st.y.cpu().numpy(), y_ref) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.gx.cpu().numpy(), gin) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.dp.cpu().numpy(), O.contract_dp(om, G)) < TOL, (om.N, om.crossing)
    # CUDA graph: capture one step, replay with new inputs, compare with the oracle again
    bm.capture(backward=True)
    xs2 = [O.unit_columns(rng, om.N, x.shape[0], real=om.crossing == "orth") for om, x in zip(oms, xs)]
    for st, x in zip(bm.states, xs2):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
    for rep in range(2):
        bm.replay()
    torch.cuda.synchronize()
    for om, st, x in zip(oms, bm.states, xs2):
        assert O.rel_err(st.y.cpu().numpy(), O.propagate(om, x)) < TOL


def test_batched_equals_plain_path_bitwise():
    """The persistent kernel runs the same per-tile body: identical results to the one-mesh kernel when
    both use the same tile configuration."""
    from meshes_gb300.batched import BatchedMeshes
    from meshes_gb300 import _lib
    rng = np.random.default_rng(32)
    om = O.random_mesh(rng, 128, "clements", "mzi", 0.01)
    x = O.unit_columns(rng, 128, 300)
    m = gpu_mesh(om)
    bm = BatchedMeshes([m], [300])
    bm.states[0].x.copy_(torch.tensor(x, dtype=torch.complex64))
    bm.forward()
    m.config[0] = _lib.config(8, 4, 8, bm.states[0].info[0].CL, bm.states[0].info[0].S)
    from meshes_gb300.autograd import mesh_apply
    y_plain = mesh_apply(m, torch.tensor(x, dtype=torch.complex64, device="cuda"))
    assert torch.equal(y_plain, bm.states[0].y)


def test_many_items_per_cta():
    """A small persistent grid makes every CTA run many work items in turn (its pipeline barriers are
    released and initialised again per item); forward and back-propagation against the oracle."""
    from meshes_gb300.batched import BatchedMeshes
    rng = np.random.default_rng(33)
    specs = [("clements", "mzi", 64, 700), ("clements", "orth", 256, 90), ("reck", "mzi", 32, 300),
             ("clements", "mzi", 256, 100), ("fft", "mzi", 128, 64)]
    oms = [O.random_mesh(rng, N, geo, cr, 0.01 if cr == "mzi" else 0.0) for geo, cr, N, _ in specs]
    xs = [O.unit_columns(rng, om.N, B, real=om.crossing == "orth") for om, (*_, B) in zip(oms, specs)]
    gs = [O.unit_columns(rng, om.N, B, real=om.crossing == "orth") for om, (*_, B) in zip(oms, specs)]
    bm = BatchedMeshes([gpu_mesh(om) for om in oms], [x.shape[0] for x in xs], grid=3)
    assert bm.n_items > 3 * 4
    for st, x, g in zip(bm.states, xs, gs):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
    bm.forward()
    for st, g in zip(bm.states, gs):
        st.gy.copy_(torch.tensor(g, dtype=st.gy.dtype))
    bm.backward()
    assert bm.check_status() == 0
    for om, st, x, g in zip(oms, bm.states, xs, gs):
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(st.y.cpu().numpy(), y_ref) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.gx.cpu().numpy(), gin) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.dp.cpu().numpy(), O.contract_dp(om, G)) < TOL, (om.N, om.crossing)


def test_nearest_neighbour_launch():
    """A batch of nearest-neighbour meshes only (Clements, Reck; mzi and orth) runs the nearest-neighbour
    bodies (MG_BATCH_NN) with the same results as the oracle; forcing that launch on a batch holding a
    butterfly mesh refuses the butterfly's items with a status and leaves the other results intact."""
    from meshes_gb300 import _lib
    from meshes_gb300.batched import BatchedMeshes, _bind
    rng = np.random.default_rng(34)
    specs = [("clements", "mzi", 256, 300), ("reck", "mzi", 64, 90), ("clements", "orth", 128, 50),
             ("clements", "mzi", 512, 7), ("reck", "orth", 16, 33)]
    oms = [O.random_mesh(rng, N, geo, cr, 0.01 if cr == "mzi" else 0.0) for geo, cr, N, _ in specs]
    xs = [O.unit_columns(rng, om.N, B, real=om.crossing == "orth") for om, (*_, B) in zip(oms, specs)]
    gs = [O.unit_columns(rng, om.N, B, real=om.crossing == "orth") for om, (*_, B) in zip(oms, specs)]
    bm = BatchedMeshes([gpu_mesh(om) for om in oms], [x.shape[0] for x in xs])
    for st, x in zip(bm.states, xs):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
    bm.forward()
    for st, g in zip(bm.states, gs):
        st.gy.copy_(torch.tensor(g, dtype=st.gy.dtype))
    bm.backward()
    assert bm.check_status() == 0
    for om, st, x, g in zip(oms, bm.states, xs, gs):
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(st.y.cpu().numpy(), y_ref) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.gx.cpu().numpy(), gin) < TOL, (om.N, om.crossing)
        assert O.rel_err(st.dp.cpu().numpy(), O.contract_dp(om, G)) < TOL, (om.N, om.crossing)

    oms2 = [O.random_mesh(rng, 64, "clements", "mzi", 0.01), O.random_mesh(rng, 64, "fft", "mzi", 0.01)]
    xs2 = [O.unit_columns(rng, 64, 40) for _ in oms2]
    bm2 = BatchedMeshes([gpu_mesh(om) for om in oms2], [40, 40])
    for st, x in zip(bm2.states, xs2):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
    lib = _bind()
    bm2.head.zero_()
    assert len(bm2.groups) == 1
    _, n2, items2 = bm2.groups[0]
    _lib.check(lib.mg_batched_propagate(_lib.OP_FWD | _lib.BATCH_NN, bm2.desc[0].data_ptr(), 2, items2.data_ptr(),
                                        n2, bm2.head.data_ptr(), bm2.grid, bm2.smem[0], bm2.status.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream), "mg_batched_propagate")
    assert bm2.check_status() == 2
    assert O.rel_err(bm2.states[0].y.cpu().numpy(), O.propagate(oms2[0], xs2[0])) < TOL


def test_full_warp_class_launch():
    """By default (full_warp) meshes whose vectors fill the warp (complex M = 8, N in (128, 256]) run in their own
    launch with a compile-time lane group (full_warp=False: one launch); a launch of that class refuses an item
    of another mesh (MG_ST_BAD_WORK) and leaves it."""
    from meshes_gb300 import _lib
    from meshes_gb300.batched import MG_BATCH_FULL_WARP, MG_BATCH_ONLY, BCLS_C8, BatchedMeshes, _bind
    rng = np.random.default_rng(57)
    oms = [O.random_mesh(rng, 256, "clements", "mzi", 0.01), O.random_mesh(rng, 200, "reck", "mzi", 0.01),
           O.random_mesh(rng, 64, "clements", "mzi", 0.01)]
    Bs = [70, 45, 33]
    xs = [O.unit_columns(rng, om.N, B) for om, B in zip(oms, Bs)]
    gs = [O.unit_columns(rng, om.N, B) for om, B in zip(oms, Bs)]
    assert len(BatchedMeshes([gpu_mesh(om) for om in oms], Bs, full_warp=False).groups) == 1
    bm = BatchedMeshes([gpu_mesh(om) for om in oms], Bs)
    assert [g[0] for g in bm.groups] == [MG_BATCH_ONLY(BCLS_C8) | MG_BATCH_FULL_WARP, 0]
    for st, x, g in zip(bm.states, xs, gs):
        st.x.copy_(torch.tensor(x, dtype=st.x.dtype))
        st.gy.copy_(torch.tensor(g, dtype=st.gy.dtype))
    bm.step(True)
    assert bm.check_status() == 0
    for om, st, x, g in zip(oms, bm.states, xs, gs):
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(st.y.cpu().numpy(), y_ref) < TOL
        assert O.rel_err(st.gx.cpu().numpy(), gin) < TOL
        assert O.rel_err(st.dp.cpu().numpy(), O.contract_dp(om, G)) < TOL
    # both launch groups recorded in one CUDA graph (the side stream forked and joined inside the capture),
    # replayed with new inputs: the same results as eager steps
    bm.capture(backward=True)
    xs2 = [O.unit_columns(rng, om.N, B) for om, B in zip(oms, Bs)]
    for st, x in zip(bm.states, xs2):
        st.x.copy_(torch.tensor(x, dtype=torch.complex64))
    bm.replay()
    assert bm.check_status() == 0
    for om, st, x, g in zip(oms, bm.states, xs2, gs):
        y_ref = O.propagate(om, x)
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(st.y.cpu().numpy(), y_ref) < TOL
        assert O.rel_err(st.dp.cpu().numpy(), O.contract_dp(om, G)) < TOL
    # the N = 64 mesh's items through the full-warp launch: refused, output untouched
    lib = _bind()
    _, n_rest, items_rest = bm.groups[1]
    bm.states[2].y.zero_()
    bm.head.zero_()
    _lib.check(lib.mg_batched_propagate(_lib.OP_FWD | _lib.BATCH_NN | MG_BATCH_ONLY(BCLS_C8) | MG_BATCH_FULL_WARP,
                                        bm.desc[0].data_ptr(), 3, items_rest.data_ptr(), n_rest, bm.head.data_ptr(),
                                        bm.grid, bm.smem[0], bm.status.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream), "mg_batched_propagate")
    assert bm.check_status() == 3
    assert float(bm.states[2].y.abs().max()) == 0.0
