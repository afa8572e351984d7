"""The warp-pair back-propagation launch (mg_config.split = 3): each vector spread over the 64 lanes of two
warps (4 modes per lane) on the tiles of an M = 8, G = 32 plan.  Against the complex128 oracle (1e-5), and
against the one-warp launch on the same tiles: the fields it returns (reconstructed input, input gradient)
are bitwise the same, since every vector sees the same crossings in the same order; dJ/dp differs only in
the order of its batch sums."""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _run(om, y, g, cfg, target=None):
    from meshes_gb300 import _lib
    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    N, L, B = om.N, om.L, y.shape[0]
    lens = torch.tensor(om.lens, dtype=torch.int32, device="cuda")
    shifts = torch.tensor(om.shifts, dtype=torch.int32, device="cuda")
    p = torch.tensor(np.asarray(om.p, np.float32).reshape(-1), device="cuda")
    s = torch.tensor(np.asarray(om.s, np.float32).reshape(-1), device="cuda")
    ldp = N // 2 * 2
    c = _lib.cfg_ptr(cfg)
    wsb = lib.mg_workspace_bytes(2, N, L, B, 0, 0, c)
    assert wsb > 0, _lib.last_error()
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(lib.mg_workspace_init(ws.data_ptr(), wsb, st), "mg_workspace_init")
    _lib.check(lib.mg_build_tiles(2, N, L, 0, lens.data_ptr(), shifts.data_ptr(), None, 0, p.data_ptr(), ldp,
                                  s.data_ptr(), ldp, None, None, None, B, c, ws.data_ptr(), wsb, st), "mg_build_tiles")
    yd = torch.tensor(y.astype(np.complex64), device="cuda")
    xo = torch.zeros_like(yd)
    go = torch.zeros_like(yd)
    dp = torch.empty(L * N // 2 * 2, dtype=torch.float32, device="cuda")
    if target is None:
        gd = torch.tensor(g.astype(np.complex64), device="cuda")
        _lib.check(lib.mg_propagate(2, N, L, B, 0, 0, yd.data_ptr(), gd.data_ptr(), xo.data_ptr(), go.data_ptr(), N,
                                    dp.data_ptr(), ldp, 0, c, ws.data_ptr(), wsb, st), "mg_propagate")
    else:
        td = torch.tensor(target.astype(np.complex64), device="cuda")
        _lib.check(lib.mg_propagate_l2(N, L, B, 0, 0, yd.data_ptr(), td.data_ptr(), xo.data_ptr(), go.data_ptr(), N,
                                       dp.data_ptr(), ldp, 0, c, ws.data_ptr(), wsb, st), "mg_propagate_l2")
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
    return xo.cpu().numpy(), go.cpu().numpy(), dp.cpu().numpy().reshape(om.p.shape)


@pytest.mark.parametrize("geo,N,B,V", [("clements", 256, 1000, 7), ("clements", 256, 4096, 7), ("clements", 200, 333, 6),
                                       ("reck", 160, 257, 8), ("random", 256, 123, 7)])
def test_pair_launch_matches_oracle_and_one_warp_launch(geo, N, B, V):
    from meshes_gb300 import _lib
    rng = np.random.default_rng(N + B + V)
    if geo == "random":
        # random lens/shifts with odd and even shifts (nearest-neighbour layers of any extent)
        L = 40
        shifts = rng.integers(0, 2, L) + 2 * rng.integers(0, 20, L)
        lens = [int(rng.integers(0, (N - sh) // 2 + 1)) for sh in shifts]
        om = O.OracleMesh(N=N, L=L, crossing="mzi", lens=lens, shifts=shifts.tolist(),
                          p=rng.uniform(0, 2 * np.pi, (L, N // 2, 2)), s=rng.normal(0, 0.02, (L, N // 2, 2)))
        mask = om.active_mask()
        om.p[~mask] = 0
        om.s[~mask] = 0
    else:
        om = O.random_mesh(rng, N, geo, "mzi", 0.02)
    x = O.unit_columns(rng, N, B)
    t = O.unit_columns(rng, N, B)
    y = O.propagate(om, x)
    G, xr, gin = O.vjp_unitary(om, y, 2 * (y - t))
    dp_ref = O.contract_dp(om, G)
    pair = _lib.config(8, V, 8, 0, 0, 3)
    one = _lib.config(8, 4, 8, 0, 0, 2)
    xa, ga, da = _run(om, y, None, pair, target=t)
    assert O.rel_err(xa, x) < TOL
    assert O.rel_err(ga, gin) < TOL
    assert O.rel_err(da, dp_ref) < TOL
    xb, gb, db = _run(om, y, None, one, target=t)
    assert np.array_equal(xa, xb) and np.array_equal(ga, gb)
    assert O.rel_err(da, db) < 1e-6
    # explicit upstream gradient instead of the fused L2 target, formed in complex64 as the kernel forms it
    g32 = 2 * (y.astype(np.complex64) - t.astype(np.complex64))
    xc, gc, dc = _run(om, y, g32, pair)
    assert np.array_equal(gc, ga) and np.array_equal(dc, da)


def test_pair_launch_rejects_other_shapes():
    from meshes_gb300 import _lib
    lib = _lib.load()
    c = _lib.cfg_ptr(_lib.config(8, 7, 8, 0, 0, 3))
    assert lib.mg_workspace_bytes(0, 256, 256, 4096, 0, 0, c) == 0          # forward
    assert lib.mg_workspace_bytes(2, 256, 256, 4096, 2, 0, c) == 0          # orth
    assert lib.mg_workspace_bytes(2, 256, 8, 4096, 0, 1, c) == 0            # butterfly
    assert lib.mg_workspace_bytes(2, 64, 64, 4096, 0, 0, c) == 0            # G = 8 < 32
    assert lib.mg_workspace_bytes(2, 256, 256, 4096, 0, 0, _lib.cfg_ptr(_lib.config(8, 7, 7, 0, 0, 3))) == 0   # odd W
    assert lib.mg_workspace_bytes(2, 256, 256, 4096, 0, 0, c) > 0


@pytest.mark.parametrize("op", [0, 2])
def test_two_cta_per_sm_launch_matches_oracle(op):
    """Launch option split = 4: the nearest-neighbour kernels compiled for two resident CTAs per SM (M = 8, V = 2),
    shared memory sized for two; the same fields as the default launch, bitwise."""
    from meshes_gb300 import _lib
    rng = np.random.default_rng(91 + op)
    N, B = 256, 1000
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    x = O.unit_columns(rng, N, B)
    t = O.unit_columns(rng, N, B)
    y = O.propagate(om, x)
    occ2 = _lib.config(8, 2, 8, 0, 0, 4)
    if op == 2:
        G, xr, gin = O.vjp_unitary(om, y, 2 * (y - t))
        xa, ga, da = _run(om, y, None, occ2, target=t)
        assert O.rel_err(ga, gin) < TOL and O.rel_err(xa, x) < TOL
        assert O.rel_err(da, O.contract_dp(om, G)) < TOL
        xb, gb, db = _run(om, y, None, _lib.config(8, 2, 8, 0, 0, 2), target=t)
        assert np.array_equal(ga, gb) and np.array_equal(xa, xb)
        return
    from meshes_gb300 import _lib as L_
    lib = L_.load()
    st = torch.cuda.current_stream().cuda_stream
    lens = torch.tensor(om.lens, dtype=torch.int32, device="cuda")
    shifts = torch.tensor(om.shifts, dtype=torch.int32, device="cuda")
    p = torch.tensor(np.asarray(om.p, np.float32).reshape(-1), device="cuda")
    s = torch.tensor(np.asarray(om.s, np.float32).reshape(-1), device="cuda")
    outs = []
    for cfg in (occ2, _lib.config(8, 2, 8, 0, 0, 2)):
        c = _lib.cfg_ptr(cfg)
        wsb = lib.mg_workspace_bytes(0, N, om.L, B, 0, 0, c)
        ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
        _lib.check(lib.mg_workspace_init(ws.data_ptr(), wsb, st), "init")
        _lib.check(lib.mg_build_tiles(0, N, om.L, 0, lens.data_ptr(), shifts.data_ptr(), None, 0, p.data_ptr(), N,
                                      s.data_ptr(), N, None, None, None, B, c, ws.data_ptr(), wsb, st), "tiles")
        xd = torch.tensor(x.astype(np.complex64), device="cuda")
        yd = torch.empty_like(xd)
        _lib.check(lib.mg_propagate(0, N, om.L, B, 0, 0, xd.data_ptr(), None, yd.data_ptr(), None, N, None, 0, 0, c,
                                    ws.data_ptr(), wsb, st), "fwd")
        assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
        outs.append(yd.cpu().numpy())
    assert O.rel_err(outs[0], y) < TOL and np.array_equal(outs[0], outs[1])
