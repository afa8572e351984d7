"""Coefficient tiles: every float32 entry of the MZI transfer matrices (and of the splitter pair of the direct
gradient) is the float32 nearest to the exact complex128 value, as unbiased rounding needs (a deep mesh
accumulates a systematic error linearly).  The tiles are read back from a workspace built by mg_build_tiles
and decoded with the layout mg_plan reports; phases span ordinary and large angles of both signs."""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu


def _build(om, op, B, no_splitters=False):
    from meshes_gb300 import _lib
    from meshes_gb300.batched import plan
    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    N, L = om.N, om.L
    info = plan(op, N, L, B, 0, 0)
    ws = torch.zeros(info.total, dtype=torch.uint8, device="cuda")
    lens = torch.tensor(om.lens, dtype=torch.int32, device="cuda")
    shifts = torch.tensor(om.shifts, dtype=torch.int32, device="cuda")
    p = torch.tensor(np.asarray(om.p, np.float32).reshape(-1), device="cuda")
    s = torch.tensor(np.asarray(om.s, np.float32).reshape(-1), device="cuda")
    assert no_splitters or s.numel() == L * (N // 2) * 2          # the kernel reads a full (L, N/2, 2) grid
    _lib.check(lib.mg_build_tiles(op, N, L, 0, lens.data_ptr(), shifts.data_ptr(), None, 0, p.data_ptr(), N,
                                  None if no_splitters else s.data_ptr(), N, None, None, None, B, None,
                                  ws.data_ptr(), info.total, st), "mg_build_tiles")
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
    raw = ws.cpu().numpy()
    tiles = raw[info.off_tiles: info.off_tiles + L * info.layer_bytes].view(np.float32).reshape(L, -1)
    return info, tiles


def _decode(info, tiles, N):
    """T[l, q] (complex64) and, where present, cs[l, q] (float32 pairs) of the nearest-neighbour layers."""
    M, G = info.M, info.G
    L = tiles.shape[0]
    f4 = tiles[:, : 4 * 2 * (M // 2) * G].reshape(L, M, G, 4)     # rows [2e + h][j]
    T = np.zeros((L, N // 2, 2, 2), np.complex64)
    cs = np.zeros((L, N // 2, 2), np.float32)
    for q in range(N // 2):
        j, e = q // (M // 2), q % (M // 2)
        r0, r1 = f4[:, 2 * e, j], f4[:, 2 * e + 1, j]
        T[:, q, 0, 0] = r0[:, 0] + 1j * r0[:, 1]
        T[:, q, 0, 1] = r0[:, 2] + 1j * r0[:, 3]
        T[:, q, 1, 0] = r1[:, 0] + 1j * r1[:, 1]
        T[:, q, 1, 1] = r1[:, 2] + 1j * r1[:, 3]
        if info.layer_bytes >= (M * G * 16 + (M // 2) * G * 8):
            c2 = tiles[:, 4 * M * G:].reshape(L, -1, 2)
            cs[:, q] = c2[:, e * G + j]
    return T, cs


def _nearest(T):
    return (T.real.astype(np.float32) + 1j * T.imag.astype(np.float32)).astype(np.complex64)


@pytest.mark.parametrize("op", [0, 2])
def test_tiles_are_correctly_rounded(op):
    rng = np.random.default_rng(17 + op)
    N = 256
    om = O.random_mesh(rng, N, "clements", "mzi", 0.05)
    # phases of ordinary size, large and negative ones (trained phases drift), splitter errors to 0.2 rad
    p = om.p.astype(np.float64)
    big = rng.random(p.shape) < 0.2
    p[big] = rng.uniform(-300, 300, big.sum())
    huge = rng.random(p.shape) < 0.01              # beyond the float-float range: the double-precision path
    p[huge] = rng.uniform(-3000, 3000, huge.sum())
    om.p = (p * om.active_mask()[..., None]).astype(np.float32)
    om.s = (rng.normal(0, 0.08, om.s.shape) * om.active_mask()[..., None]).astype(np.float32)
    info, tiles = _build(om, op, 4096)
    T, cs = _decode(info, tiles, N)
    ref = _nearest(om.T_grid())
    mask = om.active_mask()
    got, want = T[mask], ref[mask]
    mism = got != want
    assert mism.mean() < 1e-4, mism.sum()
    # where they differ, by one unit in the last place at most (a value within 1e-13 of a rounding boundary)
    if mism.any():
        d = np.abs(got[mism] - want[mism])
        assert np.all(d <= 2 * np.spacing(np.abs(want[mism]).astype(np.float32)) + 1e-30)
    # inactive slots are the identity
    assert np.array_equal(T[~mask], np.broadcast_to(np.eye(2, dtype=np.complex64), T[~mask].shape))
    if op == 2:
        beta = om.s[..., 1].astype(np.float64)
        cs_ref = np.stack([np.cos(np.pi / 4 + beta), np.sin(np.pi / 4 + beta)], -1).astype(np.float32)
        assert (cs[mask] != cs_ref[mask]).mean() < 1e-4


@pytest.mark.parametrize("op", [0, 2])
def test_ideal_splitter_tiles(op):
    """Without a splitter array the coefficient pass takes its ideal-splitter form (no splitter products); its
    tiles equal those built from an explicit all-zero splitter array (the general form) entry for entry, and
    are correctly rounded."""
    rng = np.random.default_rng(23 + op)
    om = O.random_mesh(rng, 128, "clements", "mzi", 0.0)
    p = om.p.astype(np.float64)
    big = rng.random(p.shape) < 0.2
    p[big] = rng.uniform(-300, 300, big.sum())
    om.p = (p * om.active_mask()[..., None]).astype(np.float32)
    om.s = np.zeros((om.L, om.N // 2, 2), dtype=np.float32)          # an explicit all-zero splitter grid
    info, t_ideal = _build(om, op, 1024, no_splitters=True)
    _, t_zero = _build(om, op, 1024)
    assert np.array_equal(t_ideal, t_zero)          # +0 and -0 compare equal
    T, _ = _decode(info, t_ideal, 128)
    mask = om.active_mask()
    assert (T[mask] != _nearest(om.T_grid())[mask]).mean() < 1e-4
