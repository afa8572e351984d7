"""The bounded-wait failure path of the propagation kernels, made to run out on purpose without any fault.

Every wait of the kernels' shared-memory pipeline has a time limit; on expiry a CTA records MG_ST_TIMEOUT in
the workspace status word, waits (within the same limit) for the copies it issued, releases its barriers and
returns.  mg_propagate_wait_test leaves one pipeline chunk's coefficient copy unissued and sets a 1 ms limit,
so every CTA reaches a wait that nothing will complete: the call must return, the status must read
MG_ST_TIMEOUT, and the next normal call on the same (cleared) workspace must match the oracle."""
import time

import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-5
ST_TIMEOUT = 1


@pytest.mark.parametrize("op", [0, 2])
@pytest.mark.parametrize("which", ["first", "second"])
def test_expired_wait_records_timeout_and_recovers(op, which):
    from meshes_gb300 import _lib
    from meshes_gb300.batched import plan
    lib = _lib.load()
    rng = np.random.default_rng(71 + op)
    N, B = 64, 200
    om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
    L = om.L
    st = torch.cuda.current_stream().cuda_stream
    lens = torch.tensor(om.lens, dtype=torch.int32, device="cuda")
    shifts = torch.tensor(om.shifts, dtype=torch.int32, device="cuda")
    p = torch.tensor(om.p.reshape(-1), dtype=torch.float32, device="cuda")
    s = torch.tensor(om.s.reshape(-1), dtype=torch.float32, device="cuda")
    ldp = lds = N // 2 * 2
    wsb = lib.mg_workspace_bytes(op, N, L, B, 0, 0, None)
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    _lib.check(lib.mg_workspace_init(ws.data_ptr(), wsb, st), "mg_workspace_init")
    _lib.check(lib.mg_build_tiles(op, N, L, 0, lens.data_ptr(), shifts.data_ptr(), None, 0, p.data_ptr(), ldp,
                                  s.data_ptr(), lds, None, None, None, B, None, ws.data_ptr(), wsb, st), "mg_build_tiles")
    info = plan(op, N, L, B, 0, 0)
    nch = (L + info.CL - 1) // info.CL
    chunk = 0 if which == "first" else min(1, nch - 1)
    x = O.unit_columns(rng, N, B)
    y_ref = O.propagate(om, x)
    t = O.unit_columns(rng, N, B)
    g = 2 * (y_ref - t)
    if op == 0:
        a_in0 = torch.tensor(x.astype(np.complex64), device="cuda")
        a_in1 = None
    else:
        a_in0 = torch.tensor(y_ref.astype(np.complex64), device="cuda")
        a_in1 = torch.tensor(g.astype(np.complex64), device="cuda")
    out0 = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    out1 = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    ptr = lambda t_: None if t_ is None else t_.data_ptr()
    o0, o1 = (ptr(out0), None) if op == 0 else (None, ptr(out1))
    t0 = time.perf_counter()
    rc = lib.mg_propagate_wait_test(op, N, L, B, 0, ptr(a_in0), ptr(a_in1), o0, o1, N, 1000000, chunk,
                                    ws.data_ptr(), wsb, st)
    assert rc == 0, _lib.last_error()
    assert lib.mg_read_status(ws.data_ptr(), 1, st) == ST_TIMEOUT     # synchronises, then clears
    assert time.perf_counter() - t0 < 5.0
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
    # the same workspace, a normal call: complete and correct
    dp = torch.empty(L * N // 2 * 2, dtype=torch.float32, device="cuda")
    _lib.check(lib.mg_propagate(op, N, L, B, 0, 0, ptr(a_in0), ptr(a_in1), o0, o1, N,
                                dp.data_ptr() if op == 2 else None, ldp, 0, None, ws.data_ptr(), wsb, st),
               "mg_propagate")
    assert lib.mg_read_status(ws.data_ptr(), 0, st) == 0
    if op == 0:
        assert O.rel_err(out0.cpu().numpy(), y_ref) < TOL
    else:
        G, _, gin = O.vjp_unitary(om, y_ref, g)
        assert O.rel_err(out1.cpu().numpy(), gin) < TOL
        assert O.rel_err(dp.cpu().numpy().reshape(om.p.shape), O.contract_dp(om, G)) < TOL


@pytest.mark.gpu
def test_wait_test_rejects_bad_arguments():
    from meshes_gb300 import _lib
    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    N, L, B = 16, 16, 8
    wsb = lib.mg_workspace_bytes(0, N, L, B, 0, 0, None)
    ws = torch.zeros(wsb, dtype=torch.uint8, device="cuda")
    x = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    assert lib.mg_propagate_wait_test(0, N, L, B, 0, x.data_ptr(), None, x.data_ptr(), None, N, 0, 0, ws.data_ptr(),
                                      wsb, st) == -1
    assert lib.mg_propagate_wait_test(0, N, L, B, 0, x.data_ptr(), None, x.data_ptr(), None, N, 1000, 10 ** 6,
                                      ws.data_ptr(), wsb, st) == -1
    assert lib.mg_propagate_wait_test(1, N, L, B, 0, x.data_ptr(), None, x.data_ptr(), None, N, 1000, 0,
                                      ws.data_ptr(), wsb, st) == -1
