"""The allocation-free forward entry point (mg_fwdprop_noalloc) against the workspace one (mg_fwdprop).

Callers that cannot allocate device memory (plugin hosts that own the device heap, loops that must not
touch an allocator) use mg_fwdprop_noalloc, which keeps its
scratch in a fixed array compiled into the library.  This file is collected last so that a failure
here leaves every other test already run; it also passes alone in a fresh process.
"""
import numpy as np
import pytest
import torch

from oracle import meshes_oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5   # relative Frobenius error, as in the other parity tests


def _run(lib, fn_noalloc, N, L, B, lens, shifts, p, s, x, use_noalloc):
    st = torch.cuda.current_stream().cuda_stream
    out = torch.empty_like(x)
    if use_noalloc:
        rc = lib.mg_fwdprop_noalloc(N, L, B, lens.data_ptr(), shifts.data_ptr(), p.data_ptr(), N, s.data_ptr(), N,
                                    x.data_ptr(), out.data_ptr(), N, 0, st)
    else:
        nb = lib.mg_workspace_bytes(0, N, L, B, 0, 0, None)
        ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
        assert lib.mg_workspace_init(ws.data_ptr(), nb, st) == 0
        rc = lib.mg_fwdprop(N, L, B, lens.data_ptr(), shifts.data_ptr(), p.data_ptr(), N, s.data_ptr(), N,
                            x.data_ptr(), out.data_ptr(), N, 0, ws.data_ptr(), nb, st)
    assert rc == 0
    torch.cuda.synchronize()
    return out


def test_noalloc_matches_workspace_entry_on_two_calls():
    from meshes_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(77)
    for call, (N, B) in enumerate([(128, 300), (64, 1025)]):   # two calls in a row, different shapes
        om = O.random_mesh(rng, N, "clements", "mzi", 0.02)
        lens = torch.tensor(om.lens, dtype=torch.int32, device="cuda")
        shifts = torch.tensor(om.shifts, dtype=torch.int32, device="cuda")
        p = torch.from_numpy(om.p.reshape(-1)).cuda()
        s = torch.from_numpy(om.s.reshape(-1)).cuda()
        x = torch.from_numpy(O.unit_columns(rng, N, B).astype(np.complex64)).cuda()
        ref = _run(lib, None, N, om.L, B, lens, shifts, p, s, x, False)
        got = _run(lib, None, N, om.L, B, lens, shifts, p, s, x, True)
        err = (torch.linalg.norm(got - ref) / torch.linalg.norm(ref)).item()
        assert err <= TOL, (call, err)


def test_noalloc_rejects_problems_above_its_scratch():
    from meshes_gb300 import _lib
    lib = _lib.load()
    N, L, B = 512, 2048, 1
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    rc = lib.mg_fwdprop_noalloc(N, L, B, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), N, None, 0,
                                dummy.data_ptr(), dummy.data_ptr(), N, 0, torch.cuda.current_stream().cuda_stream)
    assert rc == -2
    assert "scratch" in _lib.last_error()
