"""The native autotuner (mg_autotune) and the tuning table: every timed candidate is a valid plan, the
winner is the fastest of them, a recorded winner becomes the default configuration of its shape, and
argument errors come back as status codes."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("op,cr,N,L,B", [(0, 0, 64, 64, 512), (2, 0, 32, 32, 256), (1, 2, 48, 16, 100)])
def test_tune_returns_fastest_valid_candidate(op, cr, N, L, B):
    from meshes_gb300 import _lib
    from meshes_gb300.autotune import tune
    best, results = tune(op, N, L, B, crossing=cr, reps=3)
    assert best in results and len(results) >= 8
    assert results[best] == min(results.values()) and results[best] > 0
    lib = _lib.load()
    info = _lib.mg_plan_info()
    for c in results:
        assert lib.mg_plan(op, N, L, B, cr, 0, _lib.cfg_ptr(_lib.config(*c)), ctypes.byref(info)) == 0


def test_recorded_winner_becomes_default():
    from meshes_gb300 import _lib, geometry as gm
    lib = _lib.load()
    N, B, op = 48, 300, 0            # a shape absent from the committed table
    lens, shifts = gm.clements(N)
    L = len(lens)
    dev = torch.device("cuda")
    st = torch.cuda.current_stream().cuda_stream
    lens_d = torch.tensor(lens, dtype=torch.int32, device=dev)
    shifts_d = torch.tensor(shifts, dtype=torch.int32, device=dev)
    p = torch.rand(L, N // 2, 2, device=dev) * 6.28
    best, ms, n = _lib.mg_config(), ctypes.c_float(), ctypes.c_int()
    tried = (_lib.mg_config * 128)()
    tried_ms = (ctypes.c_float * 128)()
    try:
        _lib.check(lib.mg_autotune(op, N, L, B, 0, 0, lens_d.data_ptr(), shifts_d.data_ptr(), None, p.data_ptr(), N,
                                   None, 0, 2, 1, ctypes.byref(best), ctypes.byref(ms), tried, tried_ms, 128,
                                   ctypes.byref(n), st), "mg_autotune")
        assert n.value >= 8 and ms.value == min(tried_ms[i] for i in range(min(n.value, 128)))
        info = _lib.mg_plan_info()
        assert lib.mg_plan(op, N, L, B, 0, 0, None, ctypes.byref(info)) == 0
        assert (info.M, info.V, info.W) == (best.M, best.V, best.W)
    finally:
        lib.mg_set_tuned(op, 0, 0, N, 0, 0, None)


def test_autotune_argument_errors():
    from meshes_gb300 import _lib
    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    best = _lib.mg_config()
    p = torch.zeros(8, device="cuda")
    assert lib.mg_autotune(5, 8, 2, 4, 0, 0, None, None, None, p.data_ptr(), 8, None, 0, 1, 0, ctypes.byref(best),
                           None, None, None, 0, None, st) == -1
    assert lib.mg_autotune(0, 8, 2, 4, 3, 0, None, None, None, p.data_ptr(), 8, None, 0, 1, 0, ctypes.byref(best),
                           None, None, None, 0, None, st) == -1
    assert lib.mg_autotune(0, 8, 2, 4, 0, 0, None, None, None, p.data_ptr(), 8, None, 0, 0, 0, ctypes.byref(best),
                           None, None, None, 0, None, st) == -1
    assert "mg_autotune" in _lib.last_error()
