"""Continuous-batching server: results equal alone and in the mix, memory admission, failures.

Failures are made on the host (bad requests, an over-budget request, a cancelled request, a client
thread that dies mid-stream); nothing here faults or hangs the GPU.
"""
import threading

import numpy as np
import pytest

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


def _pool(rng):
    specs = [("clements", 16), ("fft", 32), ("clements", 64), ("fft", 128), ("clements", 256), ("fft", 512),
             ("clements", 512)]
    return [O.random_mesh(rng, N, geo, "mzi", 0.02) for geo, N in specs]


def test_same_result_alone_and_in_the_mix():
    from meshes_gb300.serve import MeshServer
    rng = np.random.default_rng(41)
    oms = _pool(rng)
    srv = MeshServer([gpu_mesh(om) for om in oms], mem_budget=64 << 20)
    srv.start()
    try:
        # the probe requests, alone
        xf = O.unit_columns(rng, 256, 37).astype(np.complex64)
        xg = O.unit_columns(rng, 64, 13).astype(np.complex64)
        gg = O.unit_columns(rng, 64, 13).astype(np.complex64)
        y_alone = srv.submit(4, xf).result(60)
        yg_alone, dp_alone, gx_alone = srv.submit(2, xg, gy=gg).result(60)
        # the same requests inside a stream of mixed requests submitted while others run
        futs = []
        for k in range(200):
            i = int(rng.integers(len(oms)))
            b = int(rng.integers(1, 64))
            x = O.unit_columns(rng, oms[i].N, b).astype(np.complex64)
            g = O.unit_columns(rng, oms[i].N, b).astype(np.complex64) if k % 5 == 0 else None
            futs.append((i, x, g, srv.submit(i, x, gy=g)))
            if k == 77:
                f_probe = srv.submit(4, xf)
                f_probe_g = srv.submit(2, xg, gy=gg)
        y_mix = f_probe.result(60)
        yg_mix, dp_mix, gx_mix = f_probe_g.result(60)
        assert np.array_equal(y_alone, y_mix)
        assert np.array_equal(dp_alone, dp_mix) and np.array_equal(gx_alone, gx_mix)
        # every result of the mix against the oracle
        for i, x, g, f in futs:
            r = f.result(60)
            y_ref = O.propagate(oms[i], x)
            if g is None:
                assert O.rel_err(r, y_ref) < TOL
            else:
                y, dp, gx = r
                G, _, gin = O.vjp_unitary(oms[i], y_ref, g)
                assert O.rel_err(y, y_ref) < TOL
                assert O.rel_err(gx, gin) < TOL
                assert O.rel_err(dp, O.contract_dp(oms[i], G)) < TOL
        assert O.rel_err(y_alone, O.propagate(oms[4], xf)) < TOL
        assert srv.ticks > 2                      # the mix was served over several ticks
    finally:
        srv.stop()
    assert srv.kernel_status() == 0


def test_admission_by_memory_and_bad_requests():
    from meshes_gb300.serve import MeshServer, ServerError
    rng = np.random.default_rng(42)
    oms = _pool(rng)[:3]
    srv = MeshServer([gpu_mesh(om) for om in oms], mem_budget=1 << 20)   # 1 MiB arena
    srv.start()
    try:
        with pytest.raises(ServerError):
            srv.submit(0, np.zeros((3, 17), np.complex64))               # wrong N
        with pytest.raises(ServerError):
            srv.submit(9, np.zeros((3, 16), np.complex64))               # no such mesh
        with pytest.raises(ServerError):
            srv.submit(2, np.zeros((4096, 64), np.complex64))            # never fits the arena
        # many requests that together exceed the arena: admitted as memory frees up
        futs = [(i % 3, srv.submit(i % 3, O.unit_columns(rng, oms[i % 3].N, 200).astype(np.complex64)))
                for i in range(60)]
        for i, f in futs:
            assert f.result(60).shape == (200, oms[i].N)
        # a cancelled request is skipped
        f = srv.submit(0, np.ones((2, 16), np.complex64))
        f.cancel()
    finally:
        srv.stop()


@pytest.mark.filterwarnings("ignore::pytest.PytestUnhandledThreadExceptionWarning")   # the crash is the point
def test_client_thread_dying_midway_leaves_the_loop_draining():
    from meshes_gb300.serve import MeshServer
    rng = np.random.default_rng(43)
    oms = _pool(rng)[:2]
    srv = MeshServer([gpu_mesh(om) for om in oms], mem_budget=16 << 20)
    srv.start()
    futs = []

    def client():
        for k in range(50):
            futs.append(srv.submit(k % 2, np.ones((8, oms[k % 2].N), np.complex64)))
            if k == 30:
                raise RuntimeError("client crashed")

    t = threading.Thread(target=client)
    t.start()
    t.join()
    srv.stop(drain=True)
    assert len(futs) == 31
    assert all(f.done() and not f.cancelled() and f.exception() is None for f in futs)
    assert srv.error is None
