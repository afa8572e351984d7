"""The benchmark's CPU legs on small cases (no GPU): the port-based baselines of every workload return a positive
rate with their core count and sample description, and the reference arm's port is pinned against the
reference's fixtures.  The GPU legs of bench.py run on the GPU machine only."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench as bn  # noqa: E402


def _check(cb, unit="MZI-apps/s"):
    assert cb["value"] > 0 and cb["unit"] == unit
    assert cb["cores"] >= 1 and cb["kind"] == "port" and cb["sample"]


def test_batched_baseline():
    prob = bn.make_batched_problem(n_meshes=4)
    rng = np.random.default_rng(1)
    for d in prob:
        d["gy"] = bn.unit_rows(rng, d["B"], d["N"], real=d["cr"] == "orth")
    _check(bn.cpu_baseline_batched(prob, seconds=0.05))


def test_fit_baseline():
    rng = np.random.default_rng(2)
    n = 16
    lens, shifts = bn.clements_layout(n)
    mask = bn.active_mask(n, lens, shifts)
    p0 = rng.uniform(0, 2 * np.pi, (len(lens), n // 2, 2)).astype(np.float32)
    s0 = rng.normal(0, 0.02, (len(lens), n // 2, 2)).astype(np.float32)
    p0[~mask] = 0
    s0[~mask] = 0
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    _check(bn.cpu_baseline_fit(lens, shifts, p0, s0, Q.astype(np.complex64), seconds=0.05), "steps/s")


def test_served_baseline():
    rng = np.random.default_rng(3)
    meshes_h, pools = [], []
    for i, n in enumerate((16, 32)):
        if i == 0:
            lens, shifts = bn.clements_layout(n)
            strides, L = None, len(lens)
            mask = bn.active_mask(n, lens, shifts)
        else:
            strides, lens, shifts = bn.fft_layout(n), None, None
            L = len(strides)
            mask = np.ones((L, n // 2), bool)
        p = rng.uniform(0, 2 * np.pi, (L, n // 2, 2)).astype(np.float32)
        p[~mask] = 0
        meshes_h.append(dict(N=n, lens=lens, shifts=shifts, strides=strides, p=p, s=np.zeros_like(p),
                             n_mzi=int(mask.sum())))
        pools.append(bn.unit_rows(rng, 64, n))
    ids = rng.integers(0, 2, 40)
    cb = bn.cpu_baseline_served(meshes_h, pools, ids, rng.integers(1, 64, 40), rng.random(40) < 0.3, n_req=40)
    _check(cb)
    assert cb["req_per_s"] > 0 and cb["per_request_ms_p99"] >= cb["per_request_ms_p50"] > 0


def test_lossy_baseline():
    lens, shifts, p, s, x, yt, _ = bn.make_problem()
    rng = np.random.default_rng(4)
    L = len(lens)
    s14 = np.zeros((L, bn.N // 2, 14))
    s14[..., :2] = s
    s14[..., 10:] = -0.004
    _check(bn.cpu_baseline_lossy(lens, shifts, p, s14, x[:16], yt[:16], n_vec=2, seconds=0.05))


def test_reference_port_pinned():
    pin = bn.cpu_pin_port()
    assert pin["pinned"] and pin["max_rel_err_complex128"] < 1e-12
