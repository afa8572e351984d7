"""Autotuner of the propagation kernels' tile configuration.

For a shape (op, crossing, geometry, N, L, B) the library's native tuner ``mg_autotune`` times the valid
candidates on the GPU - tiles built once, CUDA events on the launch stream, L2 flushed between
repetitions - in two stages: the register blocking and CTA width (modes per lane M, vectors per lane V,
warps per CTA W), then, around the winner, layers per pipeline stage CL, stages S and (forward) the split
launch - and keeps the fastest.  This module supplies a random mesh of the shape and keeps the table.
Results live in ``tuned_configs.json`` next to this file (keyed by op/crossing/geometry/N and a batch
range) and are loaded into the library's tuning table by ``load_table()`` (called on import of the
package), so every call that passes no explicit configuration - the reference-shaped entry points
included - uses them.

    python -m meshes_gb300.autotune --op fwd --N 256 --B 4096      # tune one shape, update the table
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
from typing import Dict, Optional, Tuple

import numpy as np

from . import _lib
from ._lib import OP_BWD, OP_FWD, OP_FWDDIFF, check, load

TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned_configs.json")
OPS = {"fwd": OP_FWD, "fwddiff": OP_FWDDIFF, "bwd": OP_BWD}
CROSS = {"mzi": 0, "sym": 1, "orth": 2}


def _key(op, crossing, geometry, N):
    return "%d/%d/%d/%d" % (op, crossing, geometry, N)


def load_table(path: str = TABLE) -> int:
    """Load the committed tuning table into the library; returns the number of entries."""
    if not os.path.exists(path):
        return 0
    lib = load()
    with open(path) as f:
        table = json.load(f)
    n = 0
    for key, entries in table.items():
        op, cr, geo, N = map(int, key.split("/"))
        for e in entries:
            cfg = _lib.config(*e["cfg"])
            check(lib.mg_set_tuned(op, cr, geo, N, int(e["B"][0]), int(e["B"][1]), _lib.cfg_ptr(cfg)), "mg_set_tuned")
            n += 1
    return n


def tune(op: int, N: int, L: int, B: int, crossing: int = 0, geometry: int = 0, reps: int = 5,
         cands: Optional[list] = None, device=None) -> Tuple[Tuple[int, ...], Dict]:
    """Time the candidates on a random mesh of this shape; returns (best config, {config: ms})."""
    import torch
    from . import geometry as gm
    lib = load()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    st = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(0)
    real = crossing == 2
    n_p = 1 if real else 2
    n_s = {0: 2, 1: 1, 2: 0}[crossing]
    if geometry == 0:                                     # Clements layer pattern, repeated to depth L
        lens0, shifts0 = gm.clements(N)
        lens_d = torch.tensor([lens0[l % len(lens0)] for l in range(L)], dtype=torch.int32, device=dev)
        shifts_d = torch.tensor([shifts0[l % len(shifts0)] for l in range(L)], dtype=torch.int32, device=dev)
        geo_args = (lens_d.data_ptr(), shifts_d.data_ptr(), None)
    else:                                                 # log-depth butterfly strides, repeated
        st0 = gm.fft(N)
        st_d = torch.tensor([st0[l % len(st0)] for l in range(L)], dtype=torch.int32, device=dev)
        geo_args = (None, None, st_d.data_ptr())
    p = torch.tensor(rng.uniform(0, 6.28, (L, N // 2, n_p)).astype(np.float32), device=dev)
    s = torch.tensor(rng.normal(0, .02, (L, N // 2, max(n_s, 1))).astype(np.float32), device=dev) if n_s else None
    if cands:
        return _time_given(op, N, L, B, crossing, geometry, geo_args, p, s, n_p, n_s, reps, cands, dev, st)
    best = _lib.mg_config()
    best_ms = ctypes.c_float()
    tried = (_lib.mg_config * 256)()
    tried_ms = (ctypes.c_float * 256)()
    n = ctypes.c_int()
    check(lib.mg_autotune(op, N, L, B, crossing, geometry, *geo_args, p.data_ptr(), N // 2 * n_p,
                          None if s is None else s.data_ptr(), N // 2 * n_s, reps, 0, ctypes.byref(best),
                          ctypes.byref(best_ms), tried, tried_ms, 256, ctypes.byref(n), st), "mg_autotune")
    as_tuple = (lambda c: (c.M, c.V, c.W, c.CL, c.S, c.split))
    results = {as_tuple(tried[i]): float(tried_ms[i]) for i in range(min(n.value, 256))}
    return as_tuple(best), results


def _time_given(op, N, L, B, crossing, geometry, geo_args, p, s, n_p, n_s, reps, cands, dev, st):
    """Time an explicit candidate list (for comparisons of chosen configurations)."""
    import torch
    lib = load()
    real = crossing == 2
    dt = torch.float32 if real else torch.complex64
    x = torch.randn(B, N, dtype=dt, device=dev)
    y = torch.empty_like(x)
    g = torch.randn_like(x)
    gi = torch.empty_like(x)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    results = {}
    for c in cands:
        cfg = _lib.config(*c)
        nb = lib.mg_workspace_bytes(op, N, L, B, crossing, geometry, _lib.cfg_ptr(cfg))
        if nb == 0:
            continue
        ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        lib.mg_workspace_init(ws.data_ptr(), nb, st)
        if lib.mg_build_tiles(op, N, L, geometry, *geo_args, crossing, p.data_ptr(), N // 2 * n_p,
                              None if s is None else s.data_ptr(), N // 2 * n_s, p.data_ptr() if op == OP_FWDDIFF
                              else None, None, None, B, _lib.cfg_ptr(cfg), ws.data_ptr(), nb, st):
            continue
        args = {OP_FWD: (x.data_ptr(), None, y.data_ptr(), None), OP_FWDDIFF: (x.data_ptr(), g.data_ptr(),
                y.data_ptr(), gi.data_ptr()), OP_BWD: (y.data_ptr(), g.data_ptr(), None, gi.data_ptr())}[op]

        def run():
            return lib.mg_propagate(op, N, L, B, crossing, geometry, *args, N, None, 0, 0, _lib.cfg_ptr(cfg),
                                    ws.data_ptr(), nb, st)

        if run():
            continue
        ts = []
        for _ in range(reps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            torch.cuda.synchronize(dev)
            ts.append(e0.elapsed_time(e1))
        if lib.mg_read_status(ws.data_ptr(), 1, st) == 0:
            results[c] = statistics.median(ts)
    best = min(results, key=results.get)
    return best, results


def record(op: int, crossing: int, geometry: int, N: int, B_range: Tuple[int, int], cfg, ms: float,
           path: str = TABLE):
    table = {}
    if os.path.exists(path):
        with open(path) as f:
            table = json.load(f)
    key = _key(op, crossing, geometry, N)
    entries = [e for e in table.get(key, []) if tuple(e["B"]) != tuple(B_range)]
    entries.append({"B": list(B_range), "cfg": list(cfg), "ms": round(ms, 5)})
    table[key] = sorted(entries, key=lambda e: e["B"][0])
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--op", default="fwd", choices=list(OPS))
    ap.add_argument("--crossing", default="mzi", choices=list(CROSS))
    ap.add_argument("--geometry", default="nn", choices=["nn", "fft"])
    ap.add_argument("--N", type=int, default=256)
    ap.add_argument("--L", type=int, default=0, help="depth (default N for nn, log2 N for fft)")
    ap.add_argument("--B", type=int, default=4096)
    ap.add_argument("--B-range", type=int, nargs=2, default=None, help="batch range the result applies to")
    ap.add_argument("--write", action="store_true", help="store the winner in tuned_configs.json")
    a = ap.parse_args()
    geo = 0 if a.geometry == "nn" else 1
    L = a.L or (a.N if geo == 0 else a.N.bit_length() - 1)
    op = OPS[a.op]
    best, res = tune(op, a.N, L, a.B, CROSS[a.crossing], geo)
    for c, ms in sorted(res.items(), key=lambda kv: kv[1])[:8]:
        print("M=%d V=%d W=%d CL=%d S=%d split=%d  %.4f ms" % (tuple(c) + (0,) * (6 - len(c)) + (ms,)))
    if a.write:
        rng = tuple(a.B_range) if a.B_range else (a.B // 2 + 1, a.B * 2)
        record(op, CROSS[a.crossing], geo, a.N, rng, best, res[best])
        print("recorded", best, "for B in", rng)


if __name__ == "__main__":
    main()
