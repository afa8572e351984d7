"""Benchmark of the mesh-propagation hot path on GB300.

Workload (one "step"): forward propagation plus back-propagation of phase gradients through an
imperfect Clements MZI mesh, N=256 modes, L=256 layers (32640 MZIs), splitting errors
alpha, beta ~ N(0, 0.02), B=4096 complex64 unit-norm input vectors, loss J = sum |y - y_t|^2:
  mg_fwdprop (x -> y), g = 2 (y - y_t), mg_backdiff (y, g -> dJ/dp, dJ/dx*).
Metric: MZI applications per second for fwd+bwd (n_MZI * B per step), with the fraction of the FP32
CUDA-core peak at the reference's own FLOP counts (32 per MZI-application forward, 96 backward).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica on its own GPU (the path needs no
collective); value = all ranks' MZI applications / max-over-ranks time.  ``--impl reference`` times
the reference algorithm's CPU implementation (the oracle's C++ port of c/dot.cpp, all host threads)
on the same workload, on rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N, B, SIGMA, SEED = 256, 4096, 0.02, 1002
FLOP_FWD, FLOP_BWD = 32, 96           # reference gpu/test.py:208,220
METRIC = "MZI-apps/s (fwd+bwd)"
WORKLOAD = "clements_mzi_N256_L256_B4096_fwd+bwd"


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:   # pragma: no cover
        return os.cpu_count() or 1


def make_problem():
    """Seeded synthetic mesh and fields (numpy), independent of the oracle."""
    from meshes_gb300 import geometry as gm
    rng = np.random.default_rng(SEED)
    lens, shifts = gm.clements(N)
    L = len(lens)
    mask = gm.active_mask_nn(N, lens, shifts)
    p = rng.uniform(0, 2 * np.pi, (L, N // 2, 2)).astype(np.float32)
    s = rng.normal(0, SIGMA, (L, N // 2, 2)).astype(np.float32)
    p[~mask] = 0
    s[~mask] = 0

    def unit(rows):
        x = rng.standard_normal((rows, N)) + 1j * rng.standard_normal((rows, N))
        return (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.complex64)

    x = unit(B)
    yt = unit(B)
    return lens, shifts, p, s, x, yt, int(mask.sum())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def gpu_id(torch, dev) -> str:
    """nvidia-smi -i selector of this process's GPU (PCI bus id when torch exposes it)."""
    pr = torch.cuda.get_device_properties(dev)
    try:
        return "%08x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
    except AttributeError:
        return str(dev.index or 0)


def cpu_baseline(problem, seconds=10.0, with_c128=True):
    """Reference algorithm on the host cores: the oracle's C++ port of c/dot.cpp (complex64, OpenMP),
    forward (mode 0) + back-propagation (mode 2) on a bounded sample of the batch."""
    from oracle import meshes_oracle as O
    from oracle import port as P
    lens, shifts, p, s, x, yt, n_mzi = problem
    om = O.OracleMesh(N=N, L=len(lens), crossing="mzi", lens=lens, shifts=shifts, p=p, s=s)
    fns = P.port_lib()
    threads = host_threads()
    bs = max(8, min(B, 16 * threads))
    xs, ts = x[:bs], yt[:bs]
    t0 = time.perf_counter()
    reps, work = 0, 0.0
    while True:
        a = time.perf_counter()
        y = P.forward(fns, om, xs, threads=threads, dtype=np.complex64)
        P.vjp(fns, om, y, 2 * (y - ts), threads=threads, dtype=np.complex64)
        work += time.perf_counter() - a
        reps += 1
        if time.perf_counter() - t0 > seconds and reps >= 2:
            break
    rate = n_mzi * bs * reps / work
    out = {"value": rate, "unit": "MZI-apps/s", "cores": threads, "kind": "port",
           "sample": "%d of the %d vectors, fwd (mode 0) + bwd (mode 2), complex64, %d repeats, %.1f s"
                     % (bs, B, reps, work)}
    if not with_c128:
        return out
    # the same in complex128 (the reference's own precision for dot / dot_vjp), a shorter sample
    a = time.perf_counter()
    reps128 = 0
    while True:
        y = P.forward(fns, om, xs, threads=threads, dtype=np.complex128)
        P.vjp(fns, om, y, 2 * (y - ts), threads=threads, dtype=np.complex128)
        reps128 += 1
        if time.perf_counter() - a > seconds / 4 and reps128 >= 2:
            break
    out["value_complex128"] = n_mzi * bs * reps128 / (time.perf_counter() - a)
    return out


def traffic_from_profiles(name: str):
    """dram bytes per launch recorded in profiles/<name> ('dram_bytes_per_launch: X'), else None."""
    fn = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(fn):
            if line.strip().startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def run_reference(args, rank):
    if rank != 0:
        return
    problem = make_problem()
    n_mzi = problem[6]
    # about a minute of CPU work in total, whatever K and W are (each step is a bounded sample)
    per_step = max(0.05, 60.0 / max(args.steps + args.warmup, 1))
    for _ in range(args.warmup):
        cpu_baseline(problem, seconds=min(per_step, 0.5), with_c128=False)
    vals = []
    for _ in range(args.steps):
        vals.append(cpu_baseline(problem, seconds=per_step, with_c128=False))
    value = statistics.median(v["value"] for v in vals)
    cb = dict(vals[0])
    cb["value"] = value
    line = {"metric": METRIC, "value": value, "unit": "MZI-apps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * n_mzi * B / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "N": N, "L": N, "B": B, "n_mzi": n_mzi, "splitter_sigma": SIGMA},
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "MZI-apps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, rank, world, local_rank):
    import torch
    import torch.distributed as dist

    from meshes_gb300 import _lib
    lib = _lib.load()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream

    lens, shifts, p, s, x_h, yt_h, n_mzi = make_problem()
    L = len(lens)
    lens_d = torch.tensor(lens, dtype=torch.int32, device=dev)
    shifts_d = torch.tensor(shifts, dtype=torch.int32, device=dev)
    p_d = torch.from_numpy(p).to(dev).reshape(-1)
    s_d = torch.from_numpy(s).to(dev).reshape(-1)
    x = torch.from_numpy(x_h).to(dev)                      # (B, N): vector b at b*N (ldu = N)
    yt = torch.from_numpy(yt_h).to(dev)
    y = torch.empty_like(x)
    g = torch.empty_like(x)
    gin = torch.empty_like(x)
    dp = torch.empty(L * N // 2 * 2, dtype=torch.float32, device=dev)
    ldp, lds = N // 2 * 2, N // 2 * 2
    wsb_f = lib.mg_workspace_bytes(0, N, L, B, 0, 0, None)
    wsb_b = lib.mg_workspace_bytes(2, N, L, B, 0, 0, None)
    ws_f = torch.empty(wsb_f, dtype=torch.uint8, device=dev)
    ws_b = torch.empty(wsb_b, dtype=torch.uint8, device=dev)
    for w, n in ((ws_f, wsb_f), (ws_b, wsb_b)):
        _lib.check(lib.mg_workspace_init(w.data_ptr(), n, st), "mg_workspace_init")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    launches_per_step = 4          # coefficient tiles, forward, back-propagation with fused L2, gradient reduce

    def step(xx, yy_t, dp_out=None):
        """One training step through the programmed-mesh C ABI: the back-propagation tiles are built once
        and serve the forward pass too; dJ/dy* = 2 (y - y_t) is formed inside the backward kernel."""
        dp_out = dp if dp_out is None else dp_out
        _lib.check(lib.mg_build_tiles(2, N, L, 0, lens_d.data_ptr(), shifts_d.data_ptr(), None, 0, p_d.data_ptr(), ldp,
                                      s_d.data_ptr(), lds, None, None, None, B, None, ws_b.data_ptr(), wsb_b, st),
                   "mg_build_tiles")
        _lib.check(lib.mg_propagate(3, N, L, B, 0, 0, xx.data_ptr(), None, y.data_ptr(), None, N, None, 0, 0, None,
                                    ws_b.data_ptr(), wsb_b, st), "mg_propagate")
        _lib.check(lib.mg_propagate_l2(N, L, B, 0, 0, y.data_ptr(), yy_t.data_ptr(), None, gin.data_ptr(), N,
                                       dp_out.data_ptr(), ldp, 0, None, ws_b.data_ptr(), wsb_b, st), "mg_propagate_l2")

    def step_dropin(xx, yy_t):
        """The same step through the reference-shaped entry points (mg_fwdprop, mg_backdiff)."""
        _lib.check(lib.mg_fwdprop(N, L, B, lens_d.data_ptr(), shifts_d.data_ptr(), p_d.data_ptr(), ldp,
                                  s_d.data_ptr(), lds, xx.data_ptr(), y.data_ptr(), N, 0, ws_f.data_ptr(), wsb_f, st),
                   "mg_fwdprop")
        torch.sub(y, yy_t, out=g).mul_(2.0)
        _lib.check(lib.mg_backdiff(N, L, B, lens_d.data_ptr(), shifts_d.data_ptr(), p_d.data_ptr(), dp.data_ptr(),
                                   ldp, s_d.data_ptr(), lds, y.data_ptr(), g.data_ptr(), None, gin.data_ptr(), N, 0, 0,
                                   ws_b.data_ptr(), wsb_b, st), "mg_backdiff")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def timed(fn, k):
        """K timed calls, each bracketed by CUDA events on the launch stream, L2 flushed in between."""
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        for a, b in evs:
            flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) * 1e-3 for a, b in evs]

    if args.profile and args.bwd_config:
        # three back-propagation launches with an explicit tile configuration (M,V,W,CL,S,split), for ncu
        # comparisons of configurations (e.g. -k regex:prop -s 1 -c 1)
        cfg = _lib.config(*[int(v) for v in args.bwd_config.split(",")])
        nb = lib.mg_workspace_bytes(2, N, L, B, 0, 0, _lib.cfg_ptr(cfg))
        if nb == 0:
            raise SystemExit("invalid configuration: " + _lib.last_error())
        ws_c = torch.empty(nb, dtype=torch.uint8, device=dev)
        _lib.check(lib.mg_workspace_init(ws_c.data_ptr(), nb, st), "mg_workspace_init")
        _lib.check(lib.mg_build_tiles(2, N, L, 0, lens_d.data_ptr(), shifts_d.data_ptr(), None, 0, p_d.data_ptr(), ldp,
                                      s_d.data_ptr(), lds, None, None, None, B, _lib.cfg_ptr(cfg), ws_c.data_ptr(), nb,
                                      st), "mg_build_tiles")
        for _ in range(3):
            _lib.check(lib.mg_propagate(2, N, L, B, 0, 0, x.data_ptr(), yt.data_ptr(), None, gin.data_ptr(), N,
                                        dp.data_ptr(), ldp, 0, _lib.cfg_ptr(cfg), ws_c.data_ptr(), nb, st),
                       "mg_propagate")
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile_bwd_config": args.bwd_config, "status": lib.mg_read_status(ws_c.data_ptr(), 0, st)}))
        return
    if args.profile:
        # one warm-up step and one profiled step, no timing (for ncu captures: -s 2 -c 2 on prop_kernel)
        step(x, yt)
        step(x, yt)
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile_steps": 2, "status": lib.mg_read_status(ws_b.data_ptr(), 0, st)}))
        return

    # ---- device-resident step (value)
    for _ in range(args.warmup):
        step(x, yt)
    barrier()
    with ClockSampler(gpu_id(torch, dev)) as cs:
        times = timed(lambda: step(x, yt), args.steps)
        barrier()
    t_step = sum(times) / len(times)
    for _ in range(3):
        step_dropin(x, yt)
    t_dropin = statistics.median(timed(lambda: step_dropin(x, yt), max(5, args.steps // 4)))
    status = max(lib.mg_read_status(ws_f.data_ptr(), 0, st), lib.mg_read_status(ws_b.data_ptr(), 0, st))
    if status != 0:
        raise RuntimeError("kernel status %d" % status)

    # ---- end to end through the C ABI with host buffers: H2D x, y_t; D2H dJ/dp and the loss
    x_pin = torch.from_numpy(x_h).pin_memory()
    yt_pin = torch.from_numpy(yt_h).pin_memory()
    dp_pin = torch.empty(dp.numel(), dtype=torch.float32).pin_memory()
    xd = torch.empty_like(x)
    ytd = torch.empty_like(yt)

    def e2e_step():
        xd.copy_(x_pin, non_blocking=True)
        ytd.copy_(yt_pin, non_blocking=True)
        step(xd, ytd)
        dp_pin.copy_(dp, non_blocking=True)                  # the step's result: dJ/dp

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier()
    times_e2e = timed(e2e_step, args.steps)
    barrier()
    t_e2e_serial = sum(times_e2e) / len(times_e2e)
    h2d = 2 * x.numel() * 8
    d2h = dp.numel() * 4

    # the same steps as a training loop runs them: on copy streams, the next step's inputs are copied into
    # the other of two buffers, and each step's dJ/dp (written to one of two device buffers) is copied back,
    # while the compute stream runs the next step (every copy still inside the timed region; one pair of
    # events around all K steps, the last read-back included)
    copy_stream = torch.cuda.Stream(dev)          # host -> device
    back_stream = torch.cuda.Stream(dev)          # device -> host (its own queue: a read-back waiting for its
                                                  # step must not hold up the next step's input copy)
    xs = [torch.empty_like(x) for _ in range(2)]
    yts = [torch.empty_like(yt) for _ in range(2)]
    dps = [torch.empty_like(dp) for _ in range(2)]
    dp_pins = [torch.empty(dp.numel(), dtype=torch.float32).pin_memory() for _ in range(2)]
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_used = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]

    def e2e_loop(k_steps):
        for k in range(k_steps):
            i = k & 1
            copy_stream.wait_event(ev_used[i])               # step k-2 is done with buffer i
            with torch.cuda.stream(copy_stream):
                xs[i].copy_(x_pin, non_blocking=True)
                yts[i].copy_(yt_pin, non_blocking=True)
                ev_in[i].record(copy_stream)
            stream.wait_event(ev_in[i])
            stream.wait_event(ev_out[i])                     # step k-2's dJ/dp has left dps[i]
            step(xs[i], yts[i], dps[i])
            ev_used[i].record(stream)
            back_stream.wait_event(ev_used[i])
            with torch.cuda.stream(back_stream):
                dp_pins[i].copy_(dps[i], non_blocking=True)  # the step's result: dJ/dp
                ev_out[i].record(back_stream)
        stream.wait_event(ev_out[(k_steps - 1) & 1])

    for e in ev_used + ev_out:
        e.record(stream)
    e2e_loop(max(2, args.warmup))
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    e2e_loop(args.steps)
    e1.record(stream)
    barrier()
    t_e2e = e0.elapsed_time(e1) * 1e-3 / args.steps

    # ---- roofline of the dominant kernel: the back-propagation kernel alone (tiles built once)
    def bwd_kernel():
        _lib.check(lib.mg_propagate(2, N, L, B, 0, 0, y.data_ptr(), g.data_ptr(), None, gin.data_ptr(), N, None, 0, 0,
                                    None, ws_b.data_ptr(), wsb_b, st), "mg_propagate")

    def fwd_kernel():
        _lib.check(lib.mg_propagate(0, N, L, B, 0, 0, x.data_ptr(), None, y.data_ptr(), None, N, None, 0, 0, None,
                                    ws_f.data_ptr(), wsb_f, st), "mg_propagate")

    bwd_kernel()
    t_bwd = statistics.median(timed(bwd_kernel, max(5, args.steps)))
    t_fwd = statistics.median(timed(fwd_kernel, max(5, args.steps)))
    # forward-mode derivative (the reference's fwddiff: y and dy along a direction of all phases)
    wsb_d = lib.mg_workspace_bytes(1, N, L, B, 0, 0, None)
    ws_d = torch.empty(wsb_d, dtype=torch.uint8, device=dev)
    _lib.check(lib.mg_workspace_init(ws_d.data_ptr(), wsb_d, st), "mg_workspace_init")
    dp_dir = torch.randn(L * N // 2 * 2, dtype=torch.float32, device=dev)
    _lib.check(lib.mg_build_tiles(1, N, L, 0, lens_d.data_ptr(), shifts_d.data_ptr(), None, 0, p_d.data_ptr(), ldp,
                                  s_d.data_ptr(), lds, dp_dir.data_ptr(), None, None, B, None, ws_d.data_ptr(), wsb_d,
                                  st), "mg_build_tiles")
    dy = torch.empty_like(x)

    def fwddiff_kernel():
        _lib.check(lib.mg_propagate(1, N, L, B, 0, 0, x.data_ptr(), None, y.data_ptr(), dy.data_ptr(), N, None, 0, 0,
                                    None, ws_d.data_ptr(), wsb_d, st), "mg_propagate")

    t_fwddiff = statistics.median(timed(fwddiff_kernel, max(5, args.steps // 4)))
    # FP32 FMA peak of this device (the measured-peaks file has HBM and bf16 only)
    props = torch.cuda.get_device_properties(dev)
    sink = torch.empty(props.multi_processor_count * 4 * 256, device=dev)
    iters = 4000

    def probe():
        _lib.check(lib.mg_fma_probe(sink.data_ptr(), props.multi_processor_count * 4, 256, iters, st), "fma_probe")

    probe()
    t_probe = min(timed(probe, 3))
    peak = props.multi_processor_count * 4 * 256 * iters * 64 * 2 / t_probe

    # ---- reduce over ranks (replicas: the job ends with its slowest rank)
    from meshes_gb300.replicas import max_over_ranks
    t_max = max_over_ranks(t_step, device=dev)
    t_e2e = max_over_ranks(t_e2e, device=dev)
    if rank != 0:
        return
    units = n_mzi * B * world
    value = units / t_max
    bwd_flops = n_mzi * B * FLOP_BWD
    achieved = bwd_flops / t_bwd
    traffic = traffic_from_profiles("prop_bwd_clements_N256_L256_B4096.md")
    bwd_bytes = B * N * 3 * 8 + n_mzi * 4 * (2 + 2) + n_mzi * 4 * 2
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak, hbm_src = float(json.load(f)["hbm_gbs"]), "measured (copy bandwidth)"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback"
    line = {
        "metric": METRIC, "value": value, "unit": "MZI-apps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded normal fields, uniform phases)",
        "config": {"workload": WORKLOAD, "N": N, "L": L, "B": B, "n_mzi": n_mzi, "splitter_sigma": SIGMA,
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas" if world > 1 else "1 GPU"},
        "pct_fp32_peak": 100 * value / world * (FLOP_FWD + FLOP_BWD) / peak,
        "fp32_peak_tflops": peak / 1e12,
        "step": "programmed mesh: mg_build_tiles(bwd) + mg_propagate(fwd from bwd tiles) + mg_propagate_l2",
        "drop_in_step": {"ms": t_dropin * 1e3, "mzi_per_s": units / world / t_dropin,
                         "path": "mg_fwdprop + 2(y - y_t) + mg_backdiff (reference-shaped entry points)"},
        "kernels": {"fwd_prop_ms": t_fwd * 1e3, "bwd_prop_ms": t_bwd * 1e3, "fwddiff_prop_ms": t_fwddiff * 1e3,
                    "fwddiff_mzi_per_s": n_mzi * B / t_fwddiff,
                    "fwd_mzi_per_s": n_mzi * B / t_fwd, "bwd_mzi_per_s": n_mzi * B / t_bwd},
        "roofline": {"kernel": "prop_kernel<BWD> (back-propagation)", "bound": "fp32", "achieved": achieved / 1e12,
                     "peak": peak / 1e12, "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": "measured: FP32 FMA probe on this GPU (no FP32 entry in the measured-peaks file)",
                     "traffic": traffic, "algorithmic_flops_per_launch": bwd_flops},
        # the same kernel against the HBM roofline (algorithmic bytes: read y and g, write g_in, the
        # parameters and dJ/dp), showing how far it is from being memory-bound
        "roofline_hbm": {"kernel": "prop_kernel<BWD> (back-propagation)", "bound": "hbm",
                         "achieved": bwd_bytes / t_bwd / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": bwd_bytes / t_bwd / 1e9 / hbm_peak, "traffic": traffic,
                         "peak_source": hbm_src, "algorithmic_bytes_per_launch": bwd_bytes},
        "e2e": {"value": units / t_e2e, "unit": "MZI-apps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "pipelined": "next step's H2D and previous step's D2H on copy streams during the current step",
                "serialized_value": units / t_e2e_serial},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": cs.summary(),
    }
    line["cpu_baseline"] = cpu_baseline((lens, shifts, p, s, x_h, yt_h, n_mzi), seconds=10.0)
    print(json.dumps(line))


def make_batched_problem(seed=1003, n_meshes=512):
    """512 meshes drawn 1:1:1 from Clements-mzi, Reck-mzi (native 2N-3 layers) and Clements-orth,
    N uniform in {8, ..., 256}, batch uniform in [1, 2048], phases U[0, 2pi), splitters N(0, 0.01)."""
    from meshes_gb300 import geometry as gm
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_meshes):
        kind = ("clements-mzi", "reck-mzi", "clements-orth")[i % 3]
        N = int(rng.choice([8, 16, 32, 64, 128, 256]))
        B = int(rng.integers(1, 2049))
        lens, shifts = gm.reck(N) if kind.startswith("reck") else gm.clements(N)
        L = len(lens)
        mask = gm.active_mask_nn(N, lens, shifts)
        cr = "orth" if kind.endswith("orth") else "mzi"
        n_p = 1 if cr == "orth" else 2
        p = rng.uniform(0, 2 * np.pi, (L, N // 2, n_p)).astype(np.float32)
        p[~mask] = 0
        s = None
        if cr == "mzi":
            s = rng.normal(0, 0.01, (L, N // 2, 2)).astype(np.float32)
            s[~mask] = 0
        x = rng.standard_normal((B, N)) + (0 if cr == "orth" else 1j * rng.standard_normal((B, N)))
        x = (x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.float32 if cr == "orth" else np.complex64)
        out.append(dict(kind=kind, N=N, B=B, L=L, lens=lens, shifts=shifts, cr=cr, p=p, s=s, x=x,
                        n_mzi=int(mask.sum())))
    return out


def run_c1(args):
    """Plain forward propagation, Clements mzi N=64 L=64 (2016 MZIs), ideal splitters, B=1024 unit-norm
    complex64 columns, through the reference-shaped entry point mg_fwdprop; with the unitarity error
    ||U U^H - I||_F of the programmed mesh."""
    import torch
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300 import geometry as gm
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(1000)
    Nc, Bc = 64, 1024
    lens, shifts = gm.clements(Nc)
    mask = gm.active_mask_nn(Nc, lens, shifts)
    p = rng.uniform(0, 2 * np.pi, (len(lens), Nc // 2, 2)).astype(np.float32)
    p[~mask] = 0
    m = MeshNetworkGPU(Nc, len(lens), lens, shifts, p.reshape(-1), None, "mzi", is_phase=False, device=dev)
    x = rng.standard_normal((Bc, Nc)) + 1j * rng.standard_normal((Bc, Nc))
    x = torch.from_numpy((x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.complex64)).to(dev).t()
    out = torch.empty_like(x)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(max(3, args.warmup)):
        m.dot(x, out=out)
    ts = []
    for _ in range(max(5, min(args.steps, 200))):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        m.dot(x, out=out)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = statistics.median(ts)
    U = m.matrix().t().to(torch.complex128)
    unit_err = float(torch.linalg.norm(U @ U.conj().t() - torch.eye(Nc, dtype=torch.complex128, device=dev)))
    n_mzi = int(mask.sum())
    print(json.dumps({"metric": "MZI-apps/s (fwd)", "value": n_mzi * Bc / t, "unit": "MZI-apps/s", "n_gpus": 1,
                      "steps": len(ts), "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
                      "config": {"workload": "clements_mzi_N64_L64_B1024_fwd", "n_mzi": n_mzi,
                                 "l2": "flushed between timed calls"},
                      "unitarity_error": unit_err, "status": m.status()}))


def run_c4(args):
    """Unitary fitting: Clements mzi N=128 L=128 with splitting errors N(0, 0.02), target a Haar-random
    unitary (QR of a complex Gaussian with the R-diagonal phase fix), x = I, J = ||U - U_t||_F^2,
    2000 Adam steps (lr 1e-2) on theta, phi through the autograd function; steps/s and the fidelity
    |tr(U^H U_t)|^2 / N^2 reached.  The headline runs the step as a CUDA graph (GraphedStep: captured
    once, replayed); the same 2000 steps run eagerly beside it, from the same start, with the same
    device-side Adam, and must end at the same loss."""
    import torch
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300 import geometry as gm
    from meshes_gb300.autograd import GraphedStep, mesh_apply
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(1004)
    Nc = 128
    lens, shifts = gm.clements(Nc)
    mask = gm.active_mask_nn(Nc, lens, shifts)
    p0 = rng.uniform(0, 2 * np.pi, (len(lens), Nc // 2, 2)).astype(np.float32)
    s0 = rng.normal(0, 0.02, (len(lens), Nc // 2, 2)).astype(np.float32)
    p0[~mask] = 0
    s0[~mask] = 0
    m = MeshNetworkGPU(Nc, len(lens), lens, shifts, p0.reshape(-1), s0, "mzi", is_phase=False, device=dev)
    Z = (rng.standard_normal((Nc, Nc)) + 1j * rng.standard_normal((Nc, Nc))) / np.sqrt(2)
    Q, R = np.linalg.qr(Z)
    Ut = (Q * (np.diag(R) / np.abs(np.diag(R)))[None, :]).astype(np.complex64)
    x = torch.eye(Nc, dtype=torch.complex64, device=dev)
    target = torch.tensor(Ut.T, device=dev)
    n_steps = 2000

    def trainer():
        p = torch.tensor(p0, device=dev, requires_grad=True)
        opt = torch.optim.Adam([p], lr=1e-2, capturable=True)

        def step():
            opt.zero_grad(set_to_none=True)
            loss = ((mesh_apply(m, x, p) - target).abs() ** 2).sum()
            loss.backward()
            opt.step()
            return loss
        return p, step

    # eager: every step from Python
    p_e, step_e = trainer()
    first = float(step_e().detach())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n_steps - 1):
        loss_e = step_e()
    torch.cuda.synchronize()
    t_eager = (time.perf_counter() - t0) / (n_steps - 1)
    # graphed: 3 warm-up steps and the capture, then replays
    p, step = trainer()
    warm = 3
    graphed = GraphedStep(step, warmup=warm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n_steps - warm):
        loss = graphed()
    torch.cuda.synchronize()
    t = (time.perf_counter() - t0) / (n_steps - warm)
    with torch.no_grad():
        U = mesh_apply(m, x, p).t().to(torch.complex128)
        fid = float(torch.abs(torch.trace(U.conj().t() @ torch.tensor(Ut, dtype=torch.complex128, device=dev))) ** 2
                    / Nc ** 2)
    print(json.dumps({"metric": "Adam steps/s (unitary fitting)", "value": 1.0 / t, "unit": "steps/s", "n_gpus": 1,
                      "steps": n_steps, "warmup": warm, "ms_per_step": t * 1e3, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded)",
                      "config": {"workload": "clements_mzi_N128_L128_haar_fit_2000_adam", "lr": 1e-2},
                      "loss_first": first, "loss_last": float(loss.detach()), "fidelity": fid,
                      "eager": {"steps_per_s": 1.0 / t_eager, "ms_per_step": t_eager * 1e3,
                                "loss_last": float(loss_e.detach()),
                                "same_phases": bool(torch.equal(p.detach(), p_e.detach()))},
                      "timing": "host wall clock per optimisation step (fwd + bwd + Adam), device synchronised; "
                                "headline: CUDA-graph replay of the whole step"}))


def run_lossy(args):
    """Lossy generic MZIs (phase errors and gains g_ij; reference crossing.py:444-488) on the Clements
    N=256 L=256 mesh, B=4096: forward + adjoint through LossyMesh (inputs checkpointed per segment,
    each segment recomputed and back-propagated from stored layer inputs), J = sum |y - y_t|^2."""
    import torch
    from meshes_gb300 import geometry as gm
    from meshes_gb300.lossy import LossyMesh
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lens, shifts, p, s, x_h, yt_h, n_mzi = make_problem()
    rng = np.random.default_rng(1006)
    L = len(lens)
    mask = gm.active_mask_nn(N, lens, shifts)
    s14 = np.zeros((L, N // 2, 14))
    s14[..., :2] = s
    s14[..., 2:10] = rng.normal(0, 0.02, (L, N // 2, 8))
    s14[..., 10:] = -np.abs(rng.normal(0.004, 0.002, (L, N // 2, 4)))
    s14[~mask] = 0
    mesh = LossyMesh(N, lens, shifts, device=dev)
    pt = torch.tensor(p, dtype=torch.float64, device=dev, requires_grad=True)
    st = torch.tensor(s14, dtype=torch.float64, device=dev)
    x = torch.from_numpy(x_h).to(dev)
    yt = torch.from_numpy(yt_h).to(dev)

    def step():
        pt.grad = None
        y = mesh(x, mesh.T(pt, st))
        loss = torch.sum(torch.abs(y - yt) ** 2)
        loss.backward()
        return loss

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    k = max(5, min(args.steps, 50))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(k):
        step()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / k
    print(json.dumps({"metric": "MZI-apps/s (fwd+bwd, lossy, checkpointed)", "value": n_mzi * B / t,
                      "unit": "MZI-apps/s", "n_gpus": 1, "steps": k, "warmup": args.warmup, "ms_per_step": t * 1e3,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
                      "data": "synthetic (seeded)",
                      "config": {"workload": "clements_lossy_mzi_N256_L256_B4096_fwd+bwd", "segment": mesh.segment_for(B),
                                 "includes": "T(p) and its phase VJP (library kernels); per segment a forward "
                                             "launch, then a recompute, a stored back-propagation and a reduce"},
                      "status": mesh.status()}))


def run_batched(args):
    """Batched uneven meshes: the one-mesh-per-call drop-in (mg_fwdprop / mg_backdiff per mesh) against
    the persistent multi-mesh launch replayed from a CUDA graph; forward and forward + backward."""
    import torch
    from meshes_gb300 import MeshNetworkGPU, _lib
    from meshes_gb300.batched import BatchedMeshes
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    st = torch.cuda.current_stream().cuda_stream
    prob = make_batched_problem(n_meshes=args.meshes)
    meshes, bufs = [], []
    for d in prob:
        m = MeshNetworkGPU(d["N"], d["L"], d["lens"], d["shifts"], d["p"].reshape(-1), d["s"], d["cr"],
                           is_phase=False, device=dev)
        meshes.append(m)
        x = torch.from_numpy(d["x"]).to(dev)
        nbf = lib.mg_workspace_bytes(0, d["N"], d["L"], d["B"], m.crossing, 0, None)
        nbb = lib.mg_workspace_bytes(2, d["N"], d["L"], d["B"], m.crossing, 0, None)
        wf = torch.empty(nbf, dtype=torch.uint8, device=dev)
        wb = torch.empty(nbb, dtype=torch.uint8, device=dev)
        lib.mg_workspace_init(wf.data_ptr(), nbf, st)
        lib.mg_workspace_init(wb.data_ptr(), nbb, st)
        bufs.append(dict(x=x, y=torch.empty_like(x), g=torch.randn_like(x) if x.is_complex() else torch.randn_like(x),
                         gi=torch.empty_like(x), dp=torch.empty(m.p_phase.numel(), device=dev),
                         wf=(wf, nbf), wb=(wb, nbb)))
    units = sum(d["n_mzi"] * d["B"] for d in prob)

    def plain(backward):
        for d, m, b in zip(prob, meshes, bufs):
            sp = m.p_splitter
            sptr = sp.data_ptr() if sp.numel() else None
            ldp, lds = d["N"] // 2 * m.X_np, d["N"] // 2 * m.X_ns
            _lib.check(lib.mg_fwdprop(d["N"], d["L"], d["B"], m.lens.data_ptr(), m.shifts.data_ptr(),
                                      m.p_phase.data_ptr(), ldp, sptr, lds, b["x"].data_ptr(), b["y"].data_ptr(),
                                      d["N"], m.crossing, b["wf"][0].data_ptr(), b["wf"][1], st), "mg_fwdprop")
            if backward:
                _lib.check(lib.mg_backdiff(d["N"], d["L"], d["B"], m.lens.data_ptr(), m.shifts.data_ptr(),
                                           m.p_phase.data_ptr(), b["dp"].data_ptr(), ldp, sptr, lds,
                                           b["y"].data_ptr(), b["g"].data_ptr(), None, b["gi"].data_ptr(), d["N"],
                                           m.crossing, 0, b["wb"][0].data_ptr(), b["wb"][1], st), "mg_backdiff")

    bm = BatchedMeshes(meshes, [d["B"] for d in prob])
    for stt, b in zip(bm.states, bufs):
        stt.x.copy_(b["x"])
        stt.gy.copy_(b["g"])
    if args.profile:
        # two untimed steps (forward + back-propagation launches) for ncu captures of batched_kernel
        bm.step(True)
        bm.step(True)
        print(json.dumps({"profile_steps": 2, "meshes": len(prob), "items": bm.n_items, "status": bm.check_status()}))
        return
    g_f = BatchedMeshes.capture(bm, backward=False)
    bm2 = bm
    g_fb = torch.cuda.CUDAGraph()
    bm2.step(True)
    torch.cuda.synchronize()
    with torch.cuda.graph(g_fb):
        bm2.step(True)

    def t_of(fn, k):
        for _ in range(max(2, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / k

    k = max(3, min(args.steps, 20))
    t_plain_f = t_of(lambda: plain(False), k)
    t_plain_fb = t_of(lambda: plain(True), k)
    t_bat_f = t_of(g_f.replay, k)
    t_bat_fb = t_of(g_fb.replay, k)
    status = bm.check_status()
    line = {"metric": "MZI-apps/s (batched uneven meshes, fwd+bwd)", "value": units / t_bat_fb, "unit": "MZI-apps/s",
            "n_gpus": 1, "steps": k, "warmup": args.warmup, "ms_per_step": t_bat_fb * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64/f32", "data": "synthetic (seeded)",
            "config": {"workload": "batched_%d_meshes_clements_reck_orth_N8-256_B1-2048" % len(prob), "meshes": len(prob),
                       "mzi_apps_per_pass": units, "items": bm.n_items, "graph": True},
            "batched": {"fwd_mzi_per_s": units / t_bat_f, "fwdbwd_mzi_per_s": units / t_bat_fb,
                        "fwd_ms": t_bat_f * 1e3, "fwdbwd_ms": t_bat_fb * 1e3},
            "plain_one_mesh_per_call": {"fwd_mzi_per_s": units / t_plain_f, "fwdbwd_mzi_per_s": units / t_plain_fb,
                                        "fwd_ms": t_plain_f * 1e3, "fwdbwd_ms": t_plain_fb * 1e3},
            "speedup_batched_vs_plain": {"fwd": t_plain_f / t_bat_f, "fwdbwd": t_plain_fb / t_bat_fb},
            "status": status}
    print(json.dumps(line))


def run_serve(args):
    """Served mixed traffic: 64 resident meshes (Clements / log-depth butterfly, N in {16..512}, splitters
    N(0, 0.02)), Poisson arrivals at 20k req/s, uniform mesh choice, batch log-uniform in [1, 512],
    80% forward / 20% gradient requests; p50/p99 latency from arrival to result and MZI-apps/s."""
    import torch
    from meshes_gb300 import MeshNetworkGPU
    from meshes_gb300 import geometry as gm
    from meshes_gb300.serve import MeshServer
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(1005)
    meshes, pools = [], []
    for i in range(64):
        N = int(rng.choice([16, 32, 64, 128, 256, 512]))
        if i % 2 == 0:
            lens, shifts = gm.clements(N)
            L, strides = len(lens), None
            mask = gm.active_mask_nn(N, lens, shifts)
        else:
            strides = gm.fft(N)
            lens = shifts = None
            L = len(strides)
            mask = np.ones((L, N // 2), bool)
        p = rng.uniform(0, 2 * np.pi, (L, N // 2, 2)).astype(np.float32)
        s = rng.normal(0, 0.02, (L, N // 2, 2)).astype(np.float32)
        p[~mask] = 0
        s[~mask] = 0
        meshes.append(MeshNetworkGPU(N, L, lens, shifts, p.reshape(-1), s, "mzi", is_phase=False, strides=strides,
                                     device=dev))
        x = rng.standard_normal((512, N)) + 1j * rng.standard_normal((512, N))
        pools.append((x / np.linalg.norm(x, axis=1, keepdims=True)).astype(np.complex64))
    srv = MeshServer(meshes, mem_budget=512 << 20)
    # the client loop and the server's scheduler thread share the interpreter: hand the GIL over every
    # 0.2 ms instead of every 5 ms, so neither side waits a whole default interval for the other
    sys.setswitchinterval(2e-4)
    n_mzi = [(sum(m.lens_h) if m.strides is None else m.L * (m.N // 2)) for m in meshes]
    rate, duration = float(args.rate), float(args.duration)
    n_req = int(rate * duration)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    mesh_ids = rng.integers(0, 64, n_req)
    bsz = np.clip(np.round(np.exp(rng.uniform(0, np.log(512), n_req))), 1, 512).astype(int)
    grad = rng.random(n_req) < 0.2
    srv.start()
    # warm-up: one request per mesh
    for i in range(64):
        srv.submit(i, pools[i][:4]).result(60)
    futs = []
    t_submit = 0.0
    # the harness keeps every future and result alive; without this the interpreter's full collections
    # walk hundreds of thousands of them and stall the client and completion threads for ~0.1-0.2 s
    import gc
    gc.disable()
    t0 = time.perf_counter()
    k = 0
    while k < n_req:
        now = time.perf_counter() - t0
        while k < n_req and arrivals[k] <= now:
            i, b = int(mesh_ids[k]), int(bsz[k])
            x = pools[i][:b]
            ts0 = time.perf_counter()
            f = srv.submit(i, x, gy=x if grad[k] else None)
            t_submit += time.perf_counter() - ts0
            futs.append((k, f))
            k += 1
        time.sleep(20e-6)
    for _, f in futs:
        f.result(120)
    t_end = max(f.t_done for _, f in futs)
    gc.enable()
    srv.stop()
    # latency of each request: result available on the host minus its scheduled arrival time
    lat = np.array([f.t_done - (t0 + arrivals[kk]) for kk, f in futs])
    apps = sum(n_mzi[int(mesh_ids[kk])] * int(bsz[kk]) * (2 if grad[kk] else 1) for kk, _ in futs)
    span = t_end - t0
    line = {"metric": "serve p50/p99 latency (ms) and MZI-apps/s", "value": float(np.percentile(lat, 50) * 1e3),
            "unit": "ms (p50 latency)", "n_gpus": 1, "steps": len(futs), "warmup": 64, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded Poisson stream)",
            "config": {"workload": "serve_64_meshes_clements_butterfly_N16-512_%dk_req_s" % round(rate / 1000), "rate_req_s": rate,
                       "duration_s": duration, "requests": len(futs), "grad_fraction": float(grad.mean())},
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "throughput_mzi_apps_per_s": apps / span, "served_req_per_s": len(futs) / span, "ticks": srv.ticks,
            "client_us_per_submit": 1e6 * t_submit / max(len(futs), 1), "scheduler": "native (mg_server)",
            "status": srv.kernel_status()}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--profile", action="store_true", help="two untimed steps only (for ncu captures)")
    ap.add_argument("--workload", default="clements256", choices=["clements256", "batched", "serve", "c1", "c4", "lossy"],
                    help="clements256: the headline fwd+bwd step; batched: 512 uneven meshes, plain vs "
                         "persistent; serve: Poisson request stream on 64 resident meshes; c1: N=64 forward; "
                         "c4: N=128 unitary fitting with Adam; lossy: checkpointed adjoint of lossy MZIs")
    ap.add_argument("--duration", type=float, default=10.0, help="serve workload: seconds of traffic")
    ap.add_argument("--meshes", type=int, default=512, help="batched workload: number of meshes")
    ap.add_argument("--bwd-config", default="", help="with --profile: back-propagation launches with tile "
                                                    "configuration M,V,W,CL,S,split only")
    ap.add_argument("--rate", type=float, default=20000.0, help="serve workload: offered requests per second")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload != "clements256":
        if rank == 0:
            {"batched": run_batched, "serve": run_serve, "c1": run_c1, "c4": run_c4,
             "lossy": run_lossy}[args.workload](args)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
