"""Serving: continuous batching of propagate and gradient requests on resident programmed meshes.

``MeshServer(meshes)`` builds every mesh's coefficient tiles once and keeps them on the device.
Clients call ``submit(mesh_id, x)`` (forward: returns y) or ``submit(mesh_id, x, gy=g)`` (gradient:
returns y, dJ/dp and dJ/dx* for the upstream gradient g = 2 dJ/dy*) and get a ``Future``.

A scheduler thread runs ticks.  Each tick
  * retires finished ticks (CUDA events) and completes their futures, freeing their arena space;
  * admits queued requests, oldest first, while their device buffers fit in the free part of a fixed
    device arena (admission by free device memory) and the tick has slots left;
  * packs them into one tick: one host->device copy of every input and of the per-request
    descriptors and work items, one persistent forward launch over all admitted requests, one
    persistent back-propagation launch plus a deterministic gradient reduction for the gradient
    requests, one device->host copy of every result, and an event;
  * rotates over several streams, so a tick starts while earlier ticks are still on the GPU:
    requests that arrive while others run are admitted as soon as memory and slots free up, and
    their work overlaps on the device.
Each request's result depends only on its own mesh and inputs (its work items cover only its own
vectors), so a request gives the same result alone and in any mix.
"""
from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import OP_BWD, OP_FWD, check, load, mg_batch_item, mg_batch_mesh
from .batched import WARPS, _CLS_MV, kernel_class, plan
from .mesh import MeshNetworkGPU

ALIGN = 256


def _align(n: int) -> int:
    return (n + ALIGN - 1) // ALIGN * ALIGN


class ServerError(RuntimeError):
    pass


@dataclass
class _Resident:
    mesh: MeshNetworkGPU
    cls: int
    M: int
    V: int
    G: int
    cap: int
    np2: int
    info: dict
    ws: dict
    n_mzi: int


@dataclass
class Request:
    rid: int
    mesh_id: int
    x: np.ndarray
    gy: Optional[np.ndarray]
    t_submit: float
    future: Future = field(default_factory=Future)
    nbytes: int = 0
    t_done: float = 0.0


@dataclass
class _Tick:
    reqs: List[Request]
    event: torch.cuda.Event
    dev_off: int
    dev_bytes: int
    host: torch.Tensor
    out_spans: list


class _Arena:
    """First-fit allocator over one device buffer (the memory admission budget)."""

    def __init__(self, nbytes: int, device):
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=device)
        self.size = nbytes
        self.free = [(0, nbytes)]                       # sorted (offset, length)

    def alloc(self, n: int) -> Optional[int]:
        n = _align(n)
        for i, (o, ln) in enumerate(self.free):
            if ln >= n:
                if ln == n:
                    self.free.pop(i)
                else:
                    self.free[i] = (o + n, ln - n)
                return o
        return None

    def release(self, o: int, n: int):
        n = _align(n)
        self.free.append((o, n))
        self.free.sort()
        merged = []
        for fo, fl in self.free:
            if merged and merged[-1][0] + merged[-1][1] == fo:
                merged[-1] = (merged[-1][0], merged[-1][1] + fl)
            else:
                merged.append((fo, fl))
        self.free = merged

    def largest(self) -> int:
        return max((ln for _, ln in self.free), default=0)


class MeshServer:
    """Continuous-batching request loop over resident meshes."""

    def __init__(self, meshes: Sequence[MeshNetworkGPU], mem_budget: int = 256 << 20, max_requests_per_tick: int = 512,
                 n_streams: int = 2, device=None, idle_sleep: float = 50e-6):
        self.device = torch.device(device) if device is not None else meshes[0].device
        self.lib = load()
        self.res: List[_Resident] = [self._program(m) for m in meshes]
        self.arena = _Arena(mem_budget, self.device)
        self.max_per_tick = max_requests_per_tick
        self.streams = [torch.cuda.Stream(self.device) for _ in range(n_streams)]
        self.sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.smem = {op: max(r.info[op].smem for r in self.res) for op in (OP_FWD, OP_BWD)}
        self.queue: deque = deque()
        self.qlock = threading.Lock()
        self.inflight: deque = deque()
        self.next_stream = 0
        self.rid = 0
        self.running = False
        self.thread: Optional[threading.Thread] = None
        self.idle_sleep = idle_sleep
        self.completed = 0
        self.mzi_apps = 0
        self.ticks = 0
        self.error: Optional[BaseException] = None
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)

    # ---- programming (tiles resident on the device)
    def _program(self, m: MeshNetworkGPU) -> _Resident:
        cls = kernel_class(m)
        M, V = _CLS_MV[cls]
        cfg = {op: _lib.config(M, V, WARPS, 0, 0) for op in (OP_FWD, OP_BWD)}
        info = {op: plan(op, m.N, m.L, 1, m.crossing, m.geometry, cfg[op]) for op in (OP_FWD, OP_BWD)}
        ws = {}
        st = torch.cuda.current_stream(m.device).cuda_stream
        geo = ((None, None, m.strides.data_ptr()) if m.strides is not None else (m.lens.data_ptr(), m.shifts.data_ptr(), None))
        s = m.p_splitter
        for op in (OP_FWD, OP_BWD):
            ws[op] = torch.empty(info[op].total, dtype=torch.uint8, device=m.device)
            check(self.lib.mg_workspace_init(ws[op].data_ptr(), ws[op].numel(), st), "mg_workspace_init")
            check(self.lib.mg_build_tiles(op, m.N, m.L, m.geometry, *geo, m.crossing, m.p_phase.data_ptr(),
                                          m.N // 2 * m.X_np, s.data_ptr() if s.numel() else None, m.N // 2 * m.X_ns,
                                          None, None, None, 1, _lib.cfg_ptr(cfg[op]), ws[op].data_ptr(),
                                          ws[op].numel(), st), "mg_build_tiles")
        G = info[OP_FWD].G
        n_mzi = sum(m.lens_h) if m.strides is None else m.L * (m.N // 2)
        return _Resident(m, cls, M, V, G, WARPS * (32 // G) * V, G * M // 2, info, ws, n_mzi)

    # ---- client side
    def submit(self, mesh_id: int, x, gy=None) -> Future:
        """Queue one request; x (b, N) complex64 (float32 for orth meshes), gy the same shape or None."""
        if not (0 <= mesh_id < len(self.res)):
            raise ServerError("no mesh %d" % mesh_id)
        r = self.res[mesh_id]
        m = r.mesh
        dt = np.float32 if m.X == "orth" else np.complex64
        x = np.ascontiguousarray(np.asarray(x, dtype=dt))
        if x.ndim != 2 or x.shape[1] != m.N or x.shape[0] < 1:
            raise ServerError("request for mesh %d must be (b, %d) with b >= 1, got %s" % (mesh_id, m.N, x.shape))
        if gy is not None:
            gy = np.ascontiguousarray(np.asarray(gy, dtype=dt))
            if gy.shape != x.shape:
                raise ServerError("gy must have the shape of x")
        with self.qlock:
            self.rid += 1
            req = Request(self.rid, mesh_id, x, gy, time.perf_counter())
            req.nbytes = self._request_bytes(req)
            if req.nbytes > self.arena.size:
                raise ServerError("request needs %d bytes, above the %d-byte arena" % (req.nbytes, self.arena.size))
            self.queue.append(req)
        return req.future

    def _request_bytes(self, req: Request) -> int:
        r = self.res[req.mesh_id]
        b, N = req.x.shape
        e = req.x.itemsize
        n = 2 * _align(b * N * e)                           # x, y
        if req.gy is not None:
            n_items = (b + r.cap - 1) // r.cap
            n += 2 * _align(b * N * e)                      # gy, gx
            n += _align(r.mesh.L * (N // 2) * r.mesh.X_np * 4)               # dp
            n += _align(n_items * r.mesh.L * r.np2 * 8)     # partials
        return n

    # ---- scheduler
    def start(self):
        self.running = True
        self.thread = threading.Thread(target=self._loop, name="mesh-server", daemon=True)
        self.thread.start()

    def stop(self, drain: bool = True, timeout: float = 60.0):
        """Stop the loop; with drain, finish every queued and in-flight request first."""
        if drain:
            t0 = time.perf_counter()
            while True:
                with self.qlock:
                    busy = bool(self.queue) or bool(self.inflight)
                if not busy or self.error is not None or time.perf_counter() - t0 > timeout:
                    break
                time.sleep(1e-3)
        self.running = False
        if self.thread is not None:
            self.thread.join(timeout)
        with self.qlock:
            pending = list(self.queue)
            self.queue.clear()
        for req in pending:
            if not req.future.done():
                req.future.set_exception(ServerError("server stopped"))

    def _loop(self):
        try:
            torch.cuda.set_device(self.device)
            while self.running:
                progressed = self._retire()
                progressed |= self._launch_tick()
                if not progressed:
                    time.sleep(self.idle_sleep)
            while self.inflight:
                self.inflight[0].event.synchronize()
                self._retire()
        except BaseException as e:   # surface loop failures to every waiting client
            self.error = e
            with self.qlock:
                pending = list(self.queue)
                self.queue.clear()
            for t in list(self.inflight):
                pending += t.reqs
            for req in pending:
                if not req.future.done():
                    req.future.set_exception(e)

    def _retire(self) -> bool:
        done = False
        while self.inflight and self.inflight[0].event.query():
            t = self.inflight.popleft()
            now = time.perf_counter()
            host = t.host
            for req, spans in zip(t.reqs, t.out_spans):
                outs = []
                for (off, nbytes, shape, dtype) in spans:
                    a = host[off: off + nbytes].numpy().view(dtype).reshape(shape).copy()
                    outs.append(a)
                req.t_done = now
                req.future.t_done = now                    # completion time, for latency accounting
                if not req.future.done():
                    req.future.set_result(outs[0] if req.gy is None else tuple(outs))
            self.arena.release(t.dev_off, t.dev_bytes)
            self.completed += len(t.reqs)
            done = True
        return done

    def _launch_tick(self) -> bool:
        with self.qlock:
            if not self.queue:
                return False
            batch, need = [], 0
            while self.queue and len(batch) < self.max_per_tick:
                req = self.queue[0]
                if req.future.cancelled():
                    self.queue.popleft()
                    continue
                n = need + req.nbytes
                if n + 65536 + 64 * (len(batch) + 1) * 32 > self.arena.largest():
                    break                                   # no memory now: wait for ticks to retire
                batch.append(self.queue.popleft())
                need = n
        if not batch:
            return False
        self._run(batch)
        return True

    def _run(self, reqs: List[Request]):
        lib = self.lib
        # ---- device layout: [per-request buffers][descriptors fwd][descriptors bwd][items fwd][items bwd][head]
        items_f, items_b = [], []
        desc_f = (mg_batch_mesh * len(reqs))()
        grads = [i for i, q in enumerate(reqs) if q.gy is not None]
        desc_b = (mg_batch_mesh * max(len(grads), 1))()
        layout = []                                        # per request: dict of offsets
        off = 0
        for q in reqs:
            r = self.res[q.mesh_id]
            b, N = q.x.shape
            fe = _align(b * N * q.x.itemsize)
            d = {"x": off, "y": off + fe}
            off += 2 * fe
            if q.gy is not None:
                n_items = (b + r.cap - 1) // r.cap
                d["gy"], d["gx"] = off, off + fe
                off += 2 * fe
                d["dp"] = off
                off += _align(r.mesh.L * (N // 2) * r.mesh.X_np * 4)
                d["part"] = off
                off += _align(n_items * r.mesh.L * r.np2 * 8)
            layout.append(d)
        data_bytes = off
        off_df = data_bytes
        off_db = off_df + _align(ctypes.sizeof(desc_f))
        n_if = sum((q.x.shape[0] + self.res[q.mesh_id].cap - 1) // self.res[q.mesh_id].cap for q in reqs)
        n_ib = sum((reqs[i].x.shape[0] + self.res[reqs[i].mesh_id].cap - 1) // self.res[reqs[i].mesh_id].cap
                   for i in grads)
        off_if = off_db + _align(ctypes.sizeof(desc_b))
        off_ib = off_if + _align(max(n_if, 1) * 16)
        off_head = off_ib + _align(max(n_ib, 1) * 16)
        total = off_head + ALIGN
        base_off = self.arena.alloc(total)
        if base_off is None:                               # raced with fragmentation: put the requests back
            with self.qlock:
                self.queue.extendleft(reversed(reqs))
            return
        base = self.arena.buf.data_ptr() + base_off
        # ---- descriptors and items (longest first)
        fl = []
        for i, (q, d) in enumerate(zip(reqs, layout)):
            r = self.res[q.mesh_id]
            m, info = r.mesh, r.info[OP_FWD]
            b = q.x.shape[0]
            ds = desc_f[i]
            ds.N, ds.L, ds.B, ds.ldu = m.N, m.L, b, m.N
            ds.cls, ds.G, ds.CL, ds.S = r.cls, info.G, info.CL, info.S
            ds.layer_bytes, ds.n_items, ds.ldp, ds.n_p = info.layer_bytes, 0, 0, m.X_np
            ds.tiles = r.ws[OP_FWD].data_ptr() + info.off_tiles
            ds.kinds = r.ws[OP_FWD].data_ptr() + info.off_kinds
            ds.in0, ds.out0 = base + d["x"], base + d["y"]
            for k in range(0, b, r.cap):
                fl.append((m.L * r.np2 * r.cap, i, k, min(k + r.cap, b), k // r.cap))
        fl.sort(key=lambda t: -t[0])
        it_f = (mg_batch_item * max(n_if, 1))()
        for n, (_, i, v0, v1, part) in enumerate(fl):
            it_f[n].mesh, it_f[n].v0, it_f[n].vend, it_f[n].part = i, v0, v1, part
        bl = []
        for j, i in enumerate(grads):
            q, d = reqs[i], layout[i]
            r = self.res[q.mesh_id]
            m, info = r.mesh, r.info[OP_BWD]
            b = q.x.shape[0]
            ds = desc_b[j]
            ds.N, ds.L, ds.B, ds.ldu = m.N, m.L, b, m.N
            ds.cls, ds.G, ds.CL, ds.S = r.cls, info.G, info.CL, info.S
            ds.layer_bytes, ds.n_items = info.layer_bytes, (b + r.cap - 1) // r.cap
            ds.ldp, ds.n_p = m.N // 2 * m.X_np, m.X_np
            ds.tiles = r.ws[OP_BWD].data_ptr() + info.off_tiles
            ds.kinds = r.ws[OP_BWD].data_ptr() + info.off_kinds
            ds.in0, ds.in1, ds.out0, ds.out1 = base + d["y"], base + d["gy"], None, base + d["gx"]
            ds.dp, ds.partial = base + d["dp"], base + d["part"]
            for k in range(0, b, r.cap):
                bl.append((m.L * r.np2 * r.cap, j, k, min(k + r.cap, b), k // r.cap))
        bl.sort(key=lambda t: -t[0])
        it_b = (mg_batch_item * max(n_ib, 1))()
        for n, (_, j, v0, v1, part) in enumerate(bl):
            it_b[n].mesh, it_b[n].v0, it_b[n].vend, it_b[n].part = j, v0, v1, part
        # ---- host staging: inputs + descriptors + items, then room for the outputs
        host = torch.empty(total, dtype=torch.uint8).pin_memory()
        hv = host.numpy()
        for q, d in zip(reqs, layout):
            xb = q.x.view(np.uint8).reshape(-1)
            hv[d["x"]: d["x"] + xb.size] = xb
            if q.gy is not None:
                gb = q.gy.view(np.uint8).reshape(-1)
                hv[d["gy"]: d["gy"] + gb.size] = gb
        for (o, st) in ((off_df, desc_f), (off_db, desc_b), (off_if, it_f), (off_ib, it_b)):
            raw = np.frombuffer(bytes(st), dtype=np.uint8)
            hv[o: o + raw.size] = raw
        hv[off_head: off_head + 8] = 0
        stream = self.streams[self.next_stream]
        self.next_stream = (self.next_stream + 1) % len(self.streams)
        dev = self.arena.buf[base_off: base_off + total]
        out_spans = []
        with torch.cuda.stream(stream):
            dev.copy_(host, non_blocking=True)
            st = stream.cuda_stream
            head = base + off_head
            check(lib.mg_batched_propagate(OP_FWD, base + off_df, len(reqs), base + off_if, n_if, head, self.sms,
                                           self.smem[OP_FWD], self.status.data_ptr(), st), "mg_batched_propagate")
            if grads:
                check(lib.mg_batched_propagate(OP_BWD, base + off_db, len(grads), base + off_ib, n_ib, head + 4,
                                               self.sms, self.smem[OP_BWD], self.status.data_ptr(), st),
                      "mg_batched_propagate")
                check(lib.mg_batched_reduce(base + off_db, len(grads), st), "mg_batched_reduce")
            # results back: y for every request, (dp, gx) for gradient requests
            for q, d in zip(reqs, layout):
                r = self.res[q.mesh_id]
                b, N = q.x.shape
                fe = b * N * q.x.itemsize
                spans = [(d["y"], fe, (b, N), q.x.dtype)]
                if q.gy is not None:
                    dpn = r.mesh.L * (N // 2) * r.mesh.X_np * 4
                    spans += [(d["dp"], dpn, (r.mesh.L, N // 2, r.mesh.X_np), np.float32), (d["gx"], fe, (b, N), q.x.dtype)]
                for (o, n, _, _) in spans:
                    host[o: o + n].copy_(dev[o: o + n], non_blocking=True)
                out_spans.append(spans)
            ev = torch.cuda.Event()
            ev.record(stream)
        for q in reqs:
            self.mzi_apps += self.res[q.mesh_id].n_mzi * q.x.shape[0] * (2 if q.gy is not None else 1)
        self.ticks += 1
        self.inflight.append(_Tick(reqs, ev, base_off, total, host, out_spans))

    def kernel_status(self) -> int:
        torch.cuda.synchronize(self.device)
        return int(self.status.item())
