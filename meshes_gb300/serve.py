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
    dp_bytes: int = 0        # aligned bytes of dJ/dp
    part_bytes: int = 0      # gradient-partial bytes of one work item


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
    host: torch.Tensor            # pinned staging buffer (returned to the pool on retirement)
    outs: tuple                   # result offsets and sizes in `host` (arrays over the tick's requests)


_DESC = np.dtype(mg_batch_mesh)
_ITEM = np.dtype(mg_batch_item)


def _alignv(n):
    return (n + ALIGN - 1) // ALIGN * ALIGN


class _PinnedPool:
    """Reusable pinned host buffers (one per tick in flight), grown on demand."""

    def __init__(self):
        self.free: List[torch.Tensor] = []

    def get(self, n: int) -> torch.Tensor:
        for i, t in enumerate(self.free):
            if t.numel() >= n:
                return self.free.pop(i)
        return torch.empty(max(n, 1 << 20), dtype=torch.uint8, pin_memory=True)

    def put(self, t: torch.Tensor):
        self.free.append(t)
        self.free.sort(key=lambda x: x.numel())


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
        self.host_s = {"pack": 0.0, "retire": 0.0}       # scheduler-thread time spent packing and retiring
        self.error: Optional[BaseException] = None
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.pool = _PinnedPool()
        self._tables()

    def _tables(self):
        """Per-mesh constants as arrays indexed by mesh id (the tick packing is vectorised over requests)."""
        R = self.res

        def col(f):
            return np.array([f(r) for r in R], dtype=np.int64)
        self.t_N, self.t_L = col(lambda r: r.mesh.N), col(lambda r: r.mesh.L)
        self.t_esz = col(lambda r: 4 if r.mesh.X == "orth" else 8)
        self.t_cap, self.t_np2 = col(lambda r: r.cap), col(lambda r: r.np2)
        self.t_cls, self.t_G, self.t_np = col(lambda r: r.cls), col(lambda r: r.G), col(lambda r: r.mesh.X_np)
        self.t_mzi = col(lambda r: r.n_mzi)
        self.t_op = {}
        for op in (OP_FWD, OP_BWD):
            self.t_op[op] = dict(CL=col(lambda r: r.info[op].CL), S=col(lambda r: r.info[op].S),
                                 lb=col(lambda r: r.info[op].layer_bytes),
                                 tiles=col(lambda r: r.ws[op].data_ptr() + r.info[op].off_tiles),
                                 kinds=col(lambda r: r.ws[op].data_ptr() + r.info[op].off_kinds))

    # ---- programming (tiles resident on the device)
    def _program(self, m: MeshNetworkGPU) -> _Resident:
        cls = kernel_class(m)
        M, V = _CLS_MV[cls]
        cfg = {op: _lib.config(M, V, WARPS, 0, 0, 2) for op in (OP_FWD, OP_BWD)}
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
        np2 = G * M // 2
        return _Resident(m, cls, M, V, G, WARPS * (32 // G) * V, np2, info, ws, n_mzi,
                         _align(m.L * (m.N // 2) * m.X_np * 4), m.L * np2 * 8)

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
        b = req.x.shape[0]
        fe = _align(req.x.nbytes)
        if req.gy is None:
            return 2 * fe                                   # x, y
        # x, y, gy, gx, dJ/dp and the gradient partials of its work items
        return 4 * fe + r.dp_bytes + _align((b + r.cap - 1) // r.cap * r.part_bytes)

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
                t0 = time.perf_counter()
                progressed = self._retire()
                if progressed:
                    self.host_s["retire"] += time.perf_counter() - t0
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
            # one copy of the tick's results out of the pinned staging buffer; every result is a view of it
            o_y, n_y, o_dp, n_dp, o_gx, gidx, lo, hi = t.outs
            buf = t.host.numpy()[lo:hi].copy()
            o_y, n_y, o_dp, n_dp, o_gx, gidx = ((a - lo if k in (0, 2, 4) else a).tolist()
                                                for k, a in enumerate((o_y, n_y, o_dp, n_dp, o_gx, gidx)))
            res = [buf[o: o + n].view(q.x.dtype).reshape(q.x.shape) for q, o, n in zip(t.reqs, o_y, n_y)]
            for k, i in enumerate(gidx):                   # gradient requests: (y, dJ/dp, dJ/dx*)
                q = t.reqs[i]
                m = self.res[q.mesh_id].mesh
                dp = buf[o_dp[k]: o_dp[k] + n_dp[k]].view(np.float32).reshape(m.L, m.N // 2, m.X_np)
                gx = buf[o_gx[k]: o_gx[k] + n_y[i]].view(q.x.dtype).reshape(q.x.shape)
                res[i] = (res[i], dp, gx)
            for req, r in zip(t.reqs, res):
                req.t_done = now
                req.future.t_done = now                    # completion time, for latency accounting
                if not req.future.done():
                    req.future.set_result(r)
            self.arena.release(t.dev_off, t.dev_bytes)
            self.pool.put(t.host)
            self.completed += len(t.reqs)
            done = True
        return done

    def _launch_tick(self) -> bool:
        with self.qlock:
            if not self.queue:
                return False
            batch, need = [], 0
            room = self.arena.largest() - 65536            # the tick's descriptors and items get 64 KB + 2 KB/request
            while self.queue and len(batch) < self.max_per_tick:
                req = self.queue[0]
                if req.future.cancelled():
                    self.queue.popleft()
                    continue
                n = need + req.nbytes
                if n + 2048 * (len(batch) + 1) > room:
                    break                                   # no memory now: wait for ticks to retire
                batch.append(self.queue.popleft())
                need = n
        if not batch:
            return False
        t0 = time.perf_counter()
        self._run(batch)
        self.host_s["pack"] += time.perf_counter() - t0
        return True

    def _run(self, reqs: List[Request]):
        """Pack one tick.  Device layout of its arena span (one H2D copy of the first part, one D2H copy of
        the outputs): [descriptors fwd | descriptors bwd | items fwd | items bwd | queue heads | inputs x |
        inputs gy][outputs y | outputs gx | outputs dJ/dp][gradient partials]."""
        lib = self.lib
        K = len(reqs)
        mid = np.fromiter((q.mesh_id for q in reqs), np.int64, K)
        b = np.fromiter((q.x.shape[0] for q in reqs), np.int64, K)
        isg = np.fromiter((q.gy is not None for q in reqs), bool, K)
        gidx = np.flatnonzero(isg)
        KG = len(gidx)
        N, L, esz, cap, np2, n_p = (self.t_N[mid], self.t_L[mid], self.t_esz[mid], self.t_cap[mid], self.t_np2[mid],
                                    self.t_np[mid])
        fe = _alignv(b * N * esz)
        nit = (b + cap - 1) // cap
        dpn = L * (N // 2) * n_p * 4
        # region sizes and per-request offsets inside each region
        def region(sizes):
            o = np.zeros(len(sizes), np.int64)
            if len(sizes) > 1:
                np.cumsum(sizes[:-1], out=o[1:])
            return o, int(sizes.sum())
        o_x, n_x = region(fe)
        o_gy, n_gy = region(fe[gidx])
        o_y, n_y = region(fe)
        o_gx, n_gx = region(fe[gidx])
        o_dp, n_dp = region(_alignv(dpn[gidx]))
        o_pt, n_pt = region(_alignv(nit[gidx] * L[gidx] * np2[gidx] * 8))
        n_if, n_ib = int(nit.sum()), int(nit[gidx].sum())
        off_df = 0
        off_db = off_df + _align(K * _DESC.itemsize)
        off_if = off_db + _align(max(KG, 1) * _DESC.itemsize)
        off_ib = off_if + _align(max(n_if, 1) * _ITEM.itemsize)
        off_head = off_ib + _align(max(n_ib, 1) * _ITEM.itemsize)
        off_x = off_head + ALIGN
        off_gy = off_x + n_x
        in_bytes = off_gy + n_gy                           # host -> device
        off_y = in_bytes
        off_gx = off_y + n_y
        off_dp = off_gx + n_gx
        out_end = off_dp + n_dp                            # device -> host: [off_y, out_end)
        off_pt = out_end
        total = off_pt + n_pt
        base_off = self.arena.alloc(total)
        if base_off is None:                               # raced with fragmentation: put the requests back
            with self.qlock:
                self.queue.extendleft(reversed(reqs))
            return
        base = self.arena.buf.data_ptr() + base_off
        host = self.pool.get(total)
        hv = host.numpy()
        # ---- forward descriptors and items (longest first)
        tf = self.t_op[OP_FWD]
        df = np.zeros(K, _DESC)
        df["N"], df["L"], df["B"], df["ldu"] = N, L, b, N
        df["cls"], df["G"], df["CL"], df["S"] = self.t_cls[mid], self.t_G[mid], tf["CL"][mid], tf["S"][mid]
        df["layer_bytes"], df["n_p"] = tf["lb"][mid], n_p
        df["tiles"], df["kinds"] = tf["tiles"][mid], tf["kinds"][mid]
        df["in0"], df["out0"] = base + off_x + o_x, base + off_y + o_y

        def items(sel, nitems, cost):
            ri = np.repeat(np.arange(len(sel)), nitems)
            k = np.arange(int(nitems.sum())) - np.repeat(np.cumsum(nitems) - nitems, nitems)
            capr, br = cap[sel][ri], b[sel][ri]
            it = np.zeros(len(ri), _ITEM)
            order = np.argsort(-cost[sel][ri], kind="stable")
            it["mesh"], it["v0"] = ri[order], (k * capr)[order]
            it["vend"], it["part"] = np.minimum((k + 1) * capr, br)[order], k[order]
            return it
        cost = L * np2 * cap
        it_f = items(np.arange(K), nit, cost)
        hv[off_df: off_df + df.nbytes] = df.view(np.uint8)
        hv[off_if: off_if + it_f.nbytes] = it_f.view(np.uint8)
        if KG:
            tb = self.t_op[OP_BWD]
            g = gidx
            db = np.zeros(KG, _DESC)
            db["N"], db["L"], db["B"], db["ldu"] = N[g], L[g], b[g], N[g]
            db["cls"], db["G"], db["CL"], db["S"] = self.t_cls[mid[g]], self.t_G[mid[g]], tb["CL"][mid[g]], tb["S"][mid[g]]
            db["layer_bytes"], db["n_items"], db["ldp"], db["n_p"] = tb["lb"][mid[g]], nit[g], N[g] // 2 * n_p[g], n_p[g]
            db["tiles"], db["kinds"] = tb["tiles"][mid[g]], tb["kinds"][mid[g]]
            db["in0"], db["in1"] = base + off_y + o_y[g], base + off_gy + o_gy
            db["out1"], db["dp"], db["partial"] = base + off_gx + o_gx, base + off_dp + o_dp, base + off_pt + o_pt
            it_b = items(g, nit[g], cost)
            hv[off_db: off_db + db.nbytes] = db.view(np.uint8)
            hv[off_ib: off_ib + it_b.nbytes] = it_b.view(np.uint8)
        hv[off_head: off_head + 8] = 0
        # ---- inputs
        for q, o in zip(reqs, o_x):
            xb = q.x.view(np.uint8).reshape(-1)
            hv[off_x + o: off_x + o + xb.size] = xb
        for i, o in zip(gidx, o_gy):
            gb = reqs[i].gy.view(np.uint8).reshape(-1)
            hv[off_gy + o: off_gy + o + gb.size] = gb
        # ---- result spans (host offsets = device offsets within the tick), read back on retirement
        outs = (off_y + o_y, b * N * esz, off_dp + o_dp, dpn[gidx], off_gx + o_gx, gidx, off_y, out_end)
        # ---- enqueue on the next stream
        stream = self.streams[self.next_stream]
        self.next_stream = (self.next_stream + 1) % len(self.streams)
        dev = self.arena.buf[base_off: base_off + total]
        with torch.cuda.stream(stream):
            dev[:in_bytes].copy_(host[:in_bytes], non_blocking=True)
            st = stream.cuda_stream
            head = base + off_head
            check(lib.mg_batched_propagate(OP_FWD, base + off_df, K, base + off_if, n_if, head, self.sms,
                                           self.smem[OP_FWD], self.status.data_ptr(), st), "mg_batched_propagate")
            if KG:
                check(lib.mg_batched_propagate(OP_BWD, base + off_db, KG, base + off_ib, n_ib, head + 4,
                                               self.sms, self.smem[OP_BWD], self.status.data_ptr(), st),
                      "mg_batched_propagate")
                check(lib.mg_batched_reduce(base + off_db, KG, st), "mg_batched_reduce")
            host[off_y:out_end].copy_(dev[off_y:out_end], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        self.mzi_apps += int((self.t_mzi[mid] * b * (1 + isg)).sum())
        self.ticks += 1
        self.inflight.append(_Tick(reqs, ev, base_off, total, host, outs))

    def kernel_status(self) -> int:
        torch.cuda.synchronize(self.device)
        return int(self.status.item())
