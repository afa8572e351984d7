"""Serving: continuous batching of propagate and gradient requests on resident programmed meshes.

``MeshServer(meshes)`` builds every mesh's coefficient tiles once and keeps them on the device.
Clients call ``submit(mesh_id, x)`` (forward: returns y) or ``submit(mesh_id, x, gy=g)`` (gradient:
returns y, dJ/dp and dJ/dx* for the upstream gradient g = 2 dJ/dy*) and get a ``Future``.

The scheduler is native (``mg_server_*`` in libmeshes_gb300, csrc/mg_server.cu): a C++ thread packs
queued requests into ticks, admitting them while their device buffers fit the free part of a fixed
device arena (admission by free device memory).  Each tick makes one host->device copy of the inputs,
descriptors and work items, one persistent forward launch over all admitted requests, one persistent
back-propagation launch and a deterministic gradient reduction for the gradient requests, and one
device->host copy of every result.  Ticks rotate over several streams, so requests that arrive while
others run start as soon as memory frees up (continuous batching).  The Python side only validates a
request, allocates its output arrays, hands their addresses to the scheduler, and completes the futures
from a thread that waits on the scheduler's completion queue (the waits run without the interpreter
lock).  Each request's work items cover only its own vectors, so a request gives the same result alone
and in any mix.
"""
from __future__ import annotations

import atexit
import ctypes
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import OP_BWD, OP_FWD, check, load, mg_server_mesh
from .batched import WARPS, _CLS_MV, kernel_class, plan
from .mesh import MeshNetworkGPU


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


class MeshServer:
    """Continuous-batching request server over resident meshes (native scheduler)."""

    def __init__(self, meshes: Sequence[MeshNetworkGPU], mem_budget: int = 256 << 20, max_requests_per_tick: int = 512,
                 n_streams: int = 2, device=None):
        self.device = torch.device(device) if device is not None else meshes[0].device
        self.lib = load()
        self.res: List[_Resident] = [self._program(m) for m in meshes]
        self.mem_budget = int(mem_budget)
        self.max_per_tick = int(max_requests_per_tick)
        self.n_streams = int(n_streams)
        self.sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.smem = {op: max(r.info[op].smem for r in self.res) for op in (OP_FWD, OP_BWD)}
        self.handle: Optional[int] = None
        self.pending: Dict[int, tuple] = {}               # tag -> (future, inputs kept alive, outputs)
        self.plock = threading.Lock()
        self.tag = 0
        self.waiter: Optional[threading.Thread] = None
        self.error: Optional[BaseException] = None
        self.completed = 0
        self.mzi_apps = 0
        self._final_stats = (0, 0, 0)
        self._final_status = 0

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
        return _Resident(m, cls, M, V, G, WARPS * (32 // G) * V, G * M // 2, info, ws, n_mzi)

    def _descriptors(self):
        arr = (mg_server_mesh * len(self.res))()
        for d, r in zip(arr, self.res):
            m, fi, bi = r.mesh, r.info[OP_FWD], r.info[OP_BWD]
            d.N, d.L, d.cls, d.G, d.n_p, d.cap = m.N, m.L, r.cls, r.G, m.X_np, r.cap
            d.fwd_CL, d.fwd_S, d.bwd_CL, d.bwd_S = fi.CL, fi.S, bi.CL, bi.S
            d.fwd_layer_bytes, d.bwd_layer_bytes = fi.layer_bytes, bi.layer_bytes
            d.fwd_tiles = r.ws[OP_FWD].data_ptr() + fi.off_tiles
            d.fwd_kinds = r.ws[OP_FWD].data_ptr() + fi.off_kinds
            d.bwd_tiles = r.ws[OP_BWD].data_ptr() + bi.off_tiles
            d.bwd_kinds = r.ws[OP_BWD].data_ptr() + bi.off_kinds
        return arr

    # ---- lifecycle
    def start(self):
        torch.cuda.synchronize(self.device)               # tiles built before the scheduler reads them
        h = self.lib.mg_server_create(self._descriptors(), len(self.res), self.mem_budget, self.n_streams,
                                      self.max_per_tick, self.sms, self.smem[OP_FWD], self.smem[OP_BWD],
                                      self.device.index or 0)
        if not h:
            raise ServerError(_lib.last_error())
        self.handle = h
        self.waiter = threading.Thread(target=self._wait_loop, args=(h,), name="mesh-server-completions",
                                       daemon=True)
        self.waiter.start()
        # a server still running at interpreter exit is stopped (its scheduler thread joined) before CUDA
        # tears the context down
        atexit.register(self.stop, False, 5.0)

    def stop(self, drain: bool = True, timeout: float = 60.0):
        """Stop the server; with drain, finish every queued and in-flight request first."""
        h = self.handle
        if h is None:
            return
        if drain:
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < timeout and self.error is None:
                with self.plock:
                    if not self.pending:
                        break
                time.sleep(1e-3)
        self._final_stats = self.stats()
        self._final_status = self.lib.mg_server_status(h)
        with self.plock:
            self.handle = None                             # no submit reaches h after this
        if self.waiter is not None:
            self.waiter.join(timeout)                      # sees handle None within one wait period
        self.lib.mg_server_destroy(h, 1 if drain else 0)  # joins the scheduler thread, frees its memory
        with self.plock:
            left = list(self.pending.values())
            self.pending.clear()
        for fut, _, _ in left:
            if not fut.done():
                fut.set_exception(ServerError("server stopped"))

    # ---- client side
    def submit(self, mesh_id: int, x, gy=None) -> Future:
        """Queue one request; x (b, N) complex64 (float32 for orth meshes), gy the same shape or None."""
        h = self.handle
        if h is None:
            raise ServerError("server not running")
        if not (0 <= mesh_id < len(self.res)):
            raise ServerError("no mesh %d" % mesh_id)
        m = self.res[mesh_id].mesh
        dt = np.float32 if m.X == "orth" else np.complex64
        x = np.ascontiguousarray(x, dtype=dt)
        if x.ndim != 2 or x.shape[1] != m.N or x.shape[0] < 1:
            raise ServerError("request for mesh %d must be (b, %d) with b >= 1, got %s" % (mesh_id, m.N, x.shape))
        y = np.empty_like(x)
        dp = gx = None
        if gy is not None:
            gy = np.ascontiguousarray(gy, dtype=dt)
            if gy.shape != x.shape:
                raise ServerError("gy must have the shape of x")
            dp = np.empty((m.L, m.N // 2, m.X_np), dtype=np.float32)
            gx = np.empty_like(x)
        fut: Future = Future()
        with self.plock:                                   # stop() clears the handle under the same lock
            if self.handle is None:
                raise ServerError("server stopped")
            self.tag += 1
            tag = self.tag
            rc = self.lib.mg_server_submit(self.handle, mesh_id, x.shape[0], x.ctypes.data,
                                           None if gy is None else gy.ctypes.data, y.ctypes.data,
                                           None if dp is None else dp.ctypes.data,
                                           None if gx is None else gx.ctypes.data, tag)
            if rc != 0:
                raise ServerError(_lib.last_error())
            self.pending[tag] = (fut, (x, gy), (y, dp, gx))
            self.mzi_apps += self.res[mesh_id].n_mzi * x.shape[0] * (2 if gy is not None else 1)
        return fut

    def _wait_loop(self, h):
        buf = (ctypes.c_ulonglong * 4096)()
        lib = self.lib
        while self.handle == h:
            n = lib.mg_server_wait(h, buf, 4096, 2000)
            if n < 0:
                self.error = ServerError(_lib.last_error())
                with self.plock:
                    left = list(self.pending.values())
                    self.pending.clear()
                for fut, _, _ in left:
                    if not fut.done():
                        fut.set_exception(self.error)
                return
            if n == 0:
                continue
            now = time.perf_counter()
            with self.plock:
                got = [self.pending.pop(t) for t in buf[:n]]
            for fut, (_, gy), (y, dp, gx) in got:
                fut.t_done = now                            # completion time, for latency accounting
                if fut.set_running_or_notify_cancel():      # a cancelled request's result is dropped
                    fut.set_result(y if gy is None else (y, dp, gx))
            self.completed += n

    # ---- introspection
    def stats(self):
        """(completed requests, ticks, queued requests) of the native scheduler."""
        if self.handle is None:
            return self._final_stats
        out = (ctypes.c_longlong * 3)()
        check(self.lib.mg_server_stats(self.handle, out), "mg_server_stats")
        return tuple(out)

    @property
    def ticks(self) -> int:
        return self.stats()[1]

    def kernel_status(self) -> int:
        if self.handle is None:
            return self._final_status
        return self.lib.mg_server_status(self.handle)
