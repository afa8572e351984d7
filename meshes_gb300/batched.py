"""Batched meshes: many independent meshes of uneven size and depth in one persistent launch.

``BatchedMeshes(meshes)`` keeps every mesh's coefficient tiles resident (built once, rebuilt by
``update_phases``), owns device buffers for each mesh's batch, and propagates all of them with one
``mg_batched_propagate`` launch: a (mesh, batch-tile) work queue drained by one CTA per SM, items
sorted longest-first.  Forward and back-propagation (``backward`` also returns dJ/dp of every mesh,
reduced deterministically by ``mg_batched_reduce``).  ``capture()`` records the launches of one
composition in a CUDA graph; ``replay()`` re-runs it (inputs are read from, and outputs written to,
the engine's own buffers ``x[i]``, ``y[i]``, ``gy[i]``, ``gx[i]``, ``dp[i]``).
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import torch

from . import _lib
from ._lib import BATCH_NN, GEO_NN, OP_BWD, OP_FWD, check, load, mg_batch_item, mg_batch_mesh, mg_plan_info
from .mesh import MeshNetworkGPU, _stream

BCLS_C8, BCLS_C16, BCLS_R8 = 0, 1, 2
MG_BATCH_FULL_WARP = 32


def MG_BATCH_ONLY(cls: int) -> int:
    """Flag of mg_batched_propagate: every item of the launch is of kernel class cls."""
    return (cls + 1) << 8
_CLS_MV = {BCLS_C8: (8, 4), BCLS_C16: (16, 2), BCLS_R8: (8, 4)}
WARPS = 8


def _bind():
    return load()


def plan(op, N, L, B, crossing, geometry, cfg=None) -> mg_plan_info:
    lib = _bind()
    out = mg_plan_info()
    check(lib.mg_plan(op, N, L, B, crossing, geometry, _lib.cfg_ptr(cfg), ctypes.byref(out)), "mg_plan")
    return out


def kernel_class(mesh: MeshNetworkGPU) -> int:
    if getattr(mesh, "perm_table", None) is not None:
        raise ValueError("batched meshes take no permutations between layers")
    if mesh.X == "orth":
        if mesh.N > 256:
            raise ValueError("orth meshes in a batch are limited to N <= 256")
        return BCLS_R8
    if mesh.X != "mzi":
        raise ValueError("batched meshes support the mzi and orth crossings")
    return BCLS_C8 if mesh.N <= 256 else BCLS_C16


def _to_device(structs, device) -> torch.Tensor:
    raw = bytes(structs)
    return torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(device)


class _MeshState:
    def __init__(self, mesh: MeshNetworkGPU, B: int):
        self.mesh, self.B = mesh, int(B)
        self.cls = kernel_class(mesh)
        M, V = _CLS_MV[self.cls]
        self.M, self.V = M, V
        self.cfg = {op: _lib.config(M, V, WARPS, 0, 0, 2) for op in (OP_FWD, OP_BWD)}
        self.info = {op: plan(op, mesh.N, mesh.L, max(self.B, 1), mesh.crossing, mesh.geometry, self.cfg[op])
                     for op in (OP_FWD, OP_BWD)}
        self.ws = {}
        for op in (OP_FWD, OP_BWD):
            self.ws[op] = torch.empty(self.info[op].total, dtype=torch.uint8, device=mesh.device)
            check(load().mg_workspace_init(self.ws[op].data_ptr(), self.ws[op].numel(), _stream(mesh.device)),
                  "mg_workspace_init")
        G = self.info[OP_FWD].G
        self.G = G
        self.np2 = G * M // 2
        self.cap = WARPS * (32 // G) * V                  # vectors per work item
        self.n_items = (self.B + self.cap - 1) // self.cap
        dev, N = mesh.device, mesh.N
        self.x = torch.zeros((self.B, N), dtype=mesh.dtype, device=dev)
        self.y = torch.zeros_like(self.x)
        self.gy = torch.zeros_like(self.x)
        self.gx = torch.zeros_like(self.x)
        self.dp = torch.zeros((mesh.L, N // 2, mesh.X_np), dtype=torch.float32, device=dev)
        self.partial = torch.empty(max(self.n_items, 1) * mesh.L * self.np2 * 2, dtype=torch.float32, device=dev)
        self.build_tiles()

    def build_tiles(self, p: Optional[torch.Tensor] = None):
        m = self.mesh
        p = m.p_phase if p is None else p
        s = m.p_splitter
        geo = ((None, None, m.strides.data_ptr()) if m.strides is not None else (m.lens.data_ptr(), m.shifts.data_ptr(), None))
        for op in (OP_FWD, OP_BWD):
            check(load().mg_build_tiles(op, m.N, m.L, m.geometry, *geo, m.crossing, p.data_ptr(), m.N // 2 * m.X_np,
                                        s.data_ptr() if s.numel() else None, m.N // 2 * m.X_ns, None, None, None,
                                        max(self.B, 1), _lib.cfg_ptr(self.cfg[op]), self.ws[op].data_ptr(),
                                        self.ws[op].numel(), _stream(m.device)), "mg_build_tiles")

    def descriptor(self, op) -> mg_batch_mesh:
        m, info, ws = self.mesh, self.info[op], self.ws[op]
        d = mg_batch_mesh()
        d.N, d.L, d.B, d.ldu = m.N, m.L, self.B, m.N
        d.cls, d.G, d.CL, d.S = self.cls, info.G, info.CL, info.S
        d.layer_bytes, d.n_items, d.ldp, d.n_p = info.layer_bytes, self.n_items, m.N // 2 * m.X_np, m.X_np
        d.tiles = ws.data_ptr() + info.off_tiles
        d.kinds = ws.data_ptr() + info.off_kinds
        if op == OP_FWD:
            d.in0, d.in1, d.out0, d.out1 = self.x.data_ptr(), None, self.y.data_ptr(), None
            d.dp, d.partial = None, None
        else:
            d.in0, d.in1, d.out0, d.out1 = self.y.data_ptr(), self.gy.data_ptr(), None, self.gx.data_ptr()
            d.dp, d.partial = self.dp.data_ptr(), self.partial.data_ptr()
        return d

    def cost(self) -> int:
        """Padded work of one full item: layers x slots x vector capacity."""
        return self.mesh.L * self.np2 * self.cap


class BatchedMeshes:
    """A fixed composition of meshes and batch sizes, propagated by one persistent launch per op."""

    def __init__(self, meshes: Sequence[MeshNetworkGPU], batch_sizes: Sequence[int], grid: Optional[int] = None,
                 full_warp: bool = True):
        if len(meshes) != len(batch_sizes):
            raise ValueError("one batch size per mesh")
        self.device = meshes[0].device
        self.states: List[_MeshState] = [_MeshState(m, b) for m, b in zip(meshes, batch_sizes)]
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        self.grid = grid or sms
        # launch groups: with full_warp (the default) and every mesh nearest-neighbour (MG_BATCH_NN), the M = 8
        # meshes whose vector fills the warp (G = 32; complex, and real ones in a second group) run in launches
        # of their own with a compile-time lane group, issued first; everything else runs in one launch of the
        # three-class kernel on a side stream, whose CTAs take the SMs as the earlier launches' CTAs finish.  Measured on GB300 on 512 uneven meshes
        # (N 8..256): fwd+bwd 318 against 301 G MZI-apps/s for a single launch, dJ/dp bitwise the same.  Each
        # group is sorted longest-first and drained from its own counter.
        self.nn = BATCH_NN if all(st.mesh.geometry == GEO_NN for st in self.states) else 0
        groups = {}
        for i, st in enumerate(self.states):
            full = full_warp and bool(self.nn) and st.cls in (BCLS_C8, BCLS_R8) and st.G == 32
            flags = (MG_BATCH_ONLY(st.cls) | MG_BATCH_FULL_WARP) if full else 0
            for k in range(st.n_items):
                v0 = k * st.cap
                groups.setdefault(flags, []).append((st.cost(), i, v0, min(v0 + st.cap, st.B), k))
        self.groups = []
        # the full-warp groups first, the largest total work first; the mixed launch (short items) last
        order = sorted(groups.items(), key=lambda kv: (kv[0] == 0, -sum(t[0] for t in kv[1])))
        for flags, items in order:
            items.sort(key=lambda t: -t[0])               # longest processing time first
            arr = (mg_batch_item * max(len(items), 1))()
            for n, (_, i, v0, v1, k) in enumerate(items):
                arr[n].mesh, arr[n].v0, arr[n].vend, arr[n].part = i, v0, v1, k
            self.groups.append((flags, len(items), _to_device(arr, self.device)))
        self.n_items = sum(g[1] for g in self.groups)
        self.desc = {}
        self.smem = {}
        for op in (OP_FWD, OP_BWD):
            ds = (mg_batch_mesh * len(self.states))()
            for i, st in enumerate(self.states):
                ds[i] = st.descriptor(op)
            self.desc[op] = _to_device(ds, self.device)
            self.smem[op] = max(st.info[op].smem for st in self.states)
        self.head = torch.zeros(max(len(self.groups), 1), dtype=torch.int32, device=self.device)
        self.side = None
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.graph = None

    # ---- data movement
    @property
    def x(self):
        return [s.x for s in self.states]

    @property
    def y(self):
        return [s.y for s in self.states]

    @property
    def gy(self):
        return [s.gy for s in self.states]

    @property
    def gx(self):
        return [s.gx for s in self.states]

    @property
    def dp(self):
        return [s.dp for s in self.states]

    def update_phases(self, ps: Sequence[torch.Tensor]):
        for st, p in zip(self.states, ps):
            st.build_tiles(p.contiguous().float())

    # ---- launches (all on the current stream)
    def _launch(self, op):
        lib = _bind()
        stream = _stream(self.device)
        self.head.zero_()
        main = torch.cuda.current_stream(self.device)
        # the groups' persistent launches run concurrently (the first on the current stream, the others on side
        # streams joined back with events), so the CTAs of one fill the SMs the other's tail leaves idle
        if len(self.groups) > 1:
            if self.side is None:
                self.side = [torch.cuda.Stream(self.device) for _ in self.groups[1:]]
            fork = torch.cuda.Event()
            fork.record(main)
            for sd in self.side:
                sd.wait_event(fork)
        for g, (flags, n, items) in enumerate(self.groups):
            s_g = stream if g == 0 else self.side[g - 1].cuda_stream
            # all meshes nearest-neighbour: the kernel bodies without strided layers (MG_BATCH_NN)
            check(lib.mg_batched_propagate(op | self.nn | flags, self.desc[op].data_ptr(), len(self.states),
                                           items.data_ptr(), n, self.head[g:].data_ptr(), self.grid, self.smem[op],
                                           self.status.data_ptr(), s_g), "mg_batched_propagate")
        if len(self.groups) > 1:
            for sd in self.side:
                join = torch.cuda.Event()
                join.record(sd)
                main.wait_event(join)
        if op == OP_BWD:
            check(lib.mg_batched_reduce(self.desc[op].data_ptr(), len(self.states), stream), "mg_batched_reduce")

    def forward(self):
        """y[i] = U_i x[i] for every mesh, one launch."""
        self._launch(OP_FWD)
        return self.y

    def backward(self):
        """From y[i] and gy[i] (2 dJ/dy*): gx[i] = U_i^H gy[i] and dp[i] = dJ/dp_i, one launch + reduce."""
        self._launch(OP_BWD)
        return self.gx, self.dp

    def step(self, backward: bool = True):
        self.forward()
        if backward:
            self.backward()

    def capture(self, backward: bool = True):
        """Record one step (forward, optionally backward) in a CUDA graph."""
        self.step(backward)                                # warm-up (sets kernel attributes)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step(backward)
        self.graph = g
        return g

    def replay(self):
        self.graph.replay()

    def check_status(self) -> int:
        torch.cuda.synchronize(self.device)
        return int(self.status.item())

    def mzi_apps(self) -> int:
        """MZI applications of one forward pass (actual MZIs x batch)."""
        total = 0
        for st in self.states:
            m = st.mesh
            n_mzi = (sum(m.lens_h) if m.strides is None else m.L * (m.N // 2))
            total += n_mzi * st.B
        return total
