"""torch.autograd integration: y = U(p) x through the sm_103a kernels.

``mesh_apply(mesh, x, p)`` propagates a batch ``x`` (B, N) (rows are vectors, complex64; float32 for
orth meshes) through ``mesh`` (a MeshNetworkGPU giving the geometry, the crossing and the splitter
errors) with phases ``p`` (L, N/2, n_p) and returns y (B, N).  Gradients flow to x and p.

Complex convention: PyTorch's gradient of a real loss with respect to a complex tensor is
2 dL/dz*, the reference's dJ/dv convention (gpu/mesh.py:176-181, mesh.py:376), so the backward
passes ``grad_output`` to the back-propagation kernel unchanged and returns its input gradient as is.

Lossless crossings (mzi, sym, orth) store nothing for the backward pass but the output y: the kernel
rebuilds each layer's input with T^H, as the reference's backdiff does.  For nearest-neighbour meshes
the forward pass already builds the back-propagation coefficient tiles (one coefficient pass per
training step) and the backward pass reuses them unless another call rebuilt them meanwhile.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _lib
from ._lib import GEO_NN, OP_BWD, OP_FWD, OP_FWD_BWDTILES, check, load
from .mesh import MeshNetworkGPU, _stream


class _Plan:
    """Workspace cache of one (mesh, op, batch) combination."""

    def __init__(self, mesh: MeshNetworkGPU, op: int):
        self.mesh, self.op = mesh, op
        self.buf: Optional[torch.Tensor] = None

    def workspace(self, B: int):
        m = self.mesh
        nb = load().mg_workspace_bytes(self.op, m.N, m.L, B, m.crossing, m.geo_code,
                                       _lib.cfg_ptr(m.config.get(self.op)))
        if nb == 0:
            check(-1, "mg_workspace_bytes")
        if self.buf is None or self.buf.numel() < nb:
            self.buf = torch.empty(nb, dtype=torch.uint8, device=m.device)
            check(load().mg_workspace_init(self.buf.data_ptr(), nb, _stream(m.device)), "mg_workspace_init")
        return self.buf.data_ptr(), self.buf.numel()


def _plans(mesh: MeshNetworkGPU):
    p = getattr(mesh, "_autograd_plans", None)
    if p is None:
        p = {OP_FWD: _Plan(mesh, OP_FWD), OP_BWD: _Plan(mesh, OP_BWD)}
        mesh._autograd_plans = p
    return p


def _build(mesh: MeshNetworkGPU, op: int, p: torch.Tensor, B: int):
    """Build op's tiles for phases p into the mesh's cached workspace; returns (ws, bytes, version)."""
    lib = load()
    plan_ = _plans(mesh)[op]
    ws, nb = plan_.workspace(B)
    plan_.version = getattr(plan_, "version", 0) + 1
    s = mesh.p_splitter
    geo = ((None, None, mesh.strides.data_ptr()) if mesh.strides is not None
           else (mesh.lens.data_ptr(), mesh.shifts.data_ptr(), None))
    check(lib.mg_build_tiles(op, mesh.N, mesh.L, mesh.geo_code, *geo, mesh.crossing, p.data_ptr(),
                             mesh.N // 2 * mesh.X_np, s.data_ptr() if s.numel() else None, mesh.N // 2 * mesh.X_ns,
                             None, None, None, B, _lib.cfg_ptr(mesh.config.get(op)), ws, nb, _stream(mesh.device)),
          "mg_build_tiles")
    if mesh.perm_table is not None:
        check(lib.mg_build_perms(op, mesh.N, mesh.L, B, mesh.crossing, mesh.geo_code, mesh.perm_table.data_ptr(),
                                 _lib.cfg_ptr(mesh.config.get(op)), ws, nb, _stream(mesh.device)), "mg_build_perms")
    return ws, nb, plan_.version


class MeshFunction(torch.autograd.Function):
    """y = U(p) x for a lossless mesh; backward returns (dL/dx*·2, dL/dp)."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, p: torch.Tensor, mesh: MeshNetworkGPU):
        x = x.resolve_conj().resolve_neg().contiguous()
        p = p.detach().to(torch.float32).contiguous()
        # nearest-neighbour meshes: the back-propagation tiles serve the forward kernel and, later, the backward
        y, ver = _forward_y(mesh, x, p)
        ctx.mesh = mesh
        ctx.tiles_version = ver
        ctx.save_for_backward(y, p)
        return y

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        lib = load()
        y, p = ctx.saved_tensors
        mesh = ctx.mesh
        B, N = y.shape
        gy = gy.resolve_conj().resolve_neg().contiguous()
        plan_ = _plans(mesh)[OP_BWD]
        if ctx.tiles_version is not None and getattr(plan_, "version", None) == ctx.tiles_version:
            ws, nb = plan_.workspace(B)               # tiles of this forward are still in place
        else:
            ws, nb, _ = _build(mesh, OP_BWD, p, B)
        gx = torch.empty_like(gy)
        dp = torch.empty(p.numel(), dtype=torch.float32, device=y.device)
        check(lib.mg_propagate(OP_BWD, N, mesh.L, B, mesh.crossing, mesh.geo_code, y.data_ptr(), gy.data_ptr(), None,
                               gx.data_ptr(), N, dp.data_ptr(), N // 2 * mesh.X_np, 0,
                               _lib.cfg_ptr(mesh.config.get(OP_BWD)), ws, nb, _stream(mesh.device)), "mg_propagate")
        return gx, dp.view_as(p), None


def _forward_y(mesh: MeshNetworkGPU, x: torch.Tensor, p: torch.Tensor):
    """y = U(p) x through the kernels; returns (y, tiles version or None) as MeshFunction.forward does."""
    lib = load()
    B, N = x.shape
    assert N == mesh.N, "x must be (B, N) with N=%d" % mesh.N
    y = torch.empty_like(x)
    shared = mesh.geometry == GEO_NN
    if shared:
        ws, nb, ver = _build(mesh, OP_BWD, p, B)
        op, cfg = OP_FWD_BWDTILES, mesh.config.get(OP_BWD)
    else:
        ws, nb, ver = _build(mesh, OP_FWD, p, B)
        op, cfg = OP_FWD, mesh.config.get(OP_FWD)
    check(lib.mg_propagate(op, N, mesh.L, B, mesh.crossing, mesh.geo_code, x.data_ptr(), None, y.data_ptr(),
                           None, N, None, 0, 0, _lib.cfg_ptr(cfg), ws, nb, _stream(mesh.device)), "mg_propagate")
    return y, (ver if shared else None)


class MeshL2Function(torch.autograd.Function):
    """J = sum_b ||U(p) x_b - t_b||^2 for a lossless mesh.  The backward pass forms dJ/dy* = 2 (y - t)
    inside the back-propagation kernel (mg_propagate_l2) instead of in separate elementwise passes, the
    fused form of the reference's L2 gradient (gpu/mesh.py:176-181, 219-221)."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, p: torch.Tensor, t: torch.Tensor, mesh: MeshNetworkGPU):
        x = x.resolve_conj().resolve_neg().contiguous()
        t = t.resolve_conj().resolve_neg().to(x.dtype).contiguous()
        p = p.detach().to(torch.float32).contiguous()
        assert t.shape == x.shape, "target must have the shape of x"
        y, ver = _forward_y(mesh, x, p)
        d = y - t
        J = (torch.view_as_real(d) if d.is_complex() else d).square().sum()
        ctx.mesh, ctx.tiles_version = mesh, ver
        ctx.save_for_backward(y, p, t)
        return J

    @staticmethod
    def backward(ctx, gJ: torch.Tensor):
        lib = load()
        y, p, t = ctx.saved_tensors
        mesh = ctx.mesh
        B, N = y.shape
        plan_ = _plans(mesh)[OP_BWD]
        if ctx.tiles_version is not None and getattr(plan_, "version", None) == ctx.tiles_version:
            ws, nb = plan_.workspace(B)
        else:
            ws, nb, _ = _build(mesh, OP_BWD, p, B)
        gx = torch.empty_like(y)
        dp = torch.empty(p.numel(), dtype=torch.float32, device=y.device)
        check(lib.mg_propagate_l2(N, mesh.L, B, mesh.crossing, mesh.geo_code, y.data_ptr(), t.data_ptr(), None,
                                  gx.data_ptr(), N, dp.data_ptr(), N // 2 * mesh.X_np, 0,
                                  _lib.cfg_ptr(mesh.config.get(OP_BWD)), ws, nb, _stream(mesh.device)),
              "mg_propagate_l2")
        dp = dp.view_as(p).mul_(gJ)
        gx = gx.mul_(gJ) if ctx.needs_input_grad[0] else None
        gt = (y - t).mul_(-2 * gJ) if ctx.needs_input_grad[2] else None
        return gx, dp, gt, None


def mesh_l2_loss(mesh: MeshNetworkGPU, x: torch.Tensor, target: torch.Tensor,
                 p: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Differentiable J = sum |U(p) x - target|^2 over the batch; x and target (B, N), p (L, N/2, n_p)
    (defaults to the mesh's own phases).  The same J as ``((mesh_apply(mesh, x, p) - target).abs() ** 2).sum()``
    with the loss gradient formed inside the back-propagation kernel; meshes without a phase screen."""
    if p is None:
        p = mesh.p_crossing
    if mesh.is_phase:
        raise ValueError("mesh_l2_loss takes meshes without a phase screen; use mesh_apply for those")
    if x.dtype != mesh.dtype:
        x = x.to(mesh.dtype)
    return MeshL2Function.apply(x, p, target, mesh)


def mesh_apply(mesh: MeshNetworkGPU, x: torch.Tensor, p: Optional[torch.Tensor] = None,
               ph: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Differentiable y = U(p) x; x (B, N), p (L, N/2, n_p) (defaults to the mesh's own phases).

    A mesh with a phase screen (is_phase) applies D = diag(exp(i ph)) before (phi_pos 'in') or after
    ('out') the layers, as the reference's CPU path does (c/dot.cpp:97-143); ph (N,) defaults to the
    screen phases of the mesh and receives its gradient through PyTorch's autograd of the product."""
    if p is None:
        p = mesh.p_crossing
    dtype = mesh.dtype
    if x.dtype != dtype:
        x = x.to(dtype)
    if not mesh.is_phase:
        return MeshFunction.apply(x, p, mesh)
    if ph is None:
        ph = mesh.p_phase[mesh.n_cr * mesh.X_np:]
    d = torch.polar(torch.ones_like(ph, dtype=torch.float32), ph.to(torch.float32))
    if mesh.phi_pos == "in":
        return MeshFunction.apply(x * d, p, mesh)
    return MeshFunction.apply(x, p, mesh) * d


class Adam:
    """Adam (Kingma and Ba 2015, with bias correction) over float32 CUDA tensors, one fused launch per tensor
    (mg_adam_step).  The update of ``torch.optim.Adam(params, lr, betas, eps)`` without weight decay or amsgrad:
    each parameter, gradient and moment is read and written once per step instead of in a dozen elementwise
    passes.  Moments and the step count stay on the device, so ``GraphedStep`` can capture ``step()``."""

    def __init__(self, params, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8):
        self.params = list(params)
        for p in self.params:
            if p.dtype != torch.float32 or not p.is_cuda or not p.is_contiguous():
                raise ValueError("Adam takes contiguous float32 CUDA tensors")
        self.lr, self.betas, self.eps = float(lr), (float(betas[0]), float(betas[1])), float(eps)
        self.exp_avg = [torch.zeros_like(p) for p in self.params]
        self.exp_avg_sq = [torch.zeros_like(p) for p in self.params]
        self.state = [torch.zeros(2, dtype=torch.int32, device=p.device) for p in self.params]   # steps, counter

    def zero_grad(self, set_to_none: bool = True):
        for p in self.params:
            if set_to_none:
                p.grad = None
            elif p.grad is not None:
                p.grad.zero_()

    @torch.no_grad()
    def step(self):
        lib = load()
        for p, m, v, s in zip(self.params, self.exp_avg, self.exp_avg_sq, self.state):
            if p.grad is None:
                continue
            g = p.grad.to(torch.float32).contiguous()
            check(lib.mg_adam_step(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), p.numel(), self.lr,
                                   self.betas[0], self.betas[1], self.eps, s.data_ptr(), _stream(p.device)),
                  "mg_adam_step")


class GraphedStep:
    """A training step captured once in a CUDA graph and replayed.

    ``step()`` takes no arguments, runs the forward pass (through ``mesh_apply``), the backward pass and
    the optimizer update, and returns the loss tensor. A small mesh or batch makes such a step
    launch-bound: a dozen kernels (coefficient tiles, forward, loss, back-propagation, reduction,
    optimizer) and the Python around them. A replay costs one graph launch.

    Requirements, as for any CUDA-graph capture:
    - every tensor the step reads keeps its storage between replays (update inputs in place);
    - the optimizer keeps its state on the device (``torch.optim.Adam(..., capturable=True)``).

    The ``warmup`` calls before the capture are real steps; they also size the meshes' cached workspaces.
    The mesh kernels launch on the current stream and never synchronise, so the capture records them.
    Their run-time status (a bounded wait that expired, a malformed geometry) accumulates in the mesh's
    workspaces across replays: read it with ``mesh.status()`` between replays.
    """

    def __init__(self, step, warmup: int = 3):
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(warmup):
                step()
        torch.cuda.current_stream().wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = step()

    def __call__(self) -> torch.Tensor:
        """Run one more step; returns the loss tensor of that step (the same storage on every call)."""
        self.graph.replay()
        return self.loss

