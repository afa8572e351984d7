"""Lossy meshes: generic 2x2 crossings with a checkpointed adjoint on the sm_103a kernels.

The lossless path back-propagates by inverting each layer with T^H (the reference's c/dot.cpp:75-80 and
gpu/backprop.cu do the same), which needs no stored activations but is exact only for unitary crossings.
A lossy crossing - the generic MZI of crossing.py:444-488, with phase errors and gains g_ij - breaks it.
Here the adjoint keeps the mesh input of every segment of ceil(sqrt(L)) layers during the forward pass;
back-propagation then walks the
segments in reverse, recomputes each segment's layer inputs from its checkpoint (one forward launch
that writes them to a (segment, B, N) buffer) and back-propagates
through the segment from those stored inputs (one launch plus a deterministic reduction).  Each
direction is one library call (mg_lossy_forward / mg_lossy_backward) that runs all its segments.  Memory is
about 2 sqrt(L) fields instead of L; work is one extra forward pass.

The crossing is given as its transfer matrices ``T`` (L, N/2, 2, 2), complex, in the reference's slot
grid (gpu/mesh.py:77-81); ``mzi_generic_T`` builds them from (theta, phi) and the 14 error parameters
with differentiable torch operations, so gradients reach the phases (or any other parameterisation)
through PyTorch's own autograd of T.  The kernel returns dJ/dT as sum_b g_i conj(x_j) = 2 dJ/dT_ij*,
PyTorch's gradient convention for complex tensors.
"""
from __future__ import annotations

import math
from typing import Optional

import numpy as np
import torch

from . import geometry as geom
from ._lib import GENERIC, GEO_FFT, GEO_NN, OP_BWD_STORED, OP_FWD, check, load
from .mesh import _stream


def mzi_generic_T(p: torch.Tensor, s: Optional[torch.Tensor] = None) -> torch.Tensor:
    """(..., 2, 2) complex T of the lossy generic MZI, T = S(beta) D2 S(alpha) D1 (crossing.py:466-488).

    p (..., 2) = (theta, phi); s (..., 14) = (alpha, beta, fabrication phase errors e11, e21, e12, e22,
    crosstalk phase errors x11, x21, x12, x22, log-gains g11, g21, g12, g22);
    D1 = diag(exp(i(phi + e11 + x11) + g11/2), exp(i(e21 + x21) + g21/2)),
    D2 = diag(exp(i(theta + e12 + x12) + g12/2), exp(i(e22 + x22) + g22/2)),
    S(a) = [[cos(pi/4 + a), i sin(pi/4 + a)], [i sin(pi/4 + a), cos(pi/4 + a)]].
    """
    if s is None:
        s = p.new_zeros(p.shape[:-1] + (14,))
    th, ph = p[..., 0], p[..., 1]

    def ep(phase, gain):                       # exp(i phase + gain / 2)
        return torch.exp(torch.complex(gain / 2, phase))

    d1a, d1b = ep(ph + s[..., 2] + s[..., 6], s[..., 10]), ep(s[..., 3] + s[..., 7], s[..., 11])
    d2a, d2b = ep(th + s[..., 4] + s[..., 8], s[..., 12]), ep(s[..., 5] + s[..., 9], s[..., 13])
    ca, sa = torch.cos(math.pi / 4 + s[..., 0]), torch.sin(math.pi / 4 + s[..., 0])
    cb, sb = torch.cos(math.pi / 4 + s[..., 1]), torch.sin(math.pi / 4 + s[..., 1])
    # D2 S(alpha) D1
    n00, n01 = d2a * ca * d1a, d2a * (1j * sa) * d1b
    n10, n11 = d2b * (1j * sa) * d1a, d2b * ca * d1b
    # S(beta) (D2 S(alpha) D1)
    t00, t01 = cb * n00 + (1j * sb) * n10, cb * n01 + (1j * sb) * n11
    t10, t11 = (1j * sb) * n00 + cb * n10, (1j * sb) * n01 + cb * n11
    return torch.stack([torch.stack([t00, t01], -1), torch.stack([t10, t11], -1)], -2)


class GenericMZIT(torch.autograd.Function):
    """T of the lossy generic MZI from the library's double-precision kernel (complex64 result), with its
    vector-Jacobian product for the phases p; the splitter/error parameters s are held constant."""

    @staticmethod
    def forward(ctx, p: torch.Tensor, s: Optional[torch.Tensor]):
        p64 = p.detach().to(torch.float64).contiguous()
        s64 = None if s is None else s.detach().to(device=p.device, dtype=torch.float64).contiguous()
        n = p64.numel() // 2
        T = torch.empty(p64.shape[:-1] + (2, 2), dtype=torch.complex64, device=p.device)
        check(load().mg_generic_mzi_T(n, p64.data_ptr(), None if s64 is None else s64.data_ptr(), T.data_ptr(),
                                      _stream(p.device)), "mg_generic_mzi_T")
        ctx.save_for_backward(p64, s64 if s64 is not None else p64.new_empty(0))
        ctx.p_dtype = p.dtype
        return T

    @staticmethod
    def backward(ctx, gT: torch.Tensor):
        p64, s64 = ctx.saved_tensors
        g = gT.detach().to(torch.complex64).resolve_conj().resolve_neg().contiguous()
        dp = torch.empty_like(p64)
        check(load().mg_generic_mzi_T_vjp(p64.numel() // 2, p64.data_ptr(), s64.data_ptr() if s64.numel() else None,
                                          g.data_ptr(), dp.data_ptr(), _stream(p64.device)), "mg_generic_mzi_T_vjp")
        return dp.to(ctx.p_dtype), None


class LossyMesh:
    """Geometry of a mesh of generic (possibly lossy) crossings; ``mesh(x, T)`` is y = U(T) x.

    Nearest-neighbour geometry (``lens``, ``shifts``, as gpu/mesh.py:50-60) or butterfly/FFT strides.
    ``segment`` fixes the checkpoint spacing of the adjoint (default: ``segment_for(B)``).
    """

    def __init__(self, N: int, lens=None, shifts=None, strides=None, device=None, segment: Optional[int] = None):
        load()
        assert N % 2 == 0
        self.N = int(N)
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if strides is not None:
            self.geometry = GEO_FFT
            self.strides_h = [int(v) for v in np.asarray(strides).reshape(-1)]
            geom.validate_fft(N, self.strides_h)
            self.L = len(self.strides_h)
            self.strides = torch.tensor(self.strides_h, dtype=torch.int32, device=self.device)
            self.lens = self.shifts = None
            active = np.ones((self.L, N // 2), dtype=bool)
        else:
            self.geometry = GEO_NN
            self.lens_h = [int(v) for v in np.asarray(lens).reshape(-1)]
            self.shifts_h = [int(v) for v in np.asarray(shifts).reshape(-1)]
            geom.validate_nn(N, self.lens_h, self.shifts_h)
            self.L = len(self.lens_h)
            self.lens = torch.tensor(self.lens_h, dtype=torch.int32, device=self.device)
            self.shifts = torch.tensor(self.shifts_h, dtype=torch.int32, device=self.device)
            self.strides = None
            active = np.zeros((self.L, N // 2), dtype=bool)
            for l, (ln, sh) in enumerate(zip(self.lens_h, self.shifts_h)):
                active[l, sh // 2: sh // 2 + ln] = True
        self.active = torch.as_tensor(active, device=self.device)
        self._segment = int(segment) if segment else None
        self._ws = {}

    def segment_for(self, B: int) -> int:
        """Checkpoint spacing used for a batch of B vectors: ceil(sqrt(L)) layers, whatever B.  Keeping a
        segment's stored inputs inside the 129 MB L2 (8 layers at N=256, B=4096) measured slower on GB300: the
        step took 2.07 ms with 8-layer segments, 1.93 ms with 16 (sqrt L) and 1.80 ms with 32, the gradient
        bitwise the same; the fewer launches outweigh the inputs read back from HBM."""
        if self._segment:
            return self._segment
        return max(1, math.ceil(math.sqrt(max(self.L, 1))))

    @property
    def segment(self) -> int:
        return self._segment or max(1, math.ceil(math.sqrt(max(self.L, 1))))

    # ---- plumbing
    def _geo(self):
        if self.geometry == GEO_FFT:
            return None, None, self.strides.data_ptr()
        return self.lens.data_ptr(), self.shifts.data_ptr(), None

    def _workspace(self, op: int, B: int):
        lib = load()
        nb = lib.mg_workspace_bytes(op, self.N, self.L, B, GENERIC, self.geometry, None)
        if nb == 0:
            check(-1, "mg_workspace_bytes")
        buf = self._ws.get(op)
        if buf is None or buf.numel() < nb:
            buf = torch.empty(nb, dtype=torch.uint8, device=self.device)
            check(lib.mg_workspace_init(buf.data_ptr(), nb, _stream(self.device)), "mg_workspace_init")
            self._ws[op] = buf
        return buf.data_ptr(), buf.numel()

    def _build(self, op: int, Tc: torch.Tensor, B: int):
        ws, nb = self._workspace(op, B)
        check(load().mg_build_tiles(op, self.N, self.L, self.geometry, *self._geo(), GENERIC, None, 0, None, 0, None,
                                    Tc.data_ptr(), None, B, None, ws, nb, _stream(self.device)), "mg_build_tiles")
        return ws, nb

    def _range(self, op, l0, l1, B, in0, in1, out0, out1, act, dT, ws, nb):
        ptr = (lambda t: None if t is None else t.data_ptr())
        check(load().mg_propagate_range(op, self.N, self.L, l0, l1, B, GENERIC, self.geometry, ptr(in0), ptr(in1),
                                        ptr(out0), ptr(out1), self.N, ptr(act), ptr(dT), 0, None, ws, nb,
                                        _stream(self.device)), "mg_propagate_range")

    def status(self, clear: bool = True) -> int:
        """Kernel status word of the last launches (0 = ok); reads both workspaces."""
        lib = load()
        st = 0
        for buf in self._ws.values():
            r = lib.mg_read_status(buf.data_ptr(), int(clear), _stream(self.device))
            if r < 0:
                check(r, "mg_read_status")
            st = st or r
        return st

    # ---- user API
    def T(self, p: torch.Tensor, s: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Lossy generic-MZI transfer matrices (L, N/2, 2, 2) from p (L, N/2, 2) and s (L, N/2, 14):
        the library kernel (complex64, gradient to p) unless s needs a gradient too, in which case
        the differentiable tensor formula ``mzi_generic_T`` (complex, dtype of p)."""
        if p.is_cuda and not (s is not None and s.requires_grad):
            return GenericMZIT.apply(p, s)
        return mzi_generic_T(p, s)

    def __call__(self, x: torch.Tensor, T: torch.Tensor) -> torch.Tensor:
        return LossyMeshFunction.apply(x, T, self)


class LossyMeshFunction(torch.autograd.Function):
    """y = U(T) x for x (B, N) complex, T (L, N/2, 2, 2) complex; gradients to x and T."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, T: torch.Tensor, mesh: LossyMesh):
        assert x.dim() == 2 and x.shape[1] == mesh.N, "x must be (B, N) with N=%d" % mesh.N
        assert tuple(T.shape) == (mesh.L, mesh.N // 2, 2, 2), "T must be (L, N/2, 2, 2)"
        x = x.detach().to(device=mesh.device, dtype=torch.complex64).resolve_conj().resolve_neg().contiguous()
        Tc = T.detach().to(device=mesh.device, dtype=torch.complex64).resolve_conj().resolve_neg().contiguous()
        B, L = x.shape[0], mesh.L
        seg = mesh.segment_for(B)
        K = -(-L // seg)
        ckpt = torch.empty((max(K - 1, 0), B, mesh.N), dtype=torch.complex64, device=mesh.device)
        y = torch.empty_like(x)
        if B > 0:
            ws, nb = mesh._build(OP_FWD, Tc, B) if L > 0 else (None, 0)
            check(load().mg_lossy_forward(mesh.N, L, B, mesh.geometry, seg, x.data_ptr(), y.data_ptr(),
                                          ckpt.data_ptr() if ckpt.numel() else None, mesh.N, ws, nb,
                                          _stream(mesh.device)), "mg_lossy_forward")
        ctx.mesh = mesh
        ctx.seg = seg
        ctx.T_dtype = T.dtype
        ctx.save_for_backward(Tc, x, ckpt)
        return y

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        mesh = ctx.mesh
        Tc, x, ckpt = ctx.saved_tensors
        B, N, L, seg = x.shape[0], mesh.N, mesh.L, ctx.seg
        gy = gy.detach().to(torch.complex64).resolve_conj().resolve_neg().contiguous()
        dT = torch.zeros((L, N // 2, 2, 2), dtype=torch.complex64, device=mesh.device)
        g = torch.empty_like(gy)
        if B > 0:
            wsf, nbf = mesh._build(OP_FWD, Tc, B) if L > 0 else (None, 0)
            wsb, nbb = mesh._build(OP_BWD_STORED, Tc, B) if L > 0 else (None, 0)
            act = torch.empty((min(seg, max(L, 1)), B, N), dtype=torch.complex64, device=mesh.device)
            gtmp = torch.empty_like(gy)
            check(load().mg_lossy_backward(N, L, B, mesh.geometry, seg, x.data_ptr(),
                                           ckpt.data_ptr() if ckpt.numel() else None, gy.data_ptr(), g.data_ptr(),
                                           gtmp.data_ptr(), act.data_ptr(), dT.data_ptr(), N, wsf, nbf, wsb, nbb,
                                           _stream(mesh.device)), "mg_lossy_backward")
        gx = g if ctx.needs_input_grad[0] else None
        gT = dT.to(ctx.T_dtype) if ctx.needs_input_grad[1] else None
        return gx, gT, None


class GenericMeshGPU:
    """The MeshNetworkGPU API (``dot``, ``grad_phi``, ``L2norm``, ``grad_phi_target``, ``matrix``; reference
    gpu/mesh.py:21-297) for a mesh of any crossing in ``crossings.SIZES`` - the reference's other
    parameterisations (crossing.py:292-611), which its GPU path does not run.

    T(p, s) is built per slot by ``crossings.transfer`` (differentiable, float64), propagated by the GPU
    kernels' generic precomputed-T path, and differentiated with the checkpointed stored-activation adjoint,
    which is exact for lossy and lossless crossings alike; dJ/dp follows from dJ/dT through PyTorch's
    autograd of T.  Parameter layout as MeshNetworkGPU: p_phase = the (L, N/2, n_phase) grid flattened,
    followed by N screen phases when ``is_phase``; p_splitter (L, N/2, n_splitter).  Fields are (N, B).
    """

    def __init__(self, N: int, L: int, lens=None, shifts=None, p_phase=None, p_splitter=None, X: str = "mzi_generic",
                 phi_pos: str = "out", is_phase: bool = False, strides=None, device=None,
                 segment: Optional[int] = None):
        from .crossings import SIZES
        if X not in SIZES:
            raise ValueError("unknown crossing %r" % X)
        assert phi_pos in ("in", "out")
        self.mesh = LossyMesh(N, lens, shifts, strides, device, segment)
        assert self.mesh.L == L, "L=%d does not match the geometry (%d layers)" % (L, self.mesh.L)
        self.N, self.L, self.X = int(N), int(L), X
        self.phi_pos, self.is_phase = phi_pos, bool(is_phase)
        self.device = self.mesh.device
        self.X_np, self.X_ns = SIZES[X]
        self.n_cr = self.L * (self.N // 2)
        n_phase = self.n_cr * self.X_np + (self.N if self.is_phase else 0)
        self.p_phase = self._param(np.zeros(n_phase) if p_phase is None else p_phase).reshape(-1)
        assert self.p_phase.numel() == n_phase, "p_phase has %d entries, expected %d" % (self.p_phase.numel(), n_phase)
        self.p_splitter = None if p_splitter is None else self._param(p_splitter).reshape(self.L, self.N // 2, self.X_ns)
        # inactive slots take parameters inside every crossing's domain (the kernels use the identity there)
        self._safe_p = torch.zeros(self.X_np, dtype=torch.float64, device=self.device)
        if X == "cartesian":
            self._safe_p[0] = 2.0
        self.dtype = torch.complex64

    @property
    def n_phase(self) -> int:
        return self.p_phase.numel()

    def _param(self, x) -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            return x.detach().to(device=self.device, dtype=torch.float64)
        return torch.as_tensor(np.asarray(x, dtype=np.float64), device=self.device)

    def transfer(self, p: torch.Tensor, s: Optional[torch.Tensor] = None) -> torch.Tensor:
        """T (L, N/2, 2, 2) complex128 of the crossing parameters p (L, N/2, n_phase), identity on inactive slots."""
        from .crossings import transfer
        act = self.mesh.active[..., None]
        T = transfer(self.X, torch.where(act, p, self._safe_p), s)
        eye = torch.eye(2, dtype=T.dtype, device=T.device)
        return torch.where(act[..., None], T, eye)

    def _forward(self, x: torch.Tensor, p: torch.Tensor, s: Optional[torch.Tensor]) -> torch.Tensor:
        """y (B, N) for x (B, N) and the flat parameter vector p (differentiable in both)."""
        ncp = self.n_cr * self.X_np
        if self.is_phase and self.phi_pos == "in":
            x = x * torch.exp(1j * p[ncp:])
        y = self.mesh(x, self.transfer(p[:ncp].reshape(self.L, self.N // 2, self.X_np), s))
        if self.is_phase and self.phi_pos == "out":
            y = y * torch.exp(1j * p[ncp:])
        return y

    def _rows(self, v) -> torch.Tensor:
        v = v if isinstance(v, torch.Tensor) else torch.as_tensor(np.asarray(v))
        v = v.to(device=self.device)
        assert v.dim() == 2 and v.shape[0] == self.N, "v must be (N, B) with N=%d" % self.N
        return v.t().to(torch.complex64).resolve_conj().resolve_neg().contiguous()

    def _args(self, p_phase, p_splitter):
        p = self.p_phase if p_phase is None else self._param(p_phase).reshape(-1)
        s = self.p_splitter if p_splitter is None else self._param(p_splitter).reshape(self.L, self.N // 2, self.X_ns)
        assert p.numel() == self.n_phase
        return p, s

    def dot(self, v, p_phase=None, p_splitter=None) -> torch.Tensor:
        """y = U v for v (N, B); returns (N, B) complex64."""
        p, s = self._args(p_phase, p_splitter)
        with torch.no_grad():
            y = self._forward(self._rows(v), p, s)
        return y.to(torch.complex64).t()

    def grad_phi(self, v, dJdv, p_phase=None, p_splitter=None, out_dp=None, out_dJdv=None, vpos: str = "in"):
        """(dJ/dp, dJ/dv_in*·2) for J(v_out) with v the INPUT fields; dJdv is 2 dJ/dv_out* or a callable of
        v_out, as MeshNetworkGPU.grad_phi.  vpos 'out' (rebuilding the input from the output by T^H, what
        the reference does) is refused: it is exact only for unitary crossings."""
        if vpos != "in":
            raise NotImplementedError("generic crossings back-propagate from the input fields (vpos='in')")
        p, s = self._args(p_phase, p_splitter)
        p = p.clone().requires_grad_(True)
        x = self._rows(v).requires_grad_(True)
        with torch.enable_grad():
            y = self._forward(x, p, s)
            yv = y.detach().to(torch.complex64).t()
            g = dJdv(yv) if callable(dJdv) else dJdv
            g = self._rows(g).to(y.dtype)
            dp, gx = torch.autograd.grad(y, (p, x), g)
        dp = dp.to(torch.float32)
        if out_dp is not None:
            out_dp += dp.reshape(out_dp.shape)
            dp = out_dp
        gx = gx.to(torch.complex64).t()
        if out_dJdv is not None:
            out_dJdv.copy_(gx)
            gx = out_dJdv
        return dp, gx

    def matrix(self, p_phase=None, p_splitter=None) -> torch.Tensor:
        return self.dot(torch.eye(self.N, dtype=torch.complex64, device=self.device), p_phase, p_splitter)

    def _L2norm_fn(self, J):
        def f(U):
            V = U - torch.eye(self.N, dtype=U.dtype, device=U.device)
            if not self.is_phase:
                V = V - torch.diag(torch.diagonal(V))
            J[0] = float(torch.linalg.norm(V) ** 2)
            return 2 * V
        return f

    def L2norm(self, U_target, p_phase=None, p_splitter=None) -> float:
        """||U U_t^H - I||^2 (off-diagonal only without a screen), as MeshNetworkGPU.L2norm."""
        J = [0.0]
        self._L2norm_fn(J)(self.dot(self._adjoint(U_target), p_phase, p_splitter))
        return J[0]

    def grad_phi_target(self, U_target, p_phase=None, p_splitter=None):
        J = [0.0]
        dp = self.grad_phi(self._adjoint(U_target), self._L2norm_fn(J), p_phase, p_splitter)[0]
        return J[0], dp

    def _adjoint(self, U) -> torch.Tensor:
        U = U if isinstance(U, torch.Tensor) else torch.as_tensor(np.asarray(U))
        return U.to(device=self.device, dtype=torch.complex64).t().conj()

    def status(self, clear: bool = True) -> int:
        return self.mesh.status(clear)
