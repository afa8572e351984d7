"""MeshNetworkGPU: drop-in counterpart of the reference's ``meshes.gpu.MeshNetworkGPU``
(gpu/mesh.py:21-297) running on the sm_103a kernels of libmeshes_gb300.so.

Same constructor and methods (``dot``, ``grad_phi``, ``L2norm``, ``grad_phi_target``, ``matrix``,
``hvp``, ``hess``), same parameter grid (p_phase = L*N/2*n_p floats, p_splitter (L, N/2, n_s)) and
the same field layout: ``dot`` takes and returns (N, B) arrays whose columns are contiguous (the
reference's Fortran-order CuPy arrays), here as torch tensors with strides (1, ldu).  Inputs may be
torch tensors or numpy arrays.  Butterfly meshes take ``strides`` (stride exponents per layer)
instead of ``lens``/``shifts``, like the reference's *_ft kernels (gpu/consts.cuh:31-35).

Beyond the reference's GPU API (which refuses both, gpu/mesh.py:65 and mesh.py:573), a mesh may carry
an input or output phase screen (``is_phase``) and permutations between layers (``perm``: L+1 index
arrays or None, the reference's ``StructuredMeshNetwork.perm``, mesh.py:238-277).
"""
from __future__ import annotations

from typing import Callable, Optional, Tuple

import numpy as np
import torch

from . import _lib
from ._lib import GEO_FFT, GEO_NN, GEO_PERM, OP_BWD, OP_FWD, OP_FWDDIFF, check, load
from . import geometry as geom

_NP_NS = {"mzi": (2, 2), "sym": (2, 1), "orth": (1, 0)}   # gpu/mesh.py:72-73


def _stream(device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class Workspace:
    """Caller-side scratch for one mesh and op, grown on demand (torch caching allocator)."""

    def __init__(self, device):
        self.device = device
        self.buf: Optional[torch.Tensor] = None

    def get(self, nbytes: int) -> Tuple[int, int]:
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=self.device)
            check(load().mg_workspace_init(self.buf.data_ptr(), self.buf.numel(), _stream(self.device)),
                  "mg_workspace_init")
        return self.buf.data_ptr(), self.buf.numel()

    def status(self, clear=True) -> int:
        if self.buf is None:
            return 0
        rc = load().mg_read_status(self.buf.data_ptr(), int(clear), _stream(self.device))
        if rc < 0:
            check(rc, "mg_read_status")
        return rc


class MeshNetworkGPU:
    """Mesh network on the GPU (reference gpu/mesh.py:21-297)."""

    def __init__(self, N: int, L: int, lens=None, shifts=None, p_phase=None, p_splitter=None, X: str = "mzi",
                 phi_pos: str = "out", is_phase: bool = True, strides=None, device=None, perm=None):
        assert X in ["mzi", "sym", "orth"]
        assert phi_pos in ["in", "out"]
        # the reference GPU API forbids the phase screen (gpu/mesh.py:65); here it is supported for complex
        # crossings as the reference CPU path defines it (c/dot.cpp:97-143)
        assert not (is_phase and X == "orth"), "a phase screen needs a complex crossing"
        assert N % 2 == 0
        load()
        self._N, self._L, self.X = int(N), int(L), X
        self.phi_pos, self.is_phase = phi_pos, is_phase
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.X_np, self.X_ns = _NP_NS[X]
        self.dtype = torch.float32 if X == "orth" else torch.complex64
        self.crossing = _lib.CROSSING_CODES[X]
        if strides is not None:
            self.geometry = GEO_FFT
            self.strides_h = [int(x) for x in np.asarray(strides).reshape(-1)]
            assert len(self.strides_h) == L
            geom.validate_fft(N, self.strides_h)
            self.strides = torch.tensor(self.strides_h, dtype=torch.int32, device=self.device)
            self.lens = self.shifts = None
        else:
            self.geometry = GEO_NN
            self.lens_h = [int(x) for x in np.asarray(lens).reshape(-1)]
            self.shifts_h = [int(x) for x in np.asarray(shifts).reshape(-1)]
            assert len(self.lens_h) == L
            geom.validate_nn(N, self.lens_h, self.shifts_h)
            self.lens = torch.tensor(self.lens_h, dtype=torch.int32, device=self.device)
            self.shifts = torch.tensor(self.shifts_h, dtype=torch.int32, device=self.device)
            self.strides = None
        p_phase = np.zeros(self.n_phase) if p_phase is None else p_phase
        assert _numel(p_phase) == self.n_phase, "p_phase has %d entries, expected %d" % (_numel(p_phase), self.n_phase)
        self.p_phase = self._param(p_phase).reshape(-1)
        n_spl = 0 if p_splitter is None else _numel(p_splitter)
        assert n_spl in [self.n_splitter, 0]
        self.p_splitter = (self._param(p_splitter).reshape(L, N // 2, self.X_ns) if n_spl
                           else torch.empty((L, N // 2, 0), dtype=torch.float32, device=self.device))
        self.perm_h, self.perm_table = _perm_rows(perm, self.N, self.L)
        if self.perm_table is not None:
            self.perm_table = torch.as_tensor(self.perm_h, device=self.device)
        # geometry code of the library calls: the layout, with MG_GEO_PERM when permutations ride along
        self.geo_code = self.geometry | (GEO_PERM if self.perm_table is not None else 0)
        self._ws = {op: Workspace(self.device) for op in (OP_FWD, OP_FWDDIFF, OP_BWD)}
        self.config = {OP_FWD: None, OP_FWDDIFF: None, OP_BWD: None}   # mg_config per op (autotuner)

    # ---- sizes (gpu/mesh.py:94-123)
    @property
    def L(self):
        return self._L

    @property
    def M(self):
        return self._N

    @property
    def N(self):
        return self._N

    @property
    def n_cr(self):
        """Number of slots including blank crossings (gpu/mesh.py:111-117)."""
        return self.L * (self.N // 2)

    @property
    def n_splitter(self):
        return self.n_cr * self.X_ns

    @property
    def n_phase(self):
        return self.n_cr * self.X_np + self.is_phase * self.N

    @property
    def p_crossing(self):
        return self.p_phase[: self.n_cr * self.X_np].reshape(self.L, self.N // 2, self.X_np)

    @property
    def shape(self):
        return (self.M, self.N)

    # ---- conversions
    def _param(self, x) -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            return x.detach().to(device=self.device, dtype=torch.float32).contiguous()
        return torch.as_tensor(np.asarray(x, dtype=np.float32), device=self.device).contiguous()

    def _defaults(self, p_phase, p_splitter):
        p = self.p_phase if p_phase is None else self._param(p_phase).reshape(-1)
        s = self.p_splitter if p_splitter is None else self._param(p_splitter)
        assert p.numel() == self.n_phase and s.numel() in [self.n_splitter, 0]
        return p, s

    def _field(self, v) -> Tuple[torch.Tensor, int]:
        """(N, B) input -> (tensor whose column b starts at data_ptr + b*ldu elements, ldu)."""
        if not isinstance(v, torch.Tensor):
            v = torch.as_tensor(np.asarray(v))
        # a lazily conjugated or negated view (torch's conj/neg bits, e.g. U.t().conj()) is materialised: the
        # kernels read the memory behind data_ptr, which holds the unconjugated values
        v = v.to(device=self.device, dtype=self.dtype).resolve_conj().resolve_neg()
        assert v.dim() == 2 and v.shape[0] == self.N, "v must be (N, B) with N=%d" % self.N
        align = 8 if self.X == "orth" else 16
        if (v.stride(0) == 1 and (v.shape[1] == 1 or (v.stride(1) >= self.N and v.stride(1) % 2 == 0))
                and v.data_ptr() % align == 0):
            ldu = v.stride(1) if v.shape[1] > 1 else self.N
            return v, ldu
        return v.t().contiguous().t(), self.N

    def _out(self, out, B) -> Tuple[torch.Tensor, int]:
        if out is None:
            return torch.empty((B, self.N), dtype=self.dtype, device=self.device).t(), self.N
        assert out.shape == (self.N, B) and out.dtype == self.dtype and out.stride(0) == 1
        return out, (out.stride(1) if B > 1 else self.N)

    def _geo_args(self):
        if self.geometry == GEO_FFT:
            return (self.strides.data_ptr(),)
        return (self.lens.data_ptr(), self.shifts.data_ptr())

    def _ps_args(self, p, s):
        ldp = self.N // 2 * self.X_np
        lds = self.N // 2 * self.X_ns
        sp = s.data_ptr() if s.numel() else None
        return p.data_ptr(), ldp, sp, lds

    def _programmed(self, op, p, s, B, dp=None) -> Tuple[int, int]:
        """Tiles of op for phases p (and direction dp) plus the permutation tables, in op's workspace."""
        lib = load()
        wsb = lib.mg_workspace_bytes(op, self.N, self.L, B, self.crossing, self.geo_code, None)
        if wsb == 0:
            check(-1, "mg_workspace_bytes")
        ws, wsn = self._ws[op].get(wsb)
        stream = _stream(self.device)
        pptr, ldp, sptr, lds = self._ps_args(p, s)
        geo = ((None, None, self.strides.data_ptr()) if self.geometry == GEO_FFT
               else (self.lens.data_ptr(), self.shifts.data_ptr(), None))
        check(lib.mg_build_tiles(op, self.N, self.L, self.geo_code, *geo, self.crossing, pptr, ldp, sptr, lds,
                                 None if dp is None else dp.data_ptr(), None, None, B, None, ws, wsn, stream),
              "mg_build_tiles")
        check(lib.mg_build_perms(op, self.N, self.L, B, self.crossing, self.geo_code, self.perm_table.data_ptr(), None,
                                 ws, wsn, stream), "mg_build_perms")
        return ws, wsn

    # ---- forward / forward-mode derivative (gpu/mesh.py:147-174)
    def dot(self, v, p_phase=None, p_splitter=None, dp=None, dv=None, out=None, dout=None):
        """y = U v (v (N, B)); with dp and/or dv also the forward-mode derivative dy (gpu/mesh.py:147-174).
        With is_phase, the N screen phases (the tail of p_phase) act before (phi_pos 'in') or after
        ('out') the mesh."""
        if not self.is_phase:
            return self._dot_mesh(v, p_phase, p_splitter, dp, dv, out, dout)
        return self._dot_screened(v, p_phase, p_splitter, dp, dv, out, dout)

    def _dot_mesh(self, v, p_phase=None, p_splitter=None, dp=None, dv=None, out=None, dout=None):
        lib = load()
        v, ldu_in = self._field(v)
        p, s = self._defaults(p_phase, p_splitter)
        B = v.shape[1]
        out, ldu_out = self._out(out, B)
        stream = _stream(self.device)
        pptr, ldp, sptr, lds = self._ps_args(p, s)
        if dp is None and dv is None:
            if ldu_in != ldu_out:
                tmp, ldu = self._out(None, B)
                tmp.copy_(v)
                v, ldu_in = tmp, ldu
            if self.perm_table is not None:
                if B:
                    ws, wsn = self._programmed(OP_FWD, p, s, B)
                    check(lib.mg_propagate(OP_FWD, self.N, self.L, B, self.crossing, self.geo_code, v.data_ptr(), None,
                                           out.data_ptr(), None, ldu_out, None, 0, 0, None, ws, wsn, stream),
                          "mg_propagate")
                return out
            wsb = lib.mg_workspace_bytes(OP_FWD, self.N, self.L, B, self.crossing, self.geometry, None)
            ws, wsn = self._ws[OP_FWD].get(wsb)
            fn = lib.mg_fwdprop_ft if self.geometry == GEO_FFT else lib.mg_fwdprop
            check(fn(self.N, self.L, B, *self._geo_args(), pptr, ldp, sptr, lds, v.data_ptr(), out.data_ptr(), ldu_out,
                     self.crossing, ws, wsn, stream), fn.__name__)
            return out
        dout, ldu_dout = self._out(dout, B)
        dpp = None if dp is None else self._param(dp).reshape(-1)
        if dpp is not None:
            assert dpp.numel() in (0, p.numel())
            if dpp.numel() == 0:
                dpp = None
        if dv is not None:
            dv, ldu_dv = self._field(dv)
        # all four fields share one ldu: normalise to fresh (B, N) buffers when they differ
        if len({ldu_in, ldu_out, ldu_dout} | ({ldu_dv} if dv is not None else set())) > 1:
            v = v.t().contiguous().t()
            if dv is not None:
                dv = dv.t().contiguous().t()
            o2, _ = self._out(None, B)
            d2, _ = self._out(None, B)
            self._dot_mesh(v, p, s, dp=dpp, dv=dv, out=o2, dout=d2)
            out.copy_(o2)
            dout.copy_(d2)
            return out, dout
        if self.perm_table is not None:
            if B:
                ws, wsn = self._programmed(OP_FWDDIFF, p, s, B, dp=dpp)
                check(lib.mg_propagate(OP_FWDDIFF, self.N, self.L, B, self.crossing, self.geo_code, v.data_ptr(),
                                       None if dv is None else dv.data_ptr(), out.data_ptr(), dout.data_ptr(), ldu_out,
                                       None, 0, 0, None, ws, wsn, stream), "mg_propagate")
            return out, dout
        wsb = lib.mg_workspace_bytes(OP_FWDDIFF, self.N, self.L, B, self.crossing, self.geometry, None)
        ws, wsn = self._ws[OP_FWDDIFF].get(wsb)
        fn = lib.mg_fwddiff_ft if self.geometry == GEO_FFT else lib.mg_fwddiff
        check(fn(self.N, self.L, B, *self._geo_args(), pptr, None if dpp is None else dpp.data_ptr(), ldp, sptr, lds,
                 v.data_ptr(), None if dv is None else dv.data_ptr(), out.data_ptr(), dout.data_ptr(), ldu_out,
                 self.crossing, ws, wsn, stream), fn.__name__)
        return out, dout

    # ---- objective helpers (gpu/mesh.py:176-206)
    def _L2norm_fn(self, J):
        def f(U):
            V = U - torch.eye(self.N, dtype=self.dtype, device=self.device)
            if not self.is_phase:
                V = V - torch.diag(torch.diagonal(V))
            J[0] = torch.linalg.norm(V) ** 2
            return 2 * V
        return f

    def L2norm(self, U_target, p_phase=None, p_splitter=None):
        J = [0]
        f = self._L2norm_fn(J)
        f(self.dot(_adjoint(U_target, self), p_phase, p_splitter))
        return J[0]

    def grad_phi_target(self, U_target, p_phase=None, p_splitter=None):
        J = [0]
        f = self._L2norm_fn(J)
        grad = self.grad_phi(_adjoint(U_target, self), f, p_phase, p_splitter)[0]
        return J[0], grad

    # ---- back-propagation (gpu/mesh.py:208-234)
    def grad_phi(self, v, dJdv, p_phase=None, p_splitter=None, out_dp=None, out_dJdv=None, vpos="in"):
        """Returns (dJ/dp, dJ/dv_in*) for J(v_out); dJdv is 2 dJ/dv_out* or a callable of v_out.

        ``out_dp`` given: the gradient is added to it (the reference accumulates with atomics into
        a caller-zeroed array); otherwise a fresh array is returned.  Unlike the reference, the input
        array ``v`` is never overwritten with the reconstructed input field.
        """
        assert vpos in ["in", "out"]
        if self.is_phase:
            return self._grad_screened(v, dJdv, p_phase, p_splitter, out_dp, out_dJdv, vpos)
        return self._grad_mesh(v, dJdv, p_phase, p_splitter, out_dp, out_dJdv, vpos)

    def _grad_mesh(self, v, dJdv, p_phase=None, p_splitter=None, out_dp=None, out_dJdv=None, vpos="in",
                   out_vin=None):
        lib = load()
        p, s = self._defaults(p_phase, p_splitter)
        if vpos == "in":
            v = self._dot_mesh(v, p_phase, p_splitter)
        else:
            v, _ = self._field(v)
        if callable(dJdv):
            dJdv = dJdv(v)
        B = v.shape[1]
        g, ldu_g = self._field(dJdv)
        out_dJdv, ldu_o = self._out(out_dJdv, B)
        v2, ldu_v = v, (v.stride(1) if B > 1 else self.N)
        if len({ldu_g, ldu_o, ldu_v}) > 1 or v.stride(0) != 1:
            v2 = v.t().contiguous().t()
            g = g.t().contiguous().t()
            ldu = self.N
            if ldu_o != ldu:
                res = self._grad_mesh(v2, g, p, s, out_dp=out_dp, vpos="out", out_vin=out_vin)
                out_dJdv.copy_(res[1])
                return res[0], out_dJdv
        else:
            ldu = ldu_o
        accumulate = 1 if out_dp is not None else 0
        if out_dp is None:
            out_dp = torch.empty(p.numel(), dtype=torch.float32, device=self.device)
        else:
            assert isinstance(out_dp, torch.Tensor) and out_dp.numel() == p.numel() and out_dp.is_contiguous()
        pptr, ldp, sptr, lds = self._ps_args(p, s)
        if out_vin is not None:
            assert out_vin.shape == (self.N, B) and out_vin.stride(0) == 1 and (B == 1 or out_vin.stride(1) == ldu)
        if self.perm_table is not None:
            if B == 0:
                if not accumulate:
                    out_dp.zero_()
                return out_dp, out_dJdv
            ws, wsn = self._programmed(OP_BWD, p, s, B)
            check(lib.mg_propagate(OP_BWD, self.N, self.L, B, self.crossing, self.geo_code, v2.data_ptr(), g.data_ptr(),
                                   None if out_vin is None else out_vin.data_ptr(), out_dJdv.data_ptr(), ldu,
                                   out_dp.data_ptr(), ldp, accumulate, None, ws, wsn, _stream(self.device)),
                  "mg_propagate")
            return out_dp, out_dJdv
        wsb = lib.mg_workspace_bytes(OP_BWD, self.N, self.L, B, self.crossing, self.geometry, None)
        ws, wsn = self._ws[OP_BWD].get(wsb)
        fn = lib.mg_backdiff_ft if self.geometry == GEO_FFT else lib.mg_backdiff
        check(fn(self.N, self.L, B, *self._geo_args(), pptr, out_dp.data_ptr(), ldp, sptr, lds, v2.data_ptr(),
                 g.data_ptr(), None if out_vin is None else out_vin.data_ptr(), out_dJdv.data_ptr(), ldu,
                 self.crossing, accumulate, ws, wsn, _stream(self.device)), fn.__name__)
        return out_dp, out_dJdv

    # ---- phase screen: is_phase with phi_pos 'in' (y = U D v) or 'out' (y = D U v), D = diag(exp(i ph)),
    # the screen step of the reference CPU path (c/dot.cpp:97-143, mesh.py:335-341)
    def _fresh(self, v) -> torch.Tensor:
        """(N, B) field as a view of a (B, N) row-major tensor (leading dimension N)."""
        v, ldu = self._field(v)
        return v if (ldu == self.N and v.stride(0) == 1) else v.t().contiguous().t()

    def _screen(self, ph, sign, u, du=None, dph=None, inplace=False):
        """exp(i sign ph) u (and its derivative along dph) on fields with leading dimension N."""
        B = u.shape[1]
        out = u if inplace else self._out(None, B)[0]
        dout = None
        if du is not None or dph is not None:
            dout = du if (inplace and du is not None) else self._out(None, B)[0]
        ptr = (lambda t: None if t is None else t.data_ptr())
        check(load().mg_phase_screen(self.N, B, ph.data_ptr(), ptr(dph), sign, u.data_ptr(), out.data_ptr(), ptr(du),
                                     ptr(dout), self.N, _stream(self.device)), "mg_phase_screen")
        return out, dout

    def _dot_screened(self, v, p_phase, p_splitter, dp, dv, out, dout):
        p, s = self._defaults(p_phase, p_splitter)
        ph = p[self.n_cr * self.X_np:]
        dpp = None if dp is None else self._param(dp).reshape(-1)
        if dpp is not None and dpp.numel() == 0:
            dpp = None
        if dpp is not None:
            assert dpp.numel() == p.numel()
        dph = None if dpp is None else dpp[self.n_cr * self.X_np:]
        diff = dpp is not None or dv is not None
        if self.phi_pos == "in":
            u, du = self._screen(ph, 1, self._fresh(v), None if dv is None else self._fresh(dv), dph)
            if diff:
                return self._dot_mesh(u, p, s, dp=dpp, dv=du, out=out, dout=dout)
            return self._dot_mesh(u, p, s, out=out)
        if diff:
            y, dy = self._dot_mesh(v, p, s, dp=dpp, dv=dv)
            y, dy = self._screen(ph, 1, y, dy, dph, inplace=True)
        else:
            y, dy = self._screen(ph, 1, self._dot_mesh(v, p, s), inplace=True)
        if out is not None:
            out.copy_(y)
            y = out
        if diff and dout is not None:
            dout.copy_(dy)
            dy = dout
        return (y, dy) if diff else y

    def _grad_screened(self, v, dJdv, p_phase, p_splitter, out_dp, out_dJdv, vpos):
        lib = load()
        p, s = self._defaults(p_phase, p_splitter)
        ncp = self.n_cr * self.X_np
        ph = p[ncp:]
        y = self._dot_screened(v, p, s, None, None, None, None) if vpos == "in" else self._fresh(v)
        if callable(dJdv):
            dJdv = dJdv(y)
        g = self._fresh(dJdv)
        B = y.shape[1]
        accumulate = 1 if out_dp is not None else 0
        if out_dp is None:
            out_dp = torch.zeros(p.numel(), dtype=torch.float32, device=self.device)
        else:
            assert isinstance(out_dp, torch.Tensor) and out_dp.numel() == p.numel() and out_dp.is_contiguous()
        dph = out_dp[ncp:]
        stream = _stream(self.device)
        if self.phi_pos == "out":
            check(lib.mg_phase_screen_grad(self.N, B, y.data_ptr(), g.data_ptr(), self.N, dph.data_ptr(), accumulate,
                                           stream), "mg_phase_screen_grad")
            ym, _ = self._screen(ph, -1, y)
            gm, _ = self._screen(ph, -1, g)
            _, gx = self._grad_mesh(ym, gm, p, s, out_dp=out_dp, vpos="out")
        else:
            vin = self._out(None, B)[0]
            _, gm = self._grad_mesh(y, g, p, s, out_dp=out_dp, vpos="out", out_vin=vin)
            check(lib.mg_phase_screen_grad(self.N, B, vin.data_ptr(), gm.data_ptr(), self.N, dph.data_ptr(),
                                           accumulate, stream), "mg_phase_screen_grad")
            gx, _ = self._screen(ph, -1, gm, inplace=True)
        if out_dJdv is not None:
            out_dJdv.copy_(gx)
            gx = out_dJdv
        return out_dp, gx

    def matrix(self, p_phase=None, p_splitter=None):
        return self.dot(torch.eye(self.N, dtype=self.dtype, device=self.device), p_phase, p_splitter)

    # ---- finite-difference Hessians (gpu/mesh.py:236-288)
    def hvp(self, vec, v, w: Callable, p_phase=None, p_splitter=None, eps=1e-3):
        p = self.p_phase if p_phase is None else self._param(p_phase).reshape(-1)
        vec = self._param(vec).reshape(-1)
        return (self.grad_phi(v, w, p + vec * eps, p_splitter)[0] - self.grad_phi(v, w, p - vec * eps, p_splitter)[0]) / (
            2 * eps)

    def hvp_target(self, vec, U_target, p_phase=None, p_splitter=None, eps=1e-3):
        J = [0]
        w = self._L2norm_fn(J)
        return self.hvp(vec, _adjoint(U_target, self), w, p_phase, p_splitter, eps)

    def hess(self, v, w: Callable, p_phase=None, p_splitter=None, eps=1e-3):
        vec = torch.eye(self.n_phase, device=self.device)
        return torch.stack([self.hvp(vi, v, w, p_phase, p_splitter, eps) for vi in vec])

    def hess_target(self, U_target, p_phase=None, p_splitter=None, eps=1e-3):
        vec = torch.eye(self.n_phase, device=self.device)
        return torch.stack([self.hvp_target(vi, U_target, p_phase, p_splitter, eps) for vi in vec])

    def status(self, clear=True) -> int:
        """Run-time status recorded by the kernels (0 ok, 1 timeout, 2 bad geometry) in the workspaces of
        the drop-in methods and of the autograd function (``mesh_apply``); synchronises."""
        rc = max((ws.status(clear) for ws in self._ws.values()), default=0)
        for plan in getattr(self, "_autograd_plans", {}).values():
            if plan.buf is not None:
                v = load().mg_read_status(plan.buf.data_ptr(), int(clear), _stream(self.device))
                if v < 0:
                    check(v, "mg_read_status")
                rc = max(rc, v)
        return rc


def _perm_rows(perm, N: int, L: int):
    """(L+1, N) int32 gather rows of the reference's ``perm`` list (None rows are the identity), or
    (None, None) when no row moves anything."""
    if perm is None:
        return None, None
    rows = list(perm)
    assert len(rows) == L + 1, "perm needs L+1 = %d entries (mesh.py:277)" % (L + 1)
    if all(r is None for r in rows):
        return None, None
    out = np.empty((L + 1, N), dtype=np.int32)
    for k, r in enumerate(rows):
        out[k] = np.arange(N) if r is None else np.asarray(r).reshape(-1)
        assert np.array_equal(np.sort(out[k]), np.arange(N)), "perm[%d] is not a permutation of 0..N-1" % k
    if all(np.array_equal(r, np.arange(N)) for r in out):
        return None, None
    return out, out


def _numel(x) -> int:
    return int(x.numel()) if isinstance(x, torch.Tensor) else int(np.asarray(x).size)


def _adjoint(U, mesh: MeshNetworkGPU) -> torch.Tensor:
    if not isinstance(U, torch.Tensor):
        U = torch.as_tensor(np.asarray(U))
    return U.to(device=mesh.device, dtype=mesh.dtype).t().conj()


def from_structured(net, device=None) -> MeshNetworkGPU:
    """Counterpart of the reference ``StructuredMeshNetwork.gpu()`` (mesh.py:568-579).

    ``net`` is any object exposing N, L, lens, shifts, grid_phase, grid_splitter, X and perm (the
    reference's StructuredMeshNetwork, ClementsNetwork, ReckNetwork, ButterflyNetwork, ...).  Unlike
    the reference, which refuses them (mesh.py:573), permutations between layers and a phase screen
    (is_phase) convert too; a reference ButterflyNetwork (permutations around adjacent-pair layers)
    becomes the equivalent stride geometry, which needs no permutations.  A ClippedNetwork
    (SquareNetwork, QRNetwork, PilossNetwork) becomes a ClippedMeshGPU around its converted full mesh.
    """
    if hasattr(net, "full") and hasattr(net, "idx_in"):     # ClippedNetwork, SquareNetwork, QRNetwork
        from .clipped import ClippedMeshGPU
        return ClippedMeshGPU(from_structured(net.full, device), net.idx_in, net.idx_out)
    name = type(net.X).__name__
    N, L = int(net.N), int(net.L)
    if name not in ("MZICrossing", "SymCrossing"):
        return _from_structured_generic(net, name, device)
    X = {"MZICrossing": "mzi", "SymCrossing": "sym"}[name]
    n_p, n_s = _NP_NS[X]
    p = np.nan_to_num(np.asarray(net.grid_phase, dtype=np.float32))
    s = np.nan_to_num(np.asarray(net.grid_splitter, dtype=np.float32))
    perm = list(net.perm)
    is_phase = bool(getattr(net, "is_phase", False))
    if type(net).__name__ == "ButterflyNetwork" and not is_phase and any(x is not None for x in perm):
        strides = geom.butterfly(N)
        return MeshNetworkGPU(N, L, None, None, p, s if s.size else None, X, is_phase=False, strides=strides,
                              device=device)
    if is_phase:
        # the phase screen rides along (the reference's gpu() refuses it, gpu/mesh.py:65)
        ph = np.asarray(net.phi_out, dtype=np.float32).reshape(-1)
        return MeshNetworkGPU(N, L, np.array(net.lens), np.array(net.shifts),
                              np.concatenate([p.reshape(-1), ph]), s if s.size else None, X,
                              phi_pos=net.phi_pos, is_phase=True, device=device, perm=perm)
    return MeshNetworkGPU(N, L, np.array(net.lens), np.array(net.shifts), p, s if s.size else None, X,
                          phi_pos="out", is_phase=False, device=device, perm=perm)


def _from_structured_generic(net, name: str, device=None):
    """A StructuredMeshNetwork of another crossing class (crossing.py:292-611) as a lossy.GenericMeshGPU:
    T(p, s) per slot on the generic precomputed-T path (float64 parameters, as the reference keeps them)."""
    from .crossings import CLASS_NAMES
    from .lossy import GenericMeshGPU
    if name not in CLASS_NAMES:
        raise ValueError("crossing class %s has no GPU counterpart" % name)
    if any(x is not None for x in net.perm):
        raise ValueError("meshes of generic crossings take no permutations")
    X = CLASS_NAMES[name]
    N, L = int(net.N), int(net.L)
    p = np.nan_to_num(np.asarray(net.grid_phase, dtype=np.float64)).reshape(-1)
    sp = np.asarray(net.grid_splitter, dtype=np.float64)
    is_phase = bool(getattr(net, "is_phase", False))
    if is_phase:
        p = np.concatenate([p, np.asarray(net.phi_out, dtype=np.float64).reshape(-1)])
    return GenericMeshGPU(N, L, np.array(net.lens), np.array(net.shifts), p,
                          np.nan_to_num(sp) if sp.size else None, X, phi_pos=net.phi_pos, is_phase=is_phase,
                          device=device)
