"""Clipped meshes: a mesh of which only some input and output ports are used (reference mesh.py:718-802).

The reference's ``ClippedNetwork`` (and the SquareNet and QR meshes built on it, square.py, qr.py)
embeds an (N_in, B) input into the full mesh's ports ``idx_in`` (zeros elsewhere), propagates through
the full mesh and keeps the output ports ``idx_out``.  ``ClippedMeshGPU`` does the same around a
``MeshNetworkGPU`` (with its phase screen, if the full mesh has one), including the L2 objective
against an (M_out, N_in) target and its gradient (``grad_L2``, mesh.py:787-802).
"""
from __future__ import annotations

from typing import Tuple

import numpy as np
import torch

from .mesh import MeshNetworkGPU


def _index(idx, n: int) -> torch.Tensor:
    return torch.as_tensor(np.arange(n)[idx] if isinstance(idx, slice) or idx is None else np.asarray(idx),
                           dtype=torch.long)


class ClippedMeshGPU:
    def __init__(self, full: MeshNetworkGPU, idx_in=None, idx_out=None):
        self.full = full
        self.idx_in = _index(slice(None) if idx_in is None else idx_in, full.N).to(full.device)
        self.idx_out = _index(slice(None) if idx_out is None else idx_out, full.N).to(full.device)

    @property
    def N(self) -> int:
        return int(self.idx_in.numel())

    @property
    def M(self) -> int:
        return int(self.idx_out.numel())

    def _to_full(self, v: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
        V = torch.zeros((self.full.N,) + tuple(v.shape[1:]), dtype=self.full.dtype, device=self.full.device)
        V[idx] = v.to(device=self.full.device, dtype=self.full.dtype)
        return V

    def dot(self, v, p_phase=None, p_splitter=None) -> torch.Tensor:
        """(M_out, B) outputs for (N_in, B) inputs (reference ClippedNetwork.dot, mesh.py:783-785)."""
        v = torch.as_tensor(np.asarray(v)) if not isinstance(v, torch.Tensor) else v
        return self.full.dot(self._to_full(v, self.idx_in), p_phase, p_splitter)[self.idx_out]

    def matrix(self, p_phase=None, p_splitter=None) -> torch.Tensor:
        return self.dot(torch.eye(self.N, dtype=self.full.dtype, device=self.full.device), p_phase, p_splitter)

    def grad_L2(self, U_target, p_phase=None, p_splitter=None) -> Tuple[float, torch.Tensor]:
        """J = ||U[idx_out] - U_target||_F^2 and dJ/dp over the full mesh's parameters (crossings, then
        the phase screen if any), as ClippedNetwork.grad_L2 (mesh.py:787-802)."""
        Ut = torch.as_tensor(np.asarray(U_target)) if not isinstance(U_target, torch.Tensor) else U_target
        Ut = Ut.to(device=self.full.device, dtype=self.full.dtype)
        E = self._to_full(torch.eye(self.N, dtype=self.full.dtype, device=self.full.device), self.idx_in)
        J = [0.0]

        def f(U):
            dU = U[self.idx_out] - Ut
            J[0] = float(torch.linalg.norm(dU) ** 2)
            return self._to_full(2 * dU, self.idx_out)

        dp, _ = self.full.grad_phi(E, f, p_phase, p_splitter)
        return J[0], dp
