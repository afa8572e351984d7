"""MeshOptimizer: fit a mesh to a target matrix with scipy, gradients from the GPU adjoint.

Counterpart of the reference's ``meshes/gpu/opt.py`` (``MeshOptimizer``, opt.py:16-68).  The objective
is the reference's ``L2norm`` of the programmed mesh against a target U (gpu/mesh.py:176-206): J =
||M U^H - I||_F^2, diagonal excluded when the mesh has no phase screen.  The optimisation variables
are the crossing phases of the active slots only, in the reference's flat order (layer by layer, slot
by slot; ``StructuredMeshNetwork.p_crossing``).  ``jac`` runs one forward and one back-propagation
launch (``MeshNetworkGPU.grad_phi_target``) and caches J; ``run`` hands scipy the value and the gradient
from that one call.
"""
from __future__ import annotations

from time import time
from typing import List, Optional

import numpy as np
import torch

from .mesh import MeshNetworkGPU, from_structured


class MeshOptimizer:
    def __init__(self, mesh, U):
        """mesh: a MeshNetworkGPU, or a reference StructuredMeshNetwork (converted like mesh.gpu(), the
        phase screen switched off as opt.py:26-27 does); U: the (N, N) target matrix."""
        if not isinstance(mesh, MeshNetworkGPU):
            mesh = from_structured(mesh)
        self.mesh = mesh
        N, L, n_p = mesh.N, mesh.L, mesh.X_np
        if mesh.strides is None:
            rows = [np.arange(l * (N // 2) + sh // 2, l * (N // 2) + sh // 2 + ln)
                    for l, (ln, sh) in enumerate(zip(mesh.lens_h, mesh.shifts_h))]
        else:
            rows = [np.arange(l * (N // 2), (l + 1) * (N // 2)) for l in range(L)]
        self._inds = np.concatenate(rows) if rows else np.zeros(0, dtype=np.int64)
        self._inds_t = torch.as_tensor(self._inds, device=mesh.device)
        grid = mesh.p_crossing.reshape(-1, n_p)
        self.p = grid[self._inds_t].reshape(-1).cpu().numpy().astype(np.float64)
        self.U = torch.as_tensor(np.asarray(U), dtype=mesh.dtype, device=mesh.device)
        self._cache_key: Optional[bytes] = None
        self._cache_J = 0.0
        self.yt: List[float] = []
        self.t: List[float] = []

    # flat active-slot parameters <-> the GPU parameter grid (inactive slots 0)
    def _to_gpu(self, p: np.ndarray) -> torch.Tensor:
        m = self.mesh
        out = torch.zeros((m.n_cr, m.X_np), dtype=torch.float32, device=m.device)
        out[self._inds_t] = torch.as_tensor(np.asarray(p, np.float32).reshape(-1, m.X_np), device=m.device)
        return out.reshape(-1)

    def _from_gpu(self, dp: torch.Tensor) -> np.ndarray:
        return dp.reshape(self.mesh.n_cr, self.mesh.X_np)[self._inds_t].reshape(-1).cpu().numpy()

    def f(self, p: np.ndarray) -> float:
        key = np.asarray(p, np.float64).tobytes()
        if key == self._cache_key:
            return self._cache_J
        return float(self.mesh.L2norm(self.U, self._to_gpu(p)))

    def jac(self, p: np.ndarray) -> np.ndarray:
        J, dp = self.mesh.grad_phi_target(self.U, self._to_gpu(p))
        self._cache_key = np.asarray(p, np.float64).tobytes()
        self._cache_J = float(J)
        return self._from_gpu(dp)

    def run(self, method: str, p: Optional[np.ndarray] = None, tol: float = 1e-5, maxiter: int = 10000,
            tick: int = -1):
        """scipy.optimize.minimize(method=...) from p (default: the mesh's phases); the result carries the
        trace yt = sqrt(J / N) and wall-clock times t, as opt.py:47-68."""
        from scipy.optimize import minimize
        p = self.p if p is None else np.asarray(p, np.float64)
        self.yt, self.t = [], []
        t0 = time()

        def fun(x):
            out = self.f(x)
            self.yt.append(out)
            self.t.append(time() - t0)
            if tick > 0 and len(self.yt) % tick == 0:
                print(".", end="", flush=True)
            return np.float64(out)

        def fun_and_jac(x):                            # one forward + back-propagation per point
            g = self.jac(x).astype(np.float64)
            return fun(x), g

        res = minimize(fun=fun_and_jac, x0=p, jac=True, method=method, tol=tol, options={"maxiter": maxiter})
        if tick > 0:
            print()
        res.yt = self.yt = np.sqrt(np.asarray(self.yt)) / np.sqrt(len(self.U))
        res.t = self.t = np.asarray(self.t)
        return res
