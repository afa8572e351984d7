"""Transfer matrices of the reference's crossing parameterisations as differentiable torch functions.

``transfer(name, p, s)`` returns T (..., 2, 2) complex for phases p (..., n_phase) and splitter/error
parameters s (..., n_splitter) (None = ideal), in the dtype of p (complex128 for float64).  Gradients reach
p and s through PyTorch's autograd, so any of these crossings runs on the generic precomputed-T path of the
GPU kernels (``lossy.LossyMesh``, ``lossy.GenericMeshGPU``) with its checkpointed adjoint.

Names, the reference class each restates, and its parameters:
  mzi                   MZICrossing (crossing.py:200-221)            p (theta, phi), s (alpha, beta)
  mzi_balanced          MZICrossingBalanced (crossing.py:292-305)    p (theta, phi), s (alpha, beta)
  mzi_outphase          MZICrossingOutPhase (crossing.py:318-337)    p (theta, phi), s (alpha, beta)
  sym                   SymCrossing (crossing.py:360-381)            p (theta, phi), s (alpha,)
  mzi3                  MZICrossing3 (crossing.py:384-416)           p (theta, phi), s (alpha, beta, eta)
  mzi3_outphase         MZICrossing3OutPhase (crossing.py:425-442)   p (theta, phi), s (alpha, beta, eta)
  mzi_generic           MZICrossingGeneric (crossing.py:444-488)     p (theta, phi), s (14: see lossy.mzi_generic_T)
  mzi_generic_outphase  MZICrossingGenericOutPhase (crossing.py:493-506), same parameters
  cartesian             CartesianCrossing (crossing.py:514-544)      p (x, y) in the unit disk around (+-2, 0)
  bell                  MZICrossingBell (crossing.py:570-594)        p (theta, phi), s (alpha, beta)
"""
from __future__ import annotations

import math
from typing import Optional

import torch

from .lossy import mzi_generic_T

# (n_phase, n_splitter) per crossing
SIZES = {"mzi": (2, 2), "mzi_balanced": (2, 2), "mzi_outphase": (2, 2), "sym": (2, 1), "mzi3": (2, 3),
         "mzi3_outphase": (2, 3), "mzi_generic": (2, 14), "mzi_generic_outphase": (2, 14), "cartesian": (2, 2),
         "bell": (2, 2)}

# the reference's crossing classes by name
CLASS_NAMES = {"MZICrossing": "mzi", "MZICrossingBalanced": "mzi_balanced", "MZICrossingOutPhase": "mzi_outphase",
               "SymCrossing": "sym", "MZICrossing3": "mzi3", "MZICrossing3OutPhase": "mzi3_outphase",
               "MZICrossingGeneric": "mzi_generic", "MZICrossingGenericOutPhase": "mzi_generic_outphase",
               "CartesianCrossing": "cartesian", "MZICrossingBell": "bell"}


def _mat(t00, t01, t10, t11) -> torch.Tensor:
    return torch.stack([torch.stack([t00, t01], -1), torch.stack([t10, t11], -1)], -2)


def _cis(x: torch.Tensor) -> torch.Tensor:
    return torch.complex(torch.cos(x), torch.sin(x))


def _coupler(eta: torch.Tensor) -> torch.Tensor:
    """[[cos eta, i sin eta], [i sin eta, cos eta]]."""
    c = torch.complex(torch.cos(eta), torch.zeros_like(eta))
    i_s = torch.complex(torch.zeros_like(eta), torch.sin(eta))
    return _mat(c, i_s, i_s, c)


def _s(s: Optional[torch.Tensor], p: torch.Tensor, n: int) -> torch.Tensor:
    return p.new_zeros(p.shape[:-1] + (n,)) if s is None else s.to(p.dtype).expand(p.shape[:-1] + (n,))


def _mzi(p, s):
    th, ph = p[..., 0], p[..., 1]
    s = _s(s, p, 2)
    a, b = s[..., 0], s[..., 1]
    Cp, Cm, C = torch.cos(a + b), torch.cos(a - b), torch.cos(th / 2)
    Sp, Sm, S = torch.sin(a + b), torch.sin(a - b), torch.sin(th / 2)
    e_th, e_thph = _cis(th / 2), _cis(th / 2 + ph)
    return _mat(e_thph * torch.complex(-C * Sp, S * Cm), e_th * torch.complex(-S * Sm, C * Cp),
                e_thph * torch.complex(S * Sm, C * Cp), e_th * torch.complex(-C * Sp, -S * Cm))


def _mzi_outphase(p, s):
    # the input-phase MZI with splitters (beta + pi/2, alpha - pi/2), both indices reversed and transposed
    s = _s(s, p, 2)
    Ti = _mzi(p, torch.stack([s[..., 1] + math.pi / 2, s[..., 0] - math.pi / 2], -1))
    return _mat(Ti[..., 1, 1], Ti[..., 0, 1], Ti[..., 1, 0], Ti[..., 0, 0])


def _sym(p, s):
    th, ph = p[..., 0], p[..., 1]
    al = _s(s, p, 1)[..., 0]
    C, S, C2a, S2a = torch.cos(th / 2), torch.sin(th / 2), torch.cos(2 * al), torch.sin(2 * al)
    off = torch.complex(torch.zeros_like(C), C * C2a)
    return _mat(_cis(ph) * torch.complex(S, C * S2a), off, off, _cis(-ph) * torch.complex(S, -C * S2a))


def _generic_outphase(p, s):
    s = _s(s, p, 14)
    th, ph = p[..., 0], p[..., 1]

    def ep(phase, gain):
        return torch.exp(torch.complex(gain / 2, phase))

    d1a, d1b = ep(ph + s[..., 2] + s[..., 6], s[..., 10]), ep(s[..., 3] + s[..., 7], s[..., 11])
    d2a, d2b = ep(th + s[..., 4] + s[..., 8], s[..., 12]), ep(s[..., 5] + s[..., 9], s[..., 13])
    z = torch.zeros_like(d1a)
    # diag(d1b, d1a) S(alpha) diag(d2b, d2a) S(beta)
    T = _mat(d2b, z, z, d2a) @ _coupler(math.pi / 4 + s[..., 1])
    T = _coupler(math.pi / 4 + s[..., 0]) @ T
    return _mat(d1b, z, z, d1a) @ T


def _cartesian(p, s):
    x, y = p[..., 0], p[..., 1]
    right = x > 0
    zr = torch.where(right, x - 2, x + 2)
    z = torch.complex(zr, y)
    r = torch.sqrt(torch.clamp(1 - zr * zr - y * y, min=0.0))
    ir = torch.complex(torch.zeros_like(r), r)
    return _mat(torch.where(right, z, ir), torch.where(right, ir, z),
                torch.where(right, ir, z.conj()), torch.where(right, z.conj(), ir))


def _bell(p, s):
    th, ph = p[..., 0], p[..., 1]
    s = _s(s, p, 2)
    a, b = s[..., 0], s[..., 1]
    Cp, Cm, C = torch.cos(a + b), torch.cos(a - b), torch.cos((th - ph) / 2)
    Sp, Sm, S = torch.sin(a + b), torch.sin(a - b), torch.sin((th - ph) / 2)
    e = _cis((th + ph) / 2)
    return _mat(e * torch.complex(-C * Sp, Cm * S), e * torch.complex(-Sm * S, Cp * C),
                e * torch.complex(Sm * S, Cp * C), e * torch.complex(-C * Sp, -Cm * S))


def transfer(name: str, p: torch.Tensor, s: Optional[torch.Tensor] = None) -> torch.Tensor:
    """T (..., 2, 2) of crossing ``name`` for p (..., 2) and s (..., n_splitter) or None."""
    if name not in SIZES:
        raise ValueError("unknown crossing %r (known: %s)" % (name, ", ".join(sorted(SIZES))))
    if name == "mzi":
        return _mzi(p, s)
    if name == "mzi_balanced":
        return _mzi(p, s) * _cis(-p[..., 0] / 2)[..., None, None]
    if name == "mzi_outphase":
        return _mzi_outphase(p, s)
    if name == "sym":
        return _sym(p, s)
    if name == "mzi3":
        sp = _s(s, p, 3)
        return _mzi(p, sp[..., :2]) @ _coupler(sp[..., 2])
    if name == "mzi3_outphase":
        sp = _s(s, p, 3)
        return _coupler(sp[..., 2]) @ _mzi_outphase(p, sp[..., :2])
    if name == "mzi_generic":
        return mzi_generic_T(p, None if s is None else s.to(p.dtype))
    if name == "mzi_generic_outphase":
        return _generic_outphase(p, s)
    if name == "cartesian":
        return _cartesian(p, s)
    return _bell(p, s)
