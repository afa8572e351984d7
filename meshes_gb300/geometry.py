"""Mesh geometries in the layout the kernels consume.

Nearest-neighbour meshes are described by per-layer (lens, shifts): layer l holds lens[l] MZIs
coupling modes (shifts[l] + 2k, shifts[l] + 2k + 1).  Butterfly meshes are described by per-layer
stride exponents: layer l with stride s = 2^strides[l] couples modes (2s*(q//s) + q%s, + s) for every
slot q < N/2.  Parameters live in the reference GPU grid (gpu/mesh.py:77-81): p[l, q, k] with slot
q = shifts[l]//2 + k for nearest-neighbour layers (mesh.py:513-536).
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np


def clements(N: int) -> Tuple[List[int], List[int]]:
    """Clements rectangle, N layers (reference clements.py:56-57)."""
    return [(N - n % 2) // 2 for n in range(N)], [n % 2 for n in range(N)]


def reck(N: int) -> Tuple[List[int], List[int]]:
    """Reck triangle, 2N-3 layers (reference reck.py:47-48)."""
    shifts = list(range(N - 2, 0, -1)) + list(range(0, N - 1))
    return [(N - s) // 2 for s in shifts], shifts


def fft(N: int) -> List[int]:
    """log2(N)-layer FFT butterfly: stride exponents 0, 1, ..., log2(N)-1."""
    n = int(round(math.log2(N)))
    if 1 << n != N:
        raise ValueError("butterfly meshes need N a power of two, got %d" % N)
    return list(range(n))


def butterfly(N: int) -> List[int]:
    """The reference ButterflyNetwork's N-1 layers (butterfly.py:47-51) as stride exponents.

    The reference applies adjacent-pair layers between permutations; its odd layer i acts on modes
    (2s*j + k, 2s*j + k + s) with s the lowest set bit of i+1, even layers on adjacent pairs.
    """
    fft(N)
    out = []
    for i in range(N - 1):
        x = i + 1
        out.append(0 if i % 2 == 0 else (x & -x).bit_length() - 1)
    return out


def active_mask_nn(N: int, lens: Sequence[int], shifts: Sequence[int]) -> np.ndarray:
    m = np.zeros((len(lens), N // 2), dtype=bool)
    for l, (ln, sh) in enumerate(zip(lens, shifts)):
        m[l, sh // 2: sh // 2 + ln] = True
    return m


def validate_nn(N: int, lens: Sequence[int], shifts: Sequence[int]):
    if len(lens) != len(shifts):
        raise ValueError("lens and shifts differ in length")
    for l, (ln, sh) in enumerate(zip(lens, shifts)):
        if ln < 0 or sh < 0 or sh + 2 * ln > N:
            raise ValueError("layer %d: shift %d + 2*len %d exceeds N=%d" % (l, sh, ln, N))


def validate_fft(N: int, strides: Sequence[int]):
    for l, e in enumerate(strides):
        if e < 0 or (2 << int(e)) > N or N % (2 << int(e)):
            raise ValueError("layer %d: stride 2^%d invalid for N=%d" % (l, e, N))


def flat_to_grid(flat, lens, shifts, N: int, n: int) -> np.ndarray:
    """Reference CPU parameters p_crossing (n_cr, n) -> GPU grid (L, N//2, n), zeros elsewhere
    (mesh.py:513-536 with NaN -> 0 as in mesh.py:575-576)."""
    flat = np.asarray(flat).reshape(-1, n)
    out = np.zeros((len(lens), N // 2, n), dtype=flat.dtype)
    ind = 0
    for l, (ln, sh) in enumerate(zip(lens, shifts)):
        out[l, sh // 2: sh // 2 + ln] = flat[ind: ind + ln]
        ind += ln
    return out


def grid_to_flat(grid, lens, shifts) -> np.ndarray:
    return np.concatenate([np.asarray(grid)[l, sh // 2: sh // 2 + ln] for l, (ln, sh) in enumerate(zip(lens, shifts))], 0)
