"""ctypes wrapper of the C++ port (oracle/meshdot_port.cpp): TEST INFRASTRUCTURE ONLY.

Used by tests/ to pin the port against the reference's own c/dot.cpp, and by bench.py as the timed
CPU baseline (the reference's algorithm on the host cores of the machine the benchmark runs on).
Layouts follow the reference CPU path (mesh.py:97-113): T packed (2, 2, nT) complex for the active
MZIs in layer order, fields (N, B) row-major.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from . import meshes_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libmeshdot_port.so")
REF_LIB = os.path.join(HERE, "_ref", "dot.so")
_ARGT = (ctypes.c_int,) * 4 + (ctypes.c_void_p,) * 10 + (ctypes.c_int,) * 4


def _load(path, names):
    lib = ctypes.CDLL(path)
    fns = []
    for n in names:
        f = getattr(lib, n)
        f.argtypes = _ARGT
        f.restype = None
        fns.append(f)
    return fns


_port = None


def port_lib():
    """(meshdot_port32, meshdot_port64), building the port first if needed."""
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
        _port = _load(PORT_LIB, ["meshdot_port32", "meshdot_port64"])
    return _port


def ref_lib():
    """(meshdot_helper32, meshdot_helper64) of the reference's own c/dot.cpp, or None if not built."""
    if not os.path.exists(REF_LIB):
        return None
    return _load(REF_LIB, ["meshdot_helper32", "meshdot_helper64"])


def call(fns, T, dT, ph, dph, v, dv, inds, lens, shifts, perms, pos, mode, threads):
    """Same contract as the reference meshdot_helper_c (mesh.py:97-113); arrays updated in place."""
    is64 = v.dtype == np.complex128
    fn = fns[1 if is64 else 0]
    N = v.shape[0]
    B = v.size // N
    for a in (T, dT, v, dv, ph, dph):
        assert a.flags.c_contiguous
    # hold the int arrays in locals: a temporary's .ctypes.data would dangle during the call
    inds_ = np.ascontiguousarray(inds, np.int32)
    lens_ = np.ascontiguousarray(lens, np.int32)
    shifts_ = np.ascontiguousarray(shifts, np.int32)
    perms_ = np.ascontiguousarray(perms, np.int32)
    fn(N, B, T.shape[2], len(lens_), T.ctypes.data, dT.ctypes.data, ph.ctypes.data, dph.ctypes.data, v.ctypes.data,
       dv.ctypes.data, inds_.ctypes.data, lens_.ctypes.data, shifts_.ctypes.data, perms_.ctypes.data,
       int(perms_.size), pos, mode, threads)


def packed_T(om: "O.OracleMesh", dtype=np.complex128):
    """(T (2,2,nT), inds) of a nearest-neighbour oracle mesh in the reference CPU layout."""
    Tg = om.T_grid()
    mats, inds = [], [0]
    for n in range(om.L):
        q, _, _ = O._layer_index(om, n)
        mats.append(Tg[n, q])
        inds.append(inds[-1] + len(q))
    T = np.concatenate(mats, 0).transpose(1, 2, 0)
    return np.ascontiguousarray(T.astype(dtype)), np.array(inds[:-1], np.int32)


def forward(fns, om, x, threads=1, dtype=np.complex64):
    """y (B, N) = U x through the C path, no phase screen, no permutations."""
    T, inds = packed_T(om, dtype)
    v = np.ascontiguousarray(np.asarray(x).T.astype(dtype))
    rdt = np.float32 if dtype == np.complex64 else np.float64
    e = np.empty(0, dtype)
    call(fns, T, e.reshape(0, 0, 0), np.empty(0, rdt), np.empty(0, rdt), v, e.reshape(0, 0), inds, om.lens,
         om.shifts, np.empty((0, 0), np.int32), -1, 0, threads)
    return v.T


def vjp(fns, om, y, g, threads=1, dtype=np.complex64):
    """(dJ/dT (L, N//2, 2, 2) grid, g_in (B, N)) through mode 2 of the C path."""
    T, inds = packed_T(om, dtype)
    v = np.ascontiguousarray(np.asarray(y).T.astype(dtype))
    dv = np.ascontiguousarray(np.asarray(g).T.astype(dtype))
    dT = np.zeros_like(T)
    rdt = np.float32 if dtype == np.complex64 else np.float64
    call(fns, T, dT, np.empty(0, rdt), np.empty(0, rdt), v, dv, inds, om.lens, om.shifts,
         np.empty((0, 0), np.int32), -1, 2, threads)
    G = np.zeros((om.L, om.N // 2, 2, 2), dtype=np.complex128)
    k = 0
    for n in range(om.L):
        q, _, _ = O._layer_index(om, n)
        G[n, q] = dT[:, :, k:k + len(q)].transpose(2, 0, 1)
        k += len(q)
    return G, dv.T
