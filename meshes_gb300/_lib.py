"""ctypes binding of libmeshes_gb300.so (the C ABI declared in include/meshes_gb300.h).

The library is the only compute path: if it is missing or fails to load, every call raises
``MeshLibraryError``.  There is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
from ctypes import POINTER, Structure, c_char_p, c_double, c_float, c_int, c_size_t, c_uint, c_ulonglong, c_void_p

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libmeshes_gb300.so")

MZI, SYM, ORTH, GENERIC = 0, 1, 2, 3
OP_FWD, OP_FWDDIFF, OP_BWD, OP_FWD_BWDTILES, OP_BWD_STORED = 0, 1, 2, 3, 4
GEO_NN, GEO_FFT = 0, 1
GEO_PERM = 4          # OR-ed into a geometry: permutations between layers (mg_build_perms)
BATCH_NN = 16         # OR-ed into mg_batched_propagate's op: all meshes nearest-neighbour
CROSSING_CODES = {"mzi": MZI, "sym": SYM, "orth": ORTH, "generic": GENERIC}
STATUS_NAMES = {0: "ok", 1: "timeout", 2: "bad geometry", 3: "bad work item"}


class MeshLibraryError(RuntimeError):
    pass


class mg_config(Structure):
    _fields_ = [("M", c_int), ("V", c_int), ("W", c_int), ("CL", c_int), ("S", c_int), ("split", c_int)]

    def as_tuple(self):
        return (self.M, self.V, self.W, self.CL, self.S, self.split)


class mg_plan_info(Structure):
    _fields_ = [("M", c_int), ("V", c_int), ("W", c_int), ("CL", c_int), ("S", c_int), ("G", c_int),
                ("grid", c_int), ("nA", c_int), ("layer_bytes", c_uint), ("dlayer_bytes", c_uint), ("smem", c_size_t),
                ("off_kinds", c_size_t), ("off_tiles", c_size_t), ("off_dtiles", c_size_t),
                ("off_partial", c_size_t), ("total", c_size_t)]


class mg_batch_mesh(Structure):
    _fields_ = [("N", c_int), ("L", c_int), ("B", c_int), ("ldu", c_int), ("cls", c_int), ("G", c_int),
                ("CL", c_int), ("S", c_int), ("layer_bytes", c_uint), ("n_items", c_int), ("ldp", c_int),
                ("n_p", c_int), ("tiles", c_void_p), ("kinds", c_void_p), ("in0", c_void_p), ("in1", c_void_p),
                ("out0", c_void_p), ("out1", c_void_p), ("dp", c_void_p), ("partial", c_void_p)]


class mg_server_mesh(Structure):
    _fields_ = [("N", c_int), ("L", c_int), ("cls", c_int), ("G", c_int), ("n_p", c_int), ("cap", c_int),
                ("fwd_CL", c_int), ("fwd_S", c_int), ("bwd_CL", c_int), ("bwd_S", c_int),
                ("fwd_layer_bytes", c_uint), ("bwd_layer_bytes", c_uint), ("fwd_tiles", c_void_p),
                ("fwd_kinds", c_void_p), ("bwd_tiles", c_void_p), ("bwd_kinds", c_void_p)]


class mg_batch_item(Structure):
    _fields_ = [("mesh", c_int), ("v0", c_int), ("vend", c_int), ("part", c_int)]


_SIGS = {
    "mg_last_error": (c_char_p, []),
    "mg_version": (c_char_p, []),
    "mg_workspace_bytes": (c_size_t, [c_int, c_int, c_int, c_int, c_int, c_int, POINTER(mg_config)]),
    "mg_workspace_init": (c_int, [c_void_p, c_size_t, c_void_p]),
    "mg_read_status": (c_int, [c_void_p, c_int, c_void_p]),
    "mg_default_config": (c_int, [c_int, c_int, c_int, c_int, POINTER(mg_config)]),
    "mg_set_tuned": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, POINTER(mg_config)]),
    "mg_fwdprop": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                           c_void_p, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_fwdprop_noalloc": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int,
                                   c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "mg_fwdprop_ft": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p,
                              c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_fwddiff": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int,
                           c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_fwddiff_ft": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                              c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_backdiff": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int,
                            c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_size_t,
                            c_void_p]),
    "mg_backdiff_ft": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                               c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_build_tiles": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_int,
                               c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int, POINTER(mg_config), c_void_p,
                               c_size_t, c_void_p]),
    "mg_autotune": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                            c_void_p, c_int, c_int, c_int, POINTER(mg_config), POINTER(c_float), POINTER(mg_config),
                            POINTER(c_float), c_int, POINTER(c_int), c_void_p]),
    "mg_build_perms": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, POINTER(mg_config), c_void_p,
                               c_size_t, c_void_p]),
    "mg_propagate": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                             c_void_p, c_int, c_int, POINTER(mg_config), c_void_p, c_size_t, c_void_p]),
    "mg_propagate_l2": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                c_void_p, c_int, c_int, POINTER(mg_config), c_void_p, c_size_t, c_void_p]),
    "mg_propagate_range": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p,
                                   c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int, POINTER(mg_config), c_void_p,
                                   c_size_t, c_void_p]),
    "mg_phase_screen": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int,
                                c_void_p]),
    "mg_phase_screen_grad": (c_int, [c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "mg_server_create": (c_void_p, [c_void_p, c_int, c_size_t, c_int, c_int, c_int, c_size_t, c_size_t, c_int]),
    "mg_server_request_bytes": (c_int, [c_void_p, c_int, c_int, c_int, POINTER(c_size_t)]),
    "mg_server_submit": (c_int, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 ctypes.c_ulonglong]),
    "mg_server_wait": (c_int, [c_void_p, c_void_p, c_int, c_int]),
    "mg_server_stats": (c_int, [c_void_p, c_void_p]),
    "mg_server_status": (c_int, [c_void_p]),
    "mg_server_destroy": (None, [c_void_p, c_int]),
    "mg_lossy_forward": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p,
                                 c_size_t, c_void_p]),
    "mg_lossy_backward": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_void_p, c_void_p, c_int, c_void_p, c_size_t, c_void_p, c_size_t, c_void_p]),
    "mg_generic_mzi_T": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mg_generic_mzi_T_vjp": (c_int, [c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mg_propagate_wait_test": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_int, c_ulonglong, c_int, c_void_p, c_size_t, c_void_p]),
    "mg_diag_configure": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int,
                                  c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_int]),
    "mg_direct_configure": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
    "mg_adam_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double, c_double, c_double, c_double,
                             c_void_p, c_void_p]),
    "mg_fma_probe": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p]),
    "mg_fma2_probe": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p]),
    "mg_trig_check": (c_int, [c_void_p, c_void_p, c_int, c_void_p]),
    "mg_plan": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, POINTER(mg_config), POINTER(mg_plan_info)]),
    # mesh and item arrays live in device memory: passed as raw addresses
    "mg_batched_propagate": (c_int, [c_int, c_void_p, c_int, c_void_p, c_int, c_void_p, c_int, c_size_t, c_void_p,
                                     c_void_p]),
    "mg_batched_reduce": (c_int, [c_void_p, c_int, c_void_p]),
}

_lock = threading.Lock()
_lib = None


def load(path: str = LIB_PATH):
    """Load (once) and return the ctypes library handle."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise MeshLibraryError(
                    "libmeshes_gb300.so is not built (%s); run `python -m meshes_gb300.build`" % path)
            try:
                lib = ctypes.CDLL(path)
            except OSError as e:   # pragma: no cover - exercised only on broken installs
                raise MeshLibraryError("cannot load %s: %s" % (path, e)) from e
            for name, (res, args) in _SIGS.items():
                try:
                    f = getattr(lib, name)
                except AttributeError as e:
                    raise MeshLibraryError("%s lacks %s (built from older sources); rebuild with "
                                           "`python -m meshes_gb300.build`" % (path, name)) from e
                f.restype = res
                f.argtypes = args
            _lib = lib
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def last_error() -> str:
    return (load().mg_last_error() or b"").decode()


def check(rc: int, what: str):
    if rc != 0:
        raise MeshLibraryError("%s failed (rc=%d): %s" % (what, rc, last_error()))


def config(M=0, V=0, W=0, CL=0, S=0, split=0):
    return mg_config(M, V, W, CL, S, split)


def cfg_ptr(cfg):
    return None if cfg is None else ctypes.byref(cfg)
