"""meshes_gb300: GB300-native (sm_103a) propagation of optical fields through layered MZI meshes.

The compute path is libmeshes_gb300.so (hand-written CUDA, loaded through ctypes); PyTorch supplies
device memory and streams.  Public API:

* ``MeshNetworkGPU`` - drop-in for the reference ``meshes.gpu.MeshNetworkGPU`` (dot, grad_phi, ...)
* ``from_structured`` - the reference ``StructuredMeshNetwork.gpu()`` converter
* ``geometry`` - Clements / Reck / butterfly layouts
"""
from ._lib import MeshLibraryError  # noqa: F401
from . import geometry  # noqa: F401
from .mesh import MeshNetworkGPU, from_structured  # noqa: F401

__version__ = "0.1.0"


def _load_tuning():
    """Load the committed autotuning table into the library (silently skipped without the library)."""
    try:
        from .autotune import load_table
        load_table()
    except (MeshLibraryError, OSError):
        pass


_load_tuning()
