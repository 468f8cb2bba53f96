"""GB300 SOP engine: Python handle on libsopgpu.so (C ABI in include/sop_gpu.h).

The compute path is the CUDA library; this package only binds it (ctypes),
builds workloads in the reference's file formats, and wraps the engine.
"""
from . import _lib  # noqa: F401
from ._lib import SopError, lib  # noqa: F401

__all__ = ["SopError", "lib"]
