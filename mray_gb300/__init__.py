"""mray_gb300 -- GB300-native (sm_103a) ray-tracing hot path of MRay.

The compute path is the CUDA library ``libmray_gb300.so`` (C ABI in
``include/mray_gb300.h``); this package holds its Python bindings, the
host-side mirror of MRay's accelerator interface and the seeded workload
generators.  There is no CPU fallback: importing ``Accelerator`` and creating
one fails loudly if the library or a GPU is missing.
"""
from ._native import MRGError, lib  # noqa: F401
from .accel import Accelerator  # noqa: F401

__all__ = ["Accelerator", "MRGError", "lib"]
