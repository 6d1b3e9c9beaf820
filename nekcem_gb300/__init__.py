"""GB300-native (sm_103a) NekCEM Maxwell DG time step.

The product is the CUDA library ``libnekcem_gb300.so`` behind the C ABI of
``include/nekcem_gpu.h``; this package builds it in place and binds it for
Python callers.
"""
from . import cases
from ._lib import FORMS, MIXED, FUSED64, PLAIN, NekgpuError, load
from .build import build as build_library
from .maxwell import MaxwellGPU

__all__ = ["MaxwellGPU", "NekgpuError", "build_library", "load", "cases", "FORMS", "MIXED", "FUSED64",
           "PLAIN"]
