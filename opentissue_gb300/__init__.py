"""GB300 (sm_103a) implementation of OpenTissue's stiffness-warped tetrahedral
FEM step.  The product is the C ABI library libotfem_gpu.so (include/otfem_gpu.h)
and the drop-in C++ headers under include/OpenTissue; this package is the
Python mirror of the same interface (capi: raw ctypes bindings, fem: the
OpenTissue::fem functions)."""
from . import capi, fem  # noqa: F401

__all__ = ["capi", "fem"]
