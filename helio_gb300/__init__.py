"""helio_gb300 — GB300 (sm_103a) implementation of Helio's deferred-lighting path.

Light binning (the reference's 16-pixel tile culling, and froxel clustering) and
Cook-Torrance/GGX deferred shading run as hand-written CUDA kernels behind the C ABI in
``include/helio_gb300.h``. This package holds the kernels (``csrc/``), their build
(``build``), the ctypes binding (``native``), the reference-shaped pass classes
(``passes``), the struct layouts (``layouts``) and seeded synthetic inputs
(``synthetic``).
"""
from . import layouts  # noqa: F401

__all__ = ["layouts", "native", "passes", "synthetic", "frame", "build"]
