"""smolyax_gb300: GB300-native evaluation path of the barycentric Smolyak interpolant.

Drop-in for ``smolyax``'s ``SmolyakBarycentricInterpolator`` (``__call__``,
``gradient``, ``integral``), its ``indices`` functions and its ``nodes``
generators.  Compute runs in hand-written sm_103a CUDA kernels behind the C
ABI of ``include/smolyax_gb300.h``; there is no CPU fallback.
"""
from . import indices, nodes  # noqa: F401
from .interpolation import SmolyakBarycentricInterpolator  # noqa: F401

__all__ = ["indices", "nodes", "SmolyakBarycentricInterpolator"]
