"""GB300-native hot path of TwoScaleRich: the two-scale Richards right-hand
side G(h) and the EXPREM Krylov stage, as sm_103a CUDA behind a C-ABI
(include/tsr_capi.h) with the reference's C++ signatures on top
(include/tsr_dropin.hpp).  This package holds the ctypes binding
(``capi``), problem set-up and the reference driver loop (``problem``),
synthetic meshes (``meshgen``) and the build step (``build``)."""
from . import capi  # noqa: F401

__all__ = ["capi", "problem", "meshgen", "build"]
