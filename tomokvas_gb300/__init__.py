"""GB300-native FDK cone-beam reconstruction (drop-in for the TomoKvas GPU engine).

The compute path is libtk_fdk.so (hand-written sm_103a CUDA behind a C ABI,
include/tk_fdk.h).  This package holds the host-side mirror of the
reference interface and device-buffer helpers; it has no CPU fallback.
"""
from . import _lib
from ._lib import TKError, load
from .fbp import FilteredBackProjection, VolumeSink
from .geometry import FDKGeometry, config

__all__ = ["FilteredBackProjection", "VolumeSink", "FDKGeometry", "config", "TKError", "load", "_lib"]
