"""GB300-native FDK cone-beam reconstruction (drop-in for the TomoKvas GPU engine).

The compute path is libtk_fdk.so (hand-written sm_103a CUDA behind a C ABI,
include/tk_fdk.h).  This package holds the host-side mirror of the
reference interface (fbp), device-buffer stage calls, the adjoint pair and
the out-of-core and rsq helpers (device), batches of uneven reconstructions
(batch), the scan/volume file formats (scanfile) and the workload
geometries (geometry); it has no CPU fallback.
"""
from . import _lib
from ._lib import TKError, load
from .batch import Batch
from .fbp import FilteredBackProjection, VolumeSink
from .geometry import FDKGeometry, config

__all__ = ["FilteredBackProjection", "VolumeSink", "Batch", "FDKGeometry", "config", "TKError", "load", "_lib"]
