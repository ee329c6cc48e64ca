"""GB300-native VoroMesh optimisation step, Voronoi extraction, Poisson-disk
sampler and canvas (Python front end of libvoromesh_gb300.so).

The hot path runs in hand-written sm_103a CUDA kernels behind the C ABI of
include/vm_capi.h; this package only marshals numpy arrays to it. Importing
it requires the library to be built (there is no CPU fallback).
"""
from ._lib import LIB_PATH, VmError, load
from .canvas import Canvas, Edit
from .optimizer import OptimizerParams, Sampler, VoroMesh2D, VoroOptimizer, resample_many

__all__ = ["LIB_PATH", "VmError", "load", "Canvas", "Edit", "OptimizerParams", "Sampler", "VoroMesh2D", "VoroOptimizer",
           "resample_many"]
