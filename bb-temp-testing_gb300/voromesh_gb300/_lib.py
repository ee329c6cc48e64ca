"""Loads libvoromesh_gb300.so (built in-tree) and declares its C ABI, and
libvm_synth.so, the seeded input generators.

There is no fallback: if the library is missing or cannot be loaded the
import fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libvoromesh_gb300.so"
SYNTH_PATH = LIB_PATH.parent / "libvm_synth.so"

VM_OK = 0
ERRORS = {
    1: "invalid argument",
    2: "out of memory",
    3: "CUDA error",
    4: "invalid state",
    5: "over memory budget",
    6: "timeout",
    7: "unsupported parameter",
    8: "no CUDA device",
}


class VmError(RuntimeError):
    """A non-zero status from the library, with its message."""

    def __init__(self, code: int, what: str, msg: str):
        super().__init__(f"{what}: {ERRORS.get(code, 'error')} ({msg})")
        self.code = code


class vm_params(C.Structure):
    _fields_ = [("iterations", C.c_int), ("localIterations", C.c_int), ("lrPerSpacing", C.c_float),
                ("sampleFraction", C.c_float), ("gamma", C.c_float), ("milestones", C.c_int * 4),
                ("seed", C.c_uint), ("lossK", C.c_int)]


class vm_info_t(C.Structure):
    _fields_ = [("iteration", C.c_int), ("scheduleLength", C.c_int), ("numSlots", C.c_int),
                ("targetCapacity", C.c_int), ("liveTargets", C.c_int), ("gridW", C.c_int), ("gridH", C.c_int),
                ("lastBatchLoss", C.c_float), ("exactTargets", C.c_longlong)]


class vm_mesh_info(C.Structure):
    _fields_ = [("numGenerators", C.c_int), ("numCellVerts", C.c_int), ("numVertices", C.c_int),
                ("numEdges", C.c_int), ("watertight", C.c_int), ("loops", C.c_int), ("unsafeCells", C.c_int),
                ("overflowCells", C.c_int), ("gpuMs", C.c_float), ("hostMs", C.c_float)]


class vm_checkpoint_info(C.Structure):
    _fields_ = [("slotsW", C.c_int), ("slotsH", C.c_int), ("slotCellSize", C.c_float), ("scheduleLength", C.c_int),
                ("iteration", C.c_int), ("cx0", C.c_int), ("cy0", C.c_int), ("cx1", C.c_int), ("cy1", C.c_int),
                ("lastBatchLoss", C.c_float)]


class cv_edit(C.Structure):
    _fields_ = [("tx0", C.c_int), ("ty0", C.c_int), ("tx1", C.c_int), ("ty1", C.c_int), ("removed", C.c_int),
                ("added", C.c_int), ("flipped", C.c_int), ("ndirty", C.c_int)]


class cv_info_t(C.Structure):
    _fields_ = [("voxelsX", C.c_int), ("voxelsY", C.c_int), ("tilesX", C.c_int), ("tilesY", C.c_int),
                ("voxelSize", C.c_float), ("numSlots", C.c_int), ("freeSlots", C.c_int),
                ("surfaceCount", C.c_longlong), ("surfaceTiles", C.c_int)]


class pd_info_t(C.Structure):
    _fields_ = [("width", C.c_float), ("height", C.c_float), ("radius", C.c_float), ("cellSize", C.c_float),
                ("gridW", C.c_int), ("gridH", C.c_int), ("trials", C.c_int), ("seed", C.c_uint),
                ("roundBase", C.c_uint)]


P = C.c_void_p
I = C.c_int
F = C.c_float

# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "vm_error_string": [I],
    "vm_last_error": [C.c_char_p, I],
    "vm_version": [P, P, P],
    "vm_params_default": [P],
    "vm_create": [F, F, F, P, P],
    "vm_destroy": [P],
    "vm_set_targets": [P, P, I],
    "vm_update_targets": [P, P, I, P, I],
    "vm_set_occupancy": [P, P, I, I, F],
    "vm_update_occupancy": [P, P, I, I, I, I],
    "vm_set_generators": [P, P, I, I, F],
    "vm_update_generators": [P, P, I, I, I, I],
    "vm_begin_schedule": [P, I, I, I, I, I],
    "vm_step": [P, I, P],
    "vm_step_timed": [P, I, P],
    "vm_evaluate_loss": [P, P],
    "vm_set_loss_variant": [P, I],
    "vm_get_loss_variant": [P, P, P],
    "vm_info": [P, P],
    "vm_get_generators": [P, P],
    "vm_get_moments": [P, P, P],
    "vm_extract": [P, P],
    "vm_mesh_copy": [P, P, P, P, P, P, P, P],
    "vm_get_grid": [P, P, P, P, P],
    "vm_knn": [P, P, I, I, P, P],
    "vm_probe": [P, I, P, P, P, P, P, P],
    "vm_build_grid_noalloc": [P, I, I, I, F, P, P, P, P],
    "pd_create": [F, F, F, I, C.c_uint, P],
    "pd_destroy": [P],
    "pd_resample": [P, I, I, I, I, P],
    "pd_resample_many": [P, P, I, P],
    "pd_info": [P, P],
    "pd_cells": [P, P],
    "pd_verify": [P, I, I, I, I, P],
    "pd_count": [P, P],
    "cv_create": [F, F, F, P],
    "cv_destroy": [P],
    "cv_rasterize": [P, P, I, P],
    "cv_stamp_disc": [P, F, F, F, I, P],
    "cv_edit_dirty": [P, P, P, I],
    "cv_info": [P, P],
    "cv_get_slots": [P, P],
    "cv_get_inside": [P, P],
    "cv_get_inside_rect": [P, P, I, I, I, I],
    "cv_get_surface": [P, P, P, P],
    "cv_get_free": [P, P],
    "cv_is_inside": [P, I, I, P],
    "cv_is_surface": [P, I, I, P],
    "vm_set_targets_from_canvas": [P, P],
    "vm_checkpoint": [P, P, P, P, P],
    "vm_restore": [P, P, P, P, P],
    "vm_update_from_canvas": [P, P],
}
_RESTYPES = {"vm_error_string": C.c_char_p, "vm_params_default": None}

# the seeded input generators (libvm_synth.so, host code)
SYNTH_SIGNATURES = {
    "vm_synth_uniform": [C.c_uint64, C.c_uint64, C.c_int64, C.c_double, C.c_double, I, P],
    "vm_synth_circle": [C.c_uint64, C.c_uint64, C.c_int64, C.c_double, C.c_double, I, P],
    "vm_synth_lattice": [C.c_uint64, C.c_uint64, I, I, C.c_double, I, P],
    "vm_synth_ellipse_params": [C.c_uint64, C.c_uint64, I, P],
    "vm_synth_ellipse_union": [C.c_uint64, C.c_uint64, I, C.c_int64, I, P],
    "vm_synth_star": [C.c_uint64, C.c_uint64, I, P, C.c_double, C.c_double, C.c_double, C.c_int64, I, P],
    "vm_synth_star_params": [C.c_uint64, C.c_uint64, P, P, P],
    "vm_synth_subset": [C.c_uint64, C.c_uint64, C.c_int64, C.c_int64, P],
    "vm_synth_uniform01": [C.c_uint64, C.c_uint64, C.c_int64, P],
    "vm_synth_log": [C.c_double],
    "vm_synth_exp": [C.c_double],
}
_SYNTH_RESTYPES = {"vm_synth_uniform": None, "vm_synth_circle": None, "vm_synth_lattice": None,
                   "vm_synth_ellipse_params": None, "vm_synth_ellipse_union": C.c_int64, "vm_synth_star": None,
                   "vm_synth_star_params": None, "vm_synth_subset": C.c_int, "vm_synth_uniform01": C.c_double,
                   "vm_synth_log": C.c_double, "vm_synth_exp": C.c_double}

_lib = None


def load() -> C.CDLL:
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("VOROMESH_GB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(f"{path} not found: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'` at the repository root")
    lib = C.CDLL(str(path))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


_synth = None


def load_synth() -> C.CDLL:
    """The seeded input generators (raises if they have not been built)."""
    global _synth
    if _synth is not None:
        return _synth
    if not SYNTH_PATH.exists():
        raise ImportError(f"{SYNTH_PATH} not found: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'` at the repository root")
    lib = C.CDLL(str(SYNTH_PATH))
    for name, args in SYNTH_SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _SYNTH_RESTYPES.get(name, C.c_int)
    _synth = lib
    return lib


def check(rc: int, what: str) -> None:
    if rc != VM_OK:
        buf = C.create_string_buffer(1024)
        load().vm_last_error(buf, 1024)
        raise VmError(rc, what, buf.value.decode(errors="replace"))


def ptr(a) -> C.c_void_p:
    """Data pointer of a contiguous numpy array (or None)."""
    if a is None:
        return None
    return C.c_void_p(a.ctypes.data)
