"""Batched fits and the serving loop (vmb_* / vms_* of the C ABI).

Batch: many independent VoroMesh fits in one device arena (the HBM budget),
stepped together with one launch per stage. serve(): continuous batching of
fit requests that arrive over time, with per-request latency.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import check, load, ptr, vm_params
from .optimizer import OptimizerParams


class vmb_fit(C.Structure):
    _fields_ = [("width", C.c_float), ("height", C.c_float), ("spacing", C.c_float), ("params", vm_params),
                ("generators", C.c_void_p), ("slotsW", C.c_int), ("slotsH", C.c_int), ("slotCellSize", C.c_float),
                ("targets", C.c_void_p), ("nTargets", C.c_int)]


class vmb_fit_info_t(C.Structure):
    _fields_ = [("iteration", C.c_int), ("lastLoss", C.c_float), ("numSlots", C.c_int), ("liveTargets", C.c_int),
                ("active", C.c_int)]


class vms_request(C.Structure):
    _fields_ = [("arrival", C.c_double), ("fit", vmb_fit), ("maxSteps", C.c_int), ("relTol", C.c_float),
                ("outGenerators", C.c_void_p)]


class vms_config(C.Structure):
    _fields_ = [("hbmBudgetBytes", C.c_size_t), ("maxLive", C.c_int), ("stepsPerRound", C.c_int),
                ("lossVariant", C.c_int), ("maxLiveTargets", C.c_size_t)]


class vms_result(C.Structure):
    _fields_ = [("arrival", C.c_double), ("admitted", C.c_double), ("finished", C.c_double), ("steps", C.c_int),
                ("finalLoss", C.c_float), ("status", C.c_int)]


def _declare(lib):
    if getattr(lib, "_vmb_declared", False):
        return lib
    P, I, F = C.c_void_p, C.c_int, C.c_float
    sig = {"vmb_create": [C.c_size_t, I, I, P], "vmb_destroy": [P], "vmb_add_fit": [P, P, P],
           "vmb_remove_fit": [P, I], "vmb_set_active": [P, I, I], "vmb_step": [P, I, P], "vmb_evaluate": [P, P],
           "vmb_fit_info": [P, I, P], "vmb_get_generators": [P, I, P], "vmb_memory": [P, P, P, P],
           "vms_serve": [P, I, P, P]}
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.vmb_fit_bytes.argtypes = [I, I, I, F, F, F]
    lib.vmb_fit_bytes.restype = C.c_size_t
    lib._vmb_declared = True
    return lib


def _fit_struct(spec, params: OptimizerParams, keep: list) -> vmb_fit:
    gen = np.ascontiguousarray(spec.generators, np.float32)
    tgt = np.ascontiguousarray(spec.targets, np.float32)
    keep += [gen, tgt]
    f = vmb_fit()
    f.width, f.height, f.spacing = spec.width, spec.height, spec.spacing
    f.params = params.to_c()
    f.generators = gen.ctypes.data
    f.slotsW, f.slotsH, f.slotCellSize = spec.slotsW, spec.slotsH, spec.slotCellSize
    f.targets = tgt.ctypes.data
    f.nTargets = len(tgt)
    return f


def params_for(spec) -> OptimizerParams:
    """The schedule of a FitSpec: `steps` iterations, every target each step."""
    return OptimizerParams(iterations=spec.steps, sampleFraction=spec.sampleFraction,
                           lrPerSpacing=spec.lrPerSpacing, lossK=spec.lossK)


class Batch:
    def __init__(self, arena_bytes: int, max_fits: int = 1024, loss_variant: int = -1):
        self._lib = _declare(load())
        h = C.c_void_p()
        check(self._lib.vmb_create(arena_bytes, max_fits, loss_variant, C.byref(h)), "vmb_create")
        self._h = h
        self.max_fits = max_fits

    def close(self):
        if getattr(self, "_h", None):
            self._lib.vmb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, spec, params: OptimizerParams | None = None) -> int:
        keep = []
        f = _fit_struct(spec, params or params_for(spec), keep)
        fid = C.c_int()
        check(self._lib.vmb_add_fit(self._h, C.byref(f), C.byref(fid)), "vmb_add_fit")
        return fid.value

    def remove(self, fid: int):
        check(self._lib.vmb_remove_fit(self._h, fid), "vmb_remove_fit")

    def step(self, iterations: int) -> float:
        ms = C.c_float()
        check(self._lib.vmb_step(self._h, iterations, C.byref(ms)), "vmb_step")
        return ms.value

    def evaluate(self) -> np.ndarray:
        out = np.zeros(self.max_fits, np.float32)
        check(self._lib.vmb_evaluate(self._h, ptr(out)), "vmb_evaluate")
        return out

    def info(self, fid: int) -> vmb_fit_info_t:
        i = vmb_fit_info_t()
        check(self._lib.vmb_fit_info(self._h, fid, C.byref(i)), "vmb_fit_info")
        return i

    def generators(self, fid: int) -> np.ndarray:
        i = self.info(fid)
        out = np.empty((i.numSlots, 2), np.float32)
        check(self._lib.vmb_get_generators(self._h, fid, ptr(out)), "vmb_get_generators")
        return out

    def memory(self):
        fb, tb, lf = C.c_size_t(), C.c_size_t(), C.c_int()
        check(self._lib.vmb_memory(self._h, C.byref(fb), C.byref(tb), C.byref(lf)), "vmb_memory")
        return fb.value, tb.value, lf.value


def fit_bytes(spec) -> int:
    lib = _declare(load())
    return lib.vmb_fit_bytes(spec.slotsW, spec.slotsH, len(spec.targets), spec.width, spec.height, spec.spacing)


@dataclass
class ServeResult:
    arrival: np.ndarray
    admitted: np.ndarray
    finished: np.ndarray
    steps: np.ndarray
    final_loss: np.ndarray
    status: np.ndarray
    generators: list

    @property
    def latency(self) -> np.ndarray:
        return self.finished - self.arrival


def serve(specs, arrivals, hbm_budget: int, max_live: int = 1024, steps_per_round: int = 10, max_steps: int = 500,
          rel_tol: float = 1e-6, loss_variant: int = -1, keep_generators: bool = True,
          max_live_targets: int = 0) -> ServeResult:
    """Serves fit requests arriving at `arrivals` (seconds); maxLive=1 is the
    one-fit-at-a-time loop; max_live_targets caps the live fits' targets (0 =
    no cap)."""
    lib = _declare(load())
    n = len(specs)
    reqs = (vms_request * max(n, 1))()
    keep, outs = [], []
    for i, spec in enumerate(specs):
        reqs[i].arrival = float(arrivals[i])
        reqs[i].fit = _fit_struct(spec, params_for(spec), keep)
        reqs[i].maxSteps = max_steps
        reqs[i].relTol = rel_tol
        if keep_generators:
            out = np.empty((spec.slotsW * spec.slotsH, 2), np.float32)
            outs.append(out)
            reqs[i].outGenerators = out.ctypes.data
        else:
            outs.append(None)
    cfg = vms_config(hbm_budget, max_live, steps_per_round, loss_variant, max_live_targets)
    res = (vms_result * max(n, 1))()
    check(lib.vms_serve(reqs, n, C.byref(cfg), res), "vms_serve")
    arr = lambda f, dt: np.array([getattr(res[i], f) for i in range(n)], dt)
    return ServeResult(arr("arrival", np.float64), arr("admitted", np.float64), arr("finished", np.float64),
                       arr("steps", np.int32), arr("finalLoss", np.float32), arr("status", np.int32), outs)
