"""Python mirror of voromesh::VoroOptimizer and poisson::Sampler over the C ABI.

Method names, argument meaning and call order follow the reference's C++ API
(include/voromesh/voro_optimizer.h:70-121, include/poisson/poisson_disk.h:21-50);
point arrays are numpy float32 arrays of shape (n, 2). Failures raise
VmError instead of exiting the process.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, load, pd_info_t, ptr, vm_checkpoint_info, vm_info_t, vm_mesh_info, vm_params


def _pts(a, name: str) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != 2:
        raise ValueError(f"{name} must have shape (n, 2)")
    return a


@dataclass
class OptimizerParams:
    """OptimizerParams (voro_optimizer.h:34-44) plus the loss kNN size."""
    iterations: int = 400
    localIterations: int = 100
    lrPerSpacing: float = 0.09
    sampleFraction: float = 0.2
    gamma: float = 0.5
    milestones: tuple = (80, 150, 200, 250)
    seed: int = 1
    lossK: int = 12

    def to_c(self) -> vm_params:
        p = vm_params()
        p.iterations = self.iterations
        p.localIterations = self.localIterations
        p.lrPerSpacing = self.lrPerSpacing
        p.sampleFraction = self.sampleFraction
        p.gamma = self.gamma
        for k in range(4):
            p.milestones[k] = int(self.milestones[k])
        p.seed = self.seed
        p.lossK = self.lossK
        return p


@dataclass
class VoroMesh2D:
    """VoroMesh2D (voro_optimizer.h:46-68)."""
    generators: np.ndarray
    inside: np.ndarray
    cellStart: np.ndarray
    cellVerts: np.ndarray
    vertices: np.ndarray
    edges: np.ndarray
    cellLabels: np.ndarray
    watertight: bool = False
    loops: int = 0
    unsafeCells: int = 0
    overflowCells: int = 0
    gpuMs: float = 0.0
    hostMs: float = 0.0


class VoroOptimizer:
    """voromesh::VoroOptimizer on one GPU."""

    def __init__(self, width: float, height: float, spacing: float, params: OptimizerParams | None = None):
        self._lib = load()
        self._params = params or OptimizerParams()
        h = C.c_void_p()
        cp = self._params.to_c()
        check(self._lib.vm_create(width, height, spacing, C.byref(cp), C.byref(h)), "VoroOptimizer")
        self._h = h
        self.width, self.height, self.spacing = float(width), float(height), float(spacing)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.vm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- targets / occupancy / generators ----
    def SetTargets(self, slots) -> None:
        a = _pts(slots, "slots")
        check(self._lib.vm_set_targets(self._h, ptr(a), len(a)), "SetTargets")

    def UpdateTargets(self, dirty, slots) -> None:
        d = np.ascontiguousarray(dirty, dtype=np.int32)
        a = _pts(slots, "slots")
        check(self._lib.vm_update_targets(self._h, ptr(d), len(d), ptr(a), len(a)), "UpdateTargets")

    def SetOccupancy(self, masks, tilesX: int, tilesY: int, voxelSize: float) -> None:
        m = np.ascontiguousarray(masks, dtype=np.uint64)
        if m.size < tilesX * tilesY:
            raise ValueError("masks smaller than tilesX * tilesY")
        check(self._lib.vm_set_occupancy(self._h, ptr(m), tilesX, tilesY, voxelSize), "SetOccupancy")

    def UpdateOccupancy(self, masks, tx0: int, ty0: int, tx1: int, ty1: int) -> None:
        m = np.ascontiguousarray(masks, dtype=np.uint64)
        check(self._lib.vm_update_occupancy(self._h, ptr(m), tx0, ty0, tx1, ty1), "UpdateOccupancy")

    # ---- checkpoint / resume (GB300 extension) ----
    def Checkpoint(self) -> dict:
        """The fit's optimisation state: slot layout, schedule, step counter,
        last batch loss, generators and Adam moments."""
        info = vm_checkpoint_info()
        check(self._lib.vm_checkpoint(self._h, C.byref(info), None, None, None), "Checkpoint")
        n = info.slotsW * info.slotsH
        g, m, v = (np.empty((n, 2), np.float32) for _ in range(3))
        check(self._lib.vm_checkpoint(self._h, C.byref(info), ptr(g), ptr(m), ptr(v)), "Checkpoint")
        return {"info": {k: getattr(info, k) for k, _ in vm_checkpoint_info._fields_}, "generators": g, "m": m, "v": v}

    def Restore(self, ckpt: dict) -> None:
        """Resumes a Checkpoint() in an optimiser made with the same arguments,
        targets and occupancy: the next Step continues the saved run."""
        info = vm_checkpoint_info(**ckpt["info"])
        g, m, v = (np.ascontiguousarray(ckpt[k], np.float32) for k in ("generators", "m", "v"))
        check(self._lib.vm_restore(self._h, C.byref(info), ptr(g), ptr(m), ptr(v)), "Restore")

    # ---- device-to-device hand-off from a Canvas (GB300 extension) ----
    def SetTargetsFromCanvas(self, canvas) -> None:
        """SetTargets(canvas.TargetSlots()) + SetOccupancy(canvas.InsideMasks(), ...) without a host copy."""
        check(self._lib.vm_set_targets_from_canvas(self._h, canvas._h), "SetTargetsFromCanvas")

    def UpdateFromCanvas(self, canvas) -> None:
        """UpdateTargets + UpdateOccupancy for the canvas's last edit, device to device."""
        check(self._lib.vm_update_from_canvas(self._h, canvas._h), "UpdateFromCanvas")

    def SetGenerators(self, slots, slotsW: int, slotsH: int, slotCellSize: float) -> None:
        a = _pts(slots, "slots")
        if len(a) != slotsW * slotsH:
            raise ValueError("slots must hold slotsW * slotsH points")
        check(self._lib.vm_set_generators(self._h, ptr(a), slotsW, slotsH, slotCellSize), "SetGenerators")

    def UpdateGenerators(self, slots, cx0: int, cy0: int, cx1: int, cy1: int) -> None:
        a = _pts(slots, "slots")
        check(self._lib.vm_update_generators(self._h, ptr(a), cx0, cy0, cx1, cy1), "UpdateGenerators")

    def BeginSchedule(self, iterations: int, cx0: int | None = None, cy0: int = 0, cx1: int | None = None,
                      cy1: int | None = None) -> None:
        if cx0 is None:
            cx0, cy0, cx1, cy1 = 0, 0, 1 << 30, 1 << 30
        check(self._lib.vm_begin_schedule(self._h, iterations, cx0, cy0, cx1, cy1), "BeginSchedule")

    # ---- optimisation ----
    def Step(self, iterations: int) -> float:
        ms = C.c_float()
        check(self._lib.vm_step(self._h, iterations, C.byref(ms)), "Step")
        return ms.value

    def StepTimed(self, iterations: int) -> np.ndarray:
        """Steps kernel by kernel; mean ms per step of [loss, adam+bin, scan, scatter]."""
        out = np.zeros(4, np.float32)
        check(self._lib.vm_step_timed(self._h, iterations, ptr(out)), "StepTimed")
        return out

    def SetLossVariant(self, variant: int) -> None:
        """Loss-kernel variant (-1 = automatic); every variant gives identical results."""
        check(self._lib.vm_set_loss_variant(self._h, variant), "SetLossVariant")

    def LossVariant(self):
        v, n = C.c_int(), C.c_int()
        check(self._lib.vm_get_loss_variant(self._h, C.byref(v), C.byref(n)), "LossVariant")
        return v.value, n.value

    def Optimize(self) -> float:
        i = self.info()
        return self.Step(i.scheduleLength - i.iteration)

    def LastBatchLoss(self) -> float:
        return self.info().lastBatchLoss

    def EvaluateLoss(self) -> float:
        v = C.c_float()
        check(self._lib.vm_evaluate_loss(self._h, C.byref(v)), "EvaluateLoss")
        return v.value

    def Iteration(self) -> int:
        return self.info().iteration

    def ScheduleLength(self) -> int:
        return self.info().scheduleLength

    def NumSlots(self) -> int:
        return self.info().numSlots

    def Params(self) -> OptimizerParams:
        return self._params

    def info(self) -> vm_info_t:
        i = vm_info_t()
        check(self._lib.vm_info(self._h, C.byref(i)), "info")
        return i

    # ---- outputs ----
    def Generators(self) -> np.ndarray:
        out = np.empty((self.NumSlots(), 2), np.float32)
        check(self._lib.vm_get_generators(self._h, ptr(out)), "Generators")
        return out

    def Moments(self):
        n = self.NumSlots()
        m = np.empty((n, 2), np.float32)
        v = np.empty((n, 2), np.float32)
        check(self._lib.vm_get_moments(self._h, ptr(m), ptr(v)), "Moments")
        return m, v

    def Extract(self) -> VoroMesh2D:
        info = vm_mesh_info()
        check(self._lib.vm_extract(self._h, C.byref(info)), "Extract")
        n = info.numGenerators
        gen = np.empty((n, 2), np.float32)
        inside = np.empty(n, np.uint8)
        cs = np.empty(n + 1 if n else 0, np.int32)
        cv = np.empty((info.numCellVerts, 2), np.float32)
        vert = np.empty((info.numVertices, 2), np.float32)
        edges = np.empty((info.numEdges, 2), np.int32)
        labels = np.empty(info.numCellVerts, np.int32)
        check(self._lib.vm_mesh_copy(self._h, ptr(gen), ptr(inside), ptr(cs), ptr(cv), ptr(vert), ptr(edges),
                                     ptr(labels)), "Extract")
        return VoroMesh2D(gen, inside, cs, cv, vert, edges, labels, bool(info.watertight), info.loops,
                          info.unsafeCells, info.overflowCells, info.gpuMs, info.hostMs)

    # ---- inspection ----
    def Grid(self):
        i = self.info()
        n = i.numSlots
        start = np.empty(i.gridW * i.gridH + 1, np.int32)
        genCell = np.empty(n, np.int32)
        check(self._lib.vm_get_grid(self._h, ptr(start), None, None, ptr(genCell)), "Grid")
        live = int(start[-1])
        sidx = np.empty(live, np.int32)
        spos = np.empty((live, 2), np.float32)
        check(self._lib.vm_get_grid(self._h, None, ptr(sidx), ptr(spos), None), "Grid")
        return start, sidx, spos, genCell

    def Knn(self, queries, K: int, out=None):
        """The K nearest sites of each query (indices, squared distances).
        `out` = (idx, d2), int32 and float32 arrays of shape (n, K), are
        filled in place of new arrays (a caller reusing them skips the page
        faults of fresh output memory)."""
        q = _pts(queries, "queries")
        if out is None:
            idx = np.empty((len(q), K), np.int32)
            d2 = np.empty((len(q), K), np.float32)
        else:
            idx, d2 = out
            if (idx.shape != (len(q), K) or d2.shape != (len(q), K) or idx.dtype != np.int32
                    or d2.dtype != np.float32 or not idx.flags.c_contiguous or not d2.flags.c_contiguous):
                raise ValueError("out must be C-contiguous int32 and float32 arrays of shape (n, K)")
        check(self._lib.vm_knn(self._h, ptr(q), len(q), K, ptr(idx), ptr(d2)), "Knn")
        return idx, d2

    def Probe(self, mode: int = 0):
        """One loss pass without moving anything: per-target (i0, j, loss),
        the summed gradient (mode 0), the used-target count and loss sum."""
        i = self.info()
        cap, n = i.targetCapacity, i.numSlots
        i0 = np.empty(cap, np.int32)
        j = np.empty(cap, np.int32)
        loss = np.empty(cap, np.float32)
        grad = np.empty((n, 2), np.float32)
        cnt = C.c_int()
        ls = C.c_float()
        check(self._lib.vm_probe(self._h, mode, ptr(i0), ptr(j), ptr(loss), ptr(grad), C.byref(cnt), C.byref(ls)),
              "Probe")
        return i0, j, loss, grad, cnt.value, ls.value


class Sampler:
    """poisson::Sampler on one GPU (constructing it fills the whole domain)."""

    def __init__(self, width: float, height: float, radius: float, trials: int = 30, seed: int = 1):
        self._lib = load()
        h = C.c_void_p()
        check(self._lib.pd_create(width, height, radius, trials, seed, C.byref(h)), "Sampler")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> pd_info_t:
        i = pd_info_t()
        check(self._lib.pd_info(self._h, C.byref(i)), "info")
        return i

    def Resample(self, cx0: int, cy0: int, cx1: int, cy1: int) -> float:
        ms = C.c_float()
        check(self._lib.pd_resample(self._h, cx0, cy0, cx1, cy1, C.byref(ms)), "Resample")
        return ms.value

    def ResampleAll(self) -> float:
        i = self.info()
        return self.Resample(0, 0, i.gridW, i.gridH)

    def Verify(self, cx0: int, cy0: int, cx1: int, cy1: int) -> bool:
        ok = C.c_int()
        check(self._lib.pd_verify(self._h, cx0, cy0, cx1, cy1, C.byref(ok)), "Verify")
        return bool(ok.value)

    def VerifyAll(self) -> bool:
        i = self.info()
        return self.Verify(0, 0, i.gridW, i.gridH)

    def Cells(self) -> np.ndarray:
        i = self.info()
        out = np.empty((i.gridW * i.gridH, 2), np.float32)
        check(self._lib.pd_cells(self._h, ptr(out)), "Cells")
        return out

    def Count(self) -> int:
        n = C.c_longlong()
        check(self._lib.pd_count(self._h, C.byref(n)), "Count")
        return n.value

    def Width(self) -> float: return self.info().width
    def Height(self) -> float: return self.info().height
    def Radius(self) -> float: return self.info().radius
    def CellSize(self) -> float: return self.info().cellSize
    def GridW(self) -> int: return self.info().gridW
    def GridH(self) -> int: return self.info().gridH
    def Trials(self) -> int: return self.info().trials


def resample_many(samplers, regions) -> float:
    """Resample(*regions[i]) on each of the distinct `samplers` at once (small
    regions as one block each of a single launch); returns GPU ms."""
    lib = load()
    n = len(samplers)
    handles = (C.c_void_p * max(n, 1))(*[s._h for s in samplers])
    r = np.ascontiguousarray(np.asarray(regions, np.int32).reshape(n, 4))
    ms = C.c_float()
    check(lib.pd_resample_many(handles, ptr(r), n, C.byref(ms)), "resample_many")
    return ms.value
