"""The editor's local-edit sequence as a test case (apps/voromesh_demo.cpp:
117-140): a fit of 40x40 generator slots (one generator per slot cell),
targets on a circle, a global schedule, then one edit -- a dent pushed into
the right of the circle (UpdateTargets of the dirty slots), fresh generators
in a rectangle of slots around it (UpdateGenerators of that rectangle) and a
local schedule over the rectangle (BeginSchedule(localIterations, rect),
Optimize). The local schedule's milestones are scaled by 60/200 and three of
them fall inside its 60 steps; the sample fraction is 0.2.

Shared by the GPU parity test, the oracle's live pin against the reference's
kernels and tests/golden/make_golden.py.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class EditCase:
    slots: int
    spacing: float
    slot_cell: float
    generators: np.ndarray   # initial slots (slots x slots)
    targets: np.ndarray      # initial target slots
    targets2: np.ndarray     # target slots after the edit
    dirty: np.ndarray        # target slots the edit changed
    slots2: np.ndarray       # generator slots handed to UpdateGenerators
    rect: tuple              # (cx0, cy0, cx1, cy1) of the edit
    K: int = 12
    lr_per_spacing: float = 0.09
    fraction: float = 0.2
    iterations: int = 200
    local_iterations: int = 60
    global_steps: int = 30


def _in_cells(u: np.ndarray, w: int, cell: float) -> np.ndarray:
    """One point per slot cell of a w x w slot grid, at fraction u of the cell."""
    f32 = np.float32
    ys, xs = np.divmod(np.arange(w * w), w)
    x = (xs.astype(f32) + u[:, 0].astype(f32)) * f32(cell)
    y = (ys.astype(f32) + u[:, 1].astype(f32)) * f32(cell)
    return np.ascontiguousarray(np.stack([x, y], 1), np.float32)


def edit_case() -> EditCase:
    from voromesh_gb300 import synth

    w = 40
    cell = float(np.float32(2.0) / np.float32(w))
    gen = _in_cells(synth.uniform(41, 1, w * w, 0.0, 1.0, shift=False), w, cell)
    tgt = synth.circle(41, 2, 12000, 0.6, 1e-3)
    dirty = np.nonzero(tgt[:, 0] > np.float32(1.35))[0].astype(np.int32)
    tgt2 = tgt.copy()
    d = tgt[dirty] - np.float32(1.0)
    r = np.sqrt((d.astype(np.float64) ** 2).sum(1))[:, None]
    tgt2[dirty] = (np.float32(1.0) + (d / r * 0.45)).astype(np.float32)
    slots2 = _in_cells(synth.uniform(41, 3, w * w, 0.0, 1.0, shift=False), w, cell)
    return EditCase(w, cell, cell, gen, tgt, tgt2, dirty, slots2, (26, 14, 36, 26))


def run_oracle(orc, case: EditCase, acc=None, pow_mode=None, nthreads=4):
    """The sequence on the oracle (fixed-point mode unless acc / pow_mode say
    otherwise). Returns ((gen, m, v, losses) after the global schedule, the
    same after the local one, the oracle fit)."""
    kw = {}
    if acc is not None:
        kw.update(acc=acc, pow_mode=pow_mode)
    f = orc.Fit(2.0, 2.0, case.spacing, case.K, case.lr_per_spacing, case.fraction, case.iterations,
                nthreads=nthreads, **kw)
    f.set_targets(case.targets)
    f.set_generators(case.generators, case.slots, case.slots, case.slot_cell)
    l1 = np.float32([f.step(1) for _ in range(case.global_steps)])
    mid = f.generators() + (l1,)
    f.set_targets(case.targets2)  # UpdateTargets: same capacity, the dirty slots changed
    f.update_generators(case.slots2, *case.rect)
    f.begin_schedule(case.local_iterations, *case.rect)
    l2 = np.float32([f.step(1) for _ in range(f.schedule_length() - f.iteration())])
    return mid, f.generators() + (l2,), f
