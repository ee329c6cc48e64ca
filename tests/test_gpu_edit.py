"""GPU parity of the editor's local edit (apps/voromesh_demo.cpp:117-140):
the global schedule, then UpdateTargets of the dirty target slots,
UpdateGenerators and BeginSchedule(localIterations, rect) over a rectangle of
generator slots, and Optimize -- against the oracle (same fixed-point
arithmetic), bit for bit: positions, Adam moments, every step's batch loss and
the step counter, through three scaled milestones with a 0.2 sample fraction.
The oracle's rectangle schedule is pinned to the reference's own kernels
(tests/test_oracle_pins.py).
"""
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent))
from edit_case import edit_case, run_oracle  # noqa: E402

pytestmark = pytest.mark.gpu


def _params(vm, case):
    return vm.OptimizerParams(iterations=case.iterations, localIterations=case.local_iterations,
                              sampleFraction=case.fraction, lrPerSpacing=case.lr_per_spacing, lossK=case.K)


def test_local_edit_bit_exact(vm, orc):
    case = edit_case()
    (rg1, rm1, rv1, rl1), (rg2, rm2, rv2, rl2), ref = run_oracle(orc, case)
    opt = vm.VoroOptimizer(2.0, 2.0, case.spacing, _params(vm, case))
    opt.SetTargets(case.targets)
    opt.SetGenerators(case.generators, case.slots, case.slots, case.slot_cell)
    losses = []
    for _ in range(case.global_steps):
        opt.Step(1)
        losses.append(opt.LastBatchLoss())
    assert np.array_equal(np.float32(losses), rl1)
    m, v = opt.Moments()
    assert np.array_equal(opt.Generators(), rg1) and np.array_equal(m, rm1) and np.array_equal(v, rv1)
    # the edit, in the editor's order
    opt.UpdateTargets(case.dirty, case.targets2)
    opt.UpdateGenerators(case.slots2, *case.rect)
    opt.BeginSchedule(opt.Params().localIterations, *case.rect)
    assert opt.ScheduleLength() == case.local_iterations and opt.Iteration() == 0
    losses = []
    while opt.Iteration() < opt.ScheduleLength():
        opt.Step(1)
        losses.append(opt.LastBatchLoss())
    assert np.array_equal(np.float32(losses), rl2)
    m, v = opt.Moments()
    assert np.array_equal(opt.Generators(), rg2) and np.array_equal(m, rm2) and np.array_equal(v, rv2)
    assert opt.Iteration() == ref.iteration() == case.local_iterations
    # frozen slots kept their positions through the local schedule
    cx0, cy0, cx1, cy1 = case.rect
    frozen = np.ones((case.slots, case.slots), bool)
    frozen[cy0:cy1, cx0:cx1] = False
    assert np.array_equal(opt.Generators()[frozen.reshape(-1)], rg1[frozen.reshape(-1)])


def test_local_edit_optimize_in_one_call(vm, orc):
    """The same edit with Optimize() as one call (one graph launch per step,
    one read-back): the same final state as the oracle's."""
    case = edit_case()
    _, (rg2, rm2, rv2, rl2), _ = run_oracle(orc, case)
    opt = vm.VoroOptimizer(2.0, 2.0, case.spacing, _params(vm, case))
    opt.SetTargets(case.targets)
    opt.SetGenerators(case.generators, case.slots, case.slots, case.slot_cell)
    opt.Step(case.global_steps)
    opt.UpdateTargets(case.dirty, case.targets2)
    opt.UpdateGenerators(case.slots2, *case.rect)
    opt.BeginSchedule(case.local_iterations, *case.rect)
    opt.Optimize()
    m, v = opt.Moments()
    assert np.array_equal(opt.Generators(), rg2) and np.array_equal(m, rm2) and np.array_equal(v, rv2)
    assert np.float32(opt.LastBatchLoss()) == rl2[-1]
