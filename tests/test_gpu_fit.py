"""GPU fit parity: the CUDA optimiser against the CPU oracle, bit-exact.

The product sums gradients and losses in order-independent fixed point, so
its trajectory is a deterministic function of the inputs and the oracle
(same arithmetic, same sums) must reproduce it exactly, step for step.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(vm, orc, gen, tgt, spacing, K, steps, fraction, slots=None, seed=1, iters=300, lr_ps=0.09):
    from voromesh_gb300 import OptimizerParams, VoroOptimizer

    sw, sh = slots or (len(gen), 1)
    p = OptimizerParams(iterations=iters, sampleFraction=fraction, lrPerSpacing=lr_ps, lossK=K, seed=seed)
    opt = VoroOptimizer(2.0, 2.0, spacing, p)
    opt.SetTargets(tgt)
    opt.SetGenerators(gen, sw, sh, 2.0)
    ref = orc.Fit(2.0, 2.0, spacing, K, lr_ps, fraction, iters, seed=seed)
    ref.set_targets(tgt)
    ref.set_generators(gen, sw, sh, 2.0)
    return opt, ref


@pytest.mark.parametrize("K,fraction", [(12, 1.0), (12, 0.2), (16, 1.0), (8, 0.5), (32, 1.0)])
def test_fit_bit_exact(vm, orc, K, fraction):
    from voromesh_gb300 import synth

    gen = synth.uniform(3, 1, 1024)
    tgt = synth.circle(3, 2, 8192, 0.6, 1e-3)
    opt, ref = _pair(vm, orc, gen, tgt, 0.06, K, 0, fraction)
    for chunk in (1, 4, 15):
        opt.Step(chunk)
        lref = ref.step(chunk)
        g, m, v = ref.generators()
        assert np.array_equal(opt.Generators(), g)
        om, ov = opt.Moments()
        assert np.array_equal(om, m) and np.array_equal(ov, v)
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    assert opt.Iteration() == ref.iteration() == 20
    assert np.float32(opt.EvaluateLoss()) == np.float32(ref.eval_loss())


def test_exact_path_targets(vm, orc):
    """Targets far from every generator (outside the domain, in empty regions)
    miss the block certificates and take the deferred exact ring search."""
    from voromesh_gb300 import synth

    gen = synth.uniform(4, 1, 600, -0.5, 0.5)  # generators in the middle only
    tgt = np.concatenate([synth.circle(4, 2, 3000, 0.9, 0.05), synth.uniform(4, 3, 500, -1.2, 1.2)])
    opt, ref = _pair(vm, orc, gen, tgt, 0.05, 16, 0, 1.0)
    opt.Step(6)
    lref = ref.step(6)
    assert opt.info().exactTargets > 0
    assert np.array_equal(opt.Generators(), ref.generators()[0])
    assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    i0, j, loss, _, cnt, _ = opt.Probe(1)
    ri0, rj, rloss = orc.loss_detail(ref, tgt, 16)
    assert np.array_equal(i0, ri0) and np.array_equal(j, rj) and np.array_equal(loss, rloss)


def test_grid_bit_exact(vm, orc):
    from voromesh_gb300 import synth

    gen = synth.uniform(5, 1, 3000)
    gen[::7] = -1.0  # empty slots
    tgt = synth.circle(5, 2, 4000, 0.5, 1e-2)
    opt, ref = _pair(vm, orc, gen, tgt, 0.05, 12, 0, 1.0)
    start, sidx, spos, gcell = opt.Grid()
    r = ref.grid()
    assert np.array_equal(start, r[0]) and np.array_equal(sidx, r[1])
    assert np.array_equal(spos, r[2]) and np.array_equal(gcell, r[3])
    opt.Step(3)
    ref.step(3)
    start, sidx, spos, gcell = opt.Grid()
    r = ref.grid()
    assert np.array_equal(start, r[0]) and np.array_equal(sidx, r[1]) and np.array_equal(gcell, r[3])


@pytest.mark.parametrize("K", [8, 12, 16, 24, 32])
def test_knn_bit_exact(vm, orc, K):
    from voromesh_gb300 import synth

    gen = synth.uniform(9, 1, 2000)
    q = synth.uniform(9, 2, 3000)
    opt, _ = _pair(vm, orc, gen, q, 0.05, 12, 0, 1.0)
    idx, d2 = opt.Knn(q, K)
    grid = orc.Grid(gen, 40, 40, 0.05)
    ridx, rd2 = grid.knn(q, K)
    assert np.array_equal(idx, ridx)
    assert np.array_equal(d2, rd2)
    # the caller's own output arrays, filled in place
    out = (np.full((len(q), K), -7, np.int32), np.full((len(q), K), -7.0, np.float32))
    i2, e2 = opt.Knn(q, K, out=out)
    assert i2 is out[0] and e2 is out[1]
    assert np.array_equal(out[0], ridx) and np.array_equal(out[1], rd2)
    with pytest.raises(ValueError):
        opt.Knn(q, K, out=(out[0][:, :K - 1], out[1]))


def test_probe_matches_oracle(vm, orc):
    """Per-target decisions (nearest site, bisector neighbour, loss) and the summed gradient."""
    from voromesh_gb300 import synth

    gen = synth.uniform(11, 1, 800)
    tgt = synth.circle(11, 2, 6000, 0.7, 5e-3)
    opt, ref = _pair(vm, orc, gen, tgt, 0.07, 16, 0, 1.0)
    i0, j, loss, grad, cnt, ls = opt.Probe(0)
    g, rcnt, rls = ref.gradient()
    assert cnt == rcnt
    assert np.array_equal(grad, g)
    assert np.float32(ls) == np.float32(rls)


@pytest.mark.parametrize("sub", ["0", "2"])
def test_loss_variants_and_target_order_agree(vm, orc, monkeypatch, sub):
    """Every loss kernel variant (block shape) and target sort order gives the
    identical trajectory, equal to the oracle's: the sums are order free."""
    from voromesh_gb300 import synth

    monkeypatch.setenv("VM_TARGET_SUB", sub)
    gen = synth.uniform(5, 1, 2048)
    tgt = synth.circle(5, 2, 60000, 0.7, 2e-3)
    opt, ref = _pair(vm, orc, gen, tgt, 0.04, 16, 0, 1.0)
    ref.step(6)
    g, m, v = ref.generators()
    _, count = opt.LossVariant()
    for variant in range(count):
        opt.SetLossVariant(variant)
        opt.SetGenerators(gen, len(gen), 1, 2.0)
        opt.Step(6)
        assert np.array_equal(opt.Generators(), g), f"variant {variant}"


@pytest.mark.parametrize("jitter", [1e-6, 0.0])
def test_lattice_fit_bit_exact(vm, orc, jitter):
    """The precision-stress shape: a jittered (or exact) lattice of sites, where
    bisector distances tie or nearly tie, so the staged path's exact fallbacks
    and the deferred ring search both run; the trajectory equals the oracle's."""
    from voromesh_gb300 import synth

    gen = synth.lattice(3, 5, 64, 64, jitter)
    tgt = synth.five_arm_star(3, 6, 40000)
    opt, ref = _pair(vm, orc, gen, tgt, 2.0 / 64, 16, 0, 1.0)
    for chunk in (1, 9):
        opt.Step(chunk)
        ref.step(chunk)
        g, m, v = ref.generators()
        assert np.array_equal(opt.Generators(), g)


@pytest.mark.parametrize("fraction,rect", [(1.0, None), (0.2, None), (0.2, (3, 2, 40, 30))])
def test_checkpoint_resume_bit_exact(vm, fraction, rect):
    """Checkpoint after some steps, restore into a fresh optimiser: the rest of
    the run (positions, moments, batch loss, step counter) equals the
    uninterrupted run bit for bit, through a learning-rate milestone and with
    the step-seeded subsample."""
    from voromesh_gb300 import synth

    gen = synth.uniform(5, 1, 48 * 48).reshape(-1, 2)
    tgt = synth.circle(5, 2, 20000, 0.6, 1e-3)
    p = vm.OptimizerParams(iterations=120, sampleFraction=fraction, lossK=12)

    def fresh():
        o = vm.VoroOptimizer(2.0, 2.0, 2.0 / 48, p)
        o.SetTargets(tgt)
        return o

    a = fresh()
    a.SetGenerators(gen, 48, 48, 2.0 / 48)
    if rect:
        a.BeginSchedule(90, *rect)
    a.Step(70)  # past the first milestone (80 of 120 scaled)
    ck = a.Checkpoint()
    a.Step(30)
    b = fresh()
    b.Restore(ck)
    assert b.Iteration() == ck["info"]["iteration"] == 70
    b.Step(30)
    assert np.array_equal(a.Generators(), b.Generators())
    ma, va = a.Moments()
    mb, vb = b.Moments()
    assert np.array_equal(ma, mb) and np.array_equal(va, vb)
    assert a.LastBatchLoss() == b.LastBatchLoss() and a.Iteration() == b.Iteration()


def test_steps_after_every_target_is_removed(vm, orc):
    """With no live targets the step still follows the Adam schedule: the
    moments decay and the sites keep moving as the oracle's do."""
    from voromesh_gb300 import synth

    gen = synth.uniform(6, 1, 512)
    tgt = synth.circle(6, 2, 4096, 0.6, 1e-3)
    opt, ref = _pair(vm, orc, gen, tgt, 0.1, 12, 0, 1.0, iters=40)
    opt.Step(8)
    ref.step(8)
    empty = np.full_like(tgt, -1.0)
    opt.UpdateTargets(np.arange(len(tgt)), empty)
    ref.set_targets(empty)
    for _ in range(3):
        opt.Step(4)
        ref.step(4)
        g, m, v = ref.generators()
        assert np.array_equal(opt.Generators(), g)
        om, ov = opt.Moments()
        assert np.array_equal(om, m) and np.array_equal(ov, v)
    assert opt.info().liveTargets == 0


def _one_sided_fit():
    """Three sites and 2^20 targets in a small cluster far to their right:
    every target pulls the same site the same way, so the per-site gradient
    sums reach about 2^63.8 in fixed point, past what one int64 can hold."""
    from voromesh_gb300 import synth

    gen = np.array([[0.2, 1.0], [1.0, 1.0], [1.0, 0.2]], np.float32)
    tgt = (synth.uniform(23, 2, 1 << 20, -0.02, 0.02, shift=False) + np.float32([1.9, 1.0])).astype(np.float32)
    return gen, tgt


def test_gradient_sums_past_int64(vm, orc):
    """The exact split gradient sums: the GPU gradient equals the oracle's bit
    for bit and stays within 1e-6 of the FP64 gradient (a wrapped 64-bit sum
    would be off by 2^64 units), and three steps of positions and moments
    equal the oracle's."""
    gen, tgt = _one_sided_fit()
    opt, ref = _pair(vm, orc, gen, tgt, 0.1, 12, 0, 1.0, slots=(3, 1))
    _, _, _, grad, cnt, _ = opt.Probe(0)
    g, rcnt, _ = ref.gradient()
    assert cnt == rcnt == len(tgt)
    assert np.array_equal(grad, g)
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.1)), 12, 0.09, 1.0, 300)
    d.set_targets(tgt)
    d.set_generators(gen, 3, 1, 2.0)
    g64, _, _ = d.gradient()
    e = orc.lib().vo_fixed_grad_exp(np.float32(0.1))
    assert np.log2(np.abs(g64).max()) + e > 63.5  # the sums do pass 2^63
    assert np.abs(grad - g64).max() <= 1e-6 * np.abs(g64).max()
    opt.Step(3)
    ref.step(3)
    rg, rm, rv = ref.generators()
    om, ov = opt.Moments()
    assert np.array_equal(opt.Generators(), rg)
    assert np.array_equal(om, rm) and np.array_equal(ov, rv)


def _near_pair_fit():
    """Two sites 5e-4 apart and 2^18 targets in a small cluster diagonal to
    them, within the staged 5x5 block: every target resolves on the fast path
    with large gradient terms (the sites nearly coincide), and two sites' sums
    reach about 2^63.4 in fixed point."""
    from voromesh_gb300 import synth

    gen = np.array([[1.0, 1.0], [1.0005, 1.0], [0.3, 0.3], [1.7, 1.7]], np.float32)
    tgt = (synth.uniform(24, 2, 1 << 18, -0.003, 0.003, shift=False) + np.float32([1.018, 1.018])).astype(np.float32)
    return gen, tgt


def test_fast_path_gradient_past_int64(vm, orc):
    """A fit whose fast-path terms break the per-fit bound (most targets in a
    5x5 block times the largest term): the fit is flagged, its gradient is
    recomputed in the exact split words, and the result equals the oracle's
    bit for bit and FP64 within 1e-6, with no target deferred."""
    gen, tgt = _near_pair_fit()
    opt, ref = _pair(vm, orc, gen, tgt, 0.05, 12, 0, 1.0, slots=(4, 1))
    _, _, _, grad, cnt, _ = opt.Probe(0)
    g, rcnt, _ = ref.gradient()
    assert cnt == rcnt == len(tgt)
    assert np.array_equal(grad, g)
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.05)), 12, 0.09, 1.0, 300)
    d.set_targets(tgt)
    d.set_generators(gen, 4, 1, 2.0)
    g64, _, _ = d.gradient()
    assert np.log2(np.abs(g64).max()) + orc.lib().vo_fixed_grad_exp(np.float32(0.05)) > 63.2
    assert np.abs(grad - g64).max() <= 1e-6 * np.abs(g64).max()
    opt.Step(3)
    ref.step(3)
    rg, rm, rv = ref.generators()
    om, ov = opt.Moments()
    assert np.array_equal(opt.Generators(), rg)
    assert np.array_equal(om, rm) and np.array_equal(ov, rv)
    assert opt.info().exactTargets == 0


def test_loss_windows_follow_the_live_target_count(vm, orc):
    """The loss pass's windows follow every target change: 540,000 live
    targets walk windows of 32 in target order, 513,000 (under 2^19)
    cell-aligned windows, then 540,000 again; every phase steps exactly as
    the oracle."""
    from voromesh_gb300 import synth

    from voromesh_gb300 import OptimizerParams, VoroOptimizer

    gen = synth.uniform(8, 1, 2048)
    tgt = synth.circle(8, 2, 540000, 0.6, 2e-3)
    opt = VoroOptimizer(2.0, 2.0, 0.05, OptimizerParams(iterations=60, sampleFraction=1.0, lossK=12))
    opt.SetTargets(tgt)
    opt.SetGenerators(gen, len(gen), 1, 2.0)
    ref = orc.Fit(2.0, 2.0, 0.05, 12, 0.09, 1.0, 60, nthreads=8)
    ref.set_targets(tgt)
    ref.set_generators(gen, len(gen), 1, 2.0)
    cur = tgt.copy()
    drop = np.arange(0, len(tgt), 20)  # 27,000 targets
    for phase in range(3):
        if phase:
            cur[drop] = -1.0 if phase == 1 else tgt[drop]
            opt.UpdateTargets(drop, cur)
            ref.set_targets(cur)
        opt.Step(2)
        lref = ref.step(2)
        g, m, v = ref.generators()
        assert np.array_equal(opt.Generators(), g), phase
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
        assert opt.info().liveTargets == (513000 if phase == 1 else 540000)


@pytest.mark.parametrize("slots_w,slots_h,width,spacing", [
    (64, 64, 2.0, 2.0 / 128),   # 4,096 slots, 128 x 64 = 8,192 cells: the one-block step
    (4097, 1, 2.0, 2.0 / 128),  # one slot more: the six-kernel step
    (64, 64, 2.0, 2.0 / 129),   # 129 x 65 cells: the six-kernel step
])
def test_step_at_the_small_fit_limits(vm, orc, slots_w, slots_h, width, spacing):
    """Fits at and just past the one-block step's limits (4,096 slots, 8,192
    grid cells) step exactly as the oracle, through a milestone."""
    from voromesh_gb300 import OptimizerParams, VoroOptimizer, synth

    n = slots_w * slots_h
    # sites over [0,2] x [0,1], targets on a circle inside it
    gen = (synth.uniform(31, 1, n, -1.0, 1.0, shift=False) * np.float32([1.0, 0.5]) + np.float32([1.0, 0.5]))
    gen = gen.astype(np.float32)
    gen[::9] = -1.0  # empty slots
    tgt = (synth.circle(31, 2, 6000, 0.4, 1e-3, shift=False) + np.float32([1.0, 0.5])).astype(np.float32)
    p = OptimizerParams(iterations=40, sampleFraction=0.5, lossK=12, milestones=(6, 30, 35, 38))
    opt = VoroOptimizer(width, 1.0, spacing, p)
    opt.SetTargets(tgt)
    cs = max(2.0 / slots_w, 1.0 / slots_h)  # the slot rectangle covers the domain: every target takes part
    opt.SetGenerators(gen, slots_w, slots_h, cs)
    ref = orc.Fit(width, 1.0, spacing, 12, 0.09, 0.5, 40, milestones=(6, 30, 35, 38), nthreads=4)
    ref.set_targets(tgt)
    ref.set_generators(gen, slots_w, slots_h, cs)
    for chunk in (3, 5):
        opt.Step(chunk)
        lref = ref.step(chunk)
        g, m, v = ref.generators()
        assert np.array_equal(opt.Generators(), g)
        om, ov = opt.Moments()
        assert np.array_equal(om, m) and np.array_equal(ov, v)
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    start, sidx, spos, gcell = opt.Grid()
    r = ref.grid()
    assert np.array_equal(start, r[0]) and np.array_equal(sidx, r[1]) and np.array_equal(gcell, r[3])
