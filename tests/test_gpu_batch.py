"""Batched fits and serving: every fit's result equals the same fit run alone
(bit for bit), in a batch of uneven sizes and in the served mix, and batch
members and served requests equal the CPU oracle's fit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_batch(n_fits=12, seed=3):
    from voromesh_gb300 import synth

    return synth.uneven_batch(n_fits=n_fits, lo=200, hi=6000, tgt_per_gen=4, steps=30, seed=seed)


def alone(spec, steps):
    import voromesh_gb300 as vm
    from voromesh_gb300.batch import params_for

    o = vm.VoroOptimizer(spec.width, spec.height, spec.spacing, params_for(spec))
    o.SetTargets(spec.targets)
    o.SetGenerators(spec.generators, spec.slotsW, spec.slotsH, spec.slotCellSize)
    o.Step(steps)
    g = o.Generators()
    o.close()
    return g


def oracle_run(orc, spec, steps):
    """The fit on the CPU oracle (the same arithmetic), with the schedule
    params_for gives it; returns its generators after `steps` steps."""
    ref = orc.Fit(spec.width, spec.height, spec.spacing, spec.lossK, spec.lrPerSpacing, spec.sampleFraction,
                  spec.steps, nthreads=8)
    ref.set_targets(spec.targets)
    ref.set_generators(spec.generators, spec.slotsW, spec.slotsH, spec.slotCellSize)
    ref.step(steps)
    return ref.generators()[0]


def test_batch_equals_alone(vm, orc):
    from voromesh_gb300.batch import Batch

    specs = small_batch()
    b = Batch(1 << 30, max_fits=64)
    ids = [b.add(s) for s in specs]
    b.step(30)
    for fid, spec in zip(ids, specs):
        assert b.info(fid).iteration == 30
        assert np.array_equal(b.generators(fid), alone(spec, 30))
    # batch members against the oracle: the smallest and the largest fit
    sizes = [len(s.generators) for s in specs]
    for k in (int(np.argmin(sizes)), int(np.argmax(sizes))):
        assert np.array_equal(b.generators(ids[k]), oracle_run(orc, specs[k], 30))
    b.close()


def test_batch_membership_changes(vm):
    """Fits join and leave between steps; the others are unaffected."""
    from voromesh_gb300.batch import Batch

    specs = small_batch(6, seed=4)
    b = Batch(1 << 30, max_fits=16)
    a = [b.add(s) for s in specs[:3]]
    b.step(10)
    b.remove(a[1])
    c = [b.add(s) for s in specs[3:]]
    b.step(10)
    assert np.array_equal(b.generators(a[0]), alone(specs[0], 20))
    assert np.array_equal(b.generators(a[2]), alone(specs[2], 20))
    for fid, spec in zip(c, specs[3:]):
        assert np.array_equal(b.generators(fid), alone(spec, 10))
    b.close()


def test_budget_admission(vm):
    from voromesh_gb300.batch import Batch, fit_bytes
    from voromesh_gb300._lib import VmError

    specs = small_batch(4, seed=5)
    need = max(fit_bytes(s) for s in specs)
    b = Batch(int(need * 1.5), max_fits=8)
    b.add(specs[0])
    with pytest.raises(VmError) as e:
        for s in specs[1:]:
            b.add(s)
    assert e.value.code == 5  # VM_ERR_BUDGET
    b.close()


def test_serve_equals_alone(vm, orc):
    """Served results (continuous batching, staggered arrivals) equal each
    request run alone for the same number of steps."""
    from voromesh_gb300.batch import serve

    specs = small_batch(8, seed=6)
    arrivals = np.linspace(0.0, 0.05, len(specs))
    r = serve(specs, arrivals, hbm_budget=1 << 30, max_live=64, steps_per_round=10, max_steps=40, rel_tol=0.0)
    assert np.all(r.status == 0) and np.all(r.steps == 40)
    assert np.all(r.finished >= r.arrival)
    for spec, g in zip(specs, r.generators):
        assert np.array_equal(g, alone(spec, 40))
    # a served request against the oracle
    k = int(np.argmax([len(s.generators) for s in specs]))
    assert np.array_equal(r.generators[k], oracle_run(orc, specs[k], 40))
    one = serve(specs, arrivals, hbm_budget=1 << 30, max_live=1, steps_per_round=10, max_steps=40, rel_tol=0.0)
    for g1, g2 in zip(one.generators, r.generators):
        assert np.array_equal(g1, g2)


def test_serve_target_cap(vm):
    """A live-target cap changes when requests are admitted, not their results."""
    from voromesh_gb300.batch import serve

    specs = small_batch(6, seed=8)
    arrivals = np.zeros(len(specs))
    cap = max(len(s.targets) for s in specs) + 1
    r = serve(specs, arrivals, hbm_budget=1 << 30, max_live=64, steps_per_round=10, max_steps=20, rel_tol=0.0,
              max_live_targets=cap)
    assert np.all(r.status == 0)
    # with the cap, no two requests both larger than half of it ran together
    big = [i for i, s in enumerate(specs) if len(s.targets) > cap // 2]
    for a in big:
        for b in big:
            if a < b:
                assert r.admitted[b] >= r.finished[a] or r.admitted[a] >= r.finished[b]
    for spec, g in zip(specs, r.generators):
        assert np.array_equal(g, alone(spec, 20))


def test_serve_rejects_a_bad_request_and_serves_the_rest(vm):
    """A request the batch cannot take (an unsupported lossK) gets that status;
    the other requests are served as if it had not been sent."""
    import dataclasses

    from voromesh_gb300.batch import serve

    specs = small_batch(5, seed=9)
    specs[2] = dataclasses.replace(specs[2], lossK=7)
    arrivals = np.linspace(0.0, 0.02, len(specs))
    r = serve(specs, arrivals, hbm_budget=1 << 30, max_live=64, steps_per_round=10, max_steps=20, rel_tol=0.0)
    assert r.status[2] == 7 and r.steps[2] == 0
    for i, (spec, g) in enumerate(zip(specs, r.generators)):
        if i != 2:
            assert r.status[i] == 0 and np.array_equal(g, alone(spec, 20))
