"""GPU canvas parity: RasterizeShape and StampDisc on the device equal the
oracle's restatement of src/voromesh/canvas.cpp bit for bit (occupancy,
surface masks and points, slot values and indices, free list, edit counts and
dirty lists); the canvas-to-optimiser hand-off equals the host route."""
import numpy as np
import pytest

import canvas_shapes

pytestmark = pytest.mark.gpu


def _same(gpu_state, orc_state, orc):
    pi = orc.canvas_relabelling(gpu_state, orc_state)
    # the device visits rim voxels in the oracle's order: no relabelling at all
    assert np.array_equal(pi, np.arange(len(pi)))
    assert np.array_equal(gpu_state["free"], orc_state["free"])


@pytest.mark.parametrize("name", canvas_shapes.NAMES)
def test_rasterize_bit_exact(vm, orc, name):
    (w, h, vs), poly = canvas_shapes.shape(name)
    c = vm.Canvas(w, h, vs)
    c.RasterizeShape(poly)
    o = orc.Canvas(w, h, vs)
    o.rasterize(poly)
    _same(c.state(), o.state(), orc)
    c.close()


@pytest.mark.parametrize("name", ["heart_1k", "comb", "odd_grid"])
def test_rasterize_without_edge_buckets(vm, orc, monkeypatch, name):
    """The scanline kernels' path that tests every edge (taken when the
    per-row edge buckets would be too large) gives the same canvas."""
    monkeypatch.setenv("VM_CANVAS_BUCKET_CAP", "0")
    (w, h, vs), poly = canvas_shapes.shape(name)
    c = vm.Canvas(w, h, vs)
    c.RasterizeShape(poly)
    o = orc.Canvas(w, h, vs)
    o.rasterize(poly)
    _same(c.state(), o.state(), orc)


def test_rasterize_crossing_limit(vm, orc):
    """A scanline crossed by more than 32768 edges is reported as unsupported
    (status 7) and leaves the canvas empty; one just under the limit
    (block-per-row path) still matches the oracle."""
    from voromesh_gb300 import synth

    c = vm.Canvas(131072.0, 16.0, 1.0)
    c.RasterizeShape(synth.heart(64.0, 8.0, 12.0, 64))
    assert c.SurfaceCount() > 0
    with pytest.raises(vm.VmError) as err:
        c.RasterizeShape(synth.comb(1.0, 2.0, 131000.0, 10.0, 17000))
    assert err.value.code == 7
    assert c.SurfaceCount() == 0 and c.TargetSlots().shape == (0, 2) and not c.InsideMasks().any()
    c.close()
    poly = synth.comb(1.0, 2.0, 60000.0, 10.0, 8000)  # 16000 crossings
    c = vm.Canvas(65536.0, 16.0, 1.0)
    c.RasterizeShape(poly)
    o = orc.Canvas(65536.0, 16.0, 1.0)
    o.rasterize(poly)
    assert np.array_equal(c.InsideMasks(), o.inside())
    assert np.array_equal(c.TargetSlots().view(np.uint32), o.slots().view(np.uint32))


def test_rasterize_rejects_non_finite(vm):
    c = vm.Canvas(8.0, 8.0, 1.0)
    with pytest.raises(vm.VmError):
        c.RasterizeShape(np.array([[1.0, 1.0], [np.nan, 2.0], [3.0, 5.0]], np.float32))


def test_rasterize_empty_and_repeat(vm, orc):
    from voromesh_gb300 import synth

    c = vm.Canvas(64.0, 64.0, 1.0)
    c.RasterizeShape(synth.heart(32.0, 32.0, 50.0, 300))
    c.RasterizeShape(np.zeros((0, 2), np.float32))
    assert c.SurfaceCount() == 0 and c.TargetSlots().shape == (0, 2) and not c.InsideMasks().any()
    c.RasterizeShape(synth.heart(30.0, 33.0, 40.0, 200))
    o = orc.Canvas(64.0, 64.0, 1.0)
    o.rasterize(synth.heart(30.0, 33.0, 40.0, 200))
    _same(c.state(), o.state(), orc)


@pytest.mark.parametrize("w,vs,segs,seed", [(1024.0, 1.0, 4096, 1), (2.0, 2.0 / 1024, 4096, 2), (100.0, 0.37, 50, 3),
                                            (64.0, 1.0, 7, 4)])
def test_stamp_sequence_bit_exact(vm, orc, w, vs, segs, seed):
    from voromesh_gb300 import synth

    poly = synth.heart(0.5 * w, 0.5 * w, 0.8 * w, segs)
    c = vm.Canvas(w, w, vs)
    o = orc.Canvas(w, w, vs)
    c.RasterizeShape(poly)
    o.rasterize(poly)
    rng = np.random.default_rng(seed)
    for k in range(40):
        cx, cy = rng.uniform(-0.1 * w, 1.1 * w, 2).astype(np.float32)
        r = np.float32(rng.uniform(0.5, 0.15 * w / vs) * vs)
        ins = bool(rng.integers(2))
        eg = c.StampDisc((cx, cy), r, ins)
        eo = o.stamp(cx, cy, r, ins)
        assert (eg.tx0, eg.ty0, eg.tx1, eg.ty1) == eo.rect()
        assert (eg.removed, eg.added, eg.flipped) == eo.counts()
        assert np.array_equal(eg.dirtySlots, eo.dirty)
        assert eg.Changed() == (sum(eo.counts()) > 0)
        if k % 8 == 7:
            _same(c.state(), o.state(), orc)
    _same(c.state(), o.state(), orc)
    assert c.SurfaceTileCount() == o.counts()[3]


def test_stamp_edges(vm, orc):
    """Stamps off the domain, of zero radius, covering the whole canvas, and
    on a canvas never rasterised."""
    from voromesh_gb300 import synth

    c = vm.Canvas(64.0, 40.0, 1.0)
    o = orc.Canvas(64.0, 40.0, 1.0)
    seq = [(-100.0, -100.0, 5.0, True), (32.0, 20.0, 0.0, True), (10.0, 10.0, 6.0, True), (12.0, 12.0, 3.0, False),
           (32.0, 20.0, 100.0, False), (32.0, 20.0, 8.0, True), (70.0, 45.0, 9.0, True), (0.0, 0.0, 2.5, False)]
    for cx, cy, r, ins in seq:
        eg = c.StampDisc((cx, cy), r, ins)
        eo = o.stamp(cx, cy, r, ins)
        assert (eg.tx0, eg.ty0, eg.tx1, eg.ty1) == eo.rect() and (eg.removed, eg.added, eg.flipped) == eo.counts()
        assert np.array_equal(eg.dirtySlots, eo.dirty)
    _same(c.state(), o.state(), orc)
    poly = synth.heart(30.0, 20.0, 30.0, 64)
    c.RasterizeShape(poly)
    o.rasterize(poly)
    _same(c.state(), o.state(), orc)


def test_stamp_rejects_bad_input(vm, orc):
    """A non-finite centre or radius is an argument error and a radius whose
    rim needs more than 2^28 samples is unsupported; neither changes the
    canvas. Centres far off the domain (beyond the int range in voxels) are
    empty edits."""
    from voromesh_gb300 import synth

    poly = synth.heart(32.0, 32.0, 50.0, 300)
    c = vm.Canvas(64.0, 64.0, 1.0)
    o = orc.Canvas(64.0, 64.0, 1.0)
    c.RasterizeShape(poly)
    o.rasterize(poly)
    for cx, cy, r in [(np.nan, 3.0, 2.0), (3.0, np.inf, 2.0), (3.0, 3.0, np.nan)]:
        with pytest.raises(vm.VmError) as err:
            c.StampDisc((cx, cy), r, True)
        assert err.value.code == 1
    with pytest.raises(vm.VmError) as err:
        c.StampDisc((32.0, 32.0), 1e9, False)
    assert err.value.code == 7
    for cx, cy in [(3e10, 5.0), (-3e10, 5.0), (5.0, 3e10), (5.0, -3e10)]:
        e = c.StampDisc((cx, cy), 4.0, True)
        assert not e.Changed() and len(e.dirtySlots) == 0
    _same(c.state(), o.state(), orc)


def test_canvas_handoff_equals_host_route(vm):
    """SetTargetsFromCanvas / UpdateFromCanvas (device to device) leave the
    optimiser exactly as SetTargets/SetOccupancy and UpdateTargets/
    UpdateOccupancy with the canvas's host arrays do (the editor's sequence,
    apps/voromesh_demo.cpp:103-125)."""
    from voromesh_gb300 import synth

    W, vs, radius = 256.0, 1.0, 8.0
    canvas = vm.Canvas(W, W, vs)
    canvas.RasterizeShape(synth.heart(128.0, 128.0, 200.0, 1024))
    sampler = vm.Sampler(W, W, radius, 30, 1)
    params = vm.OptimizerParams(sampleFraction=0.2)
    a = vm.VoroOptimizer(W, W, radius, params)
    b = vm.VoroOptimizer(W, W, radius, params)
    a.SetTargetsFromCanvas(canvas)
    b.SetTargets(canvas.TargetSlots())
    b.SetOccupancy(canvas.InsideMasks(), canvas.TilesX(), canvas.TilesY(), canvas.VoxelSize())
    for o in (a, b):
        o.SetGenerators(sampler.Cells(), sampler.GridW(), sampler.GridH(), sampler.CellSize())
        o.BeginSchedule(60)
        o.Optimize()
    assert np.array_equal(a.Generators(), b.Generators())
    rng = np.random.default_rng(5)
    for k in range(6):
        cx, cy = rng.uniform(60, 196, 2)
        e = canvas.StampDisc((cx, cy), 14.0, bool(k % 2))
        if not e.Changed():
            continue
        a.UpdateFromCanvas(canvas)
        b.UpdateTargets(e.dirtySlots, canvas.TargetSlots())
        b.UpdateOccupancy(canvas.InsideMasks(), e.tx0, e.ty0, e.tx1, e.ty1)
        for o in (a, b):
            o.BeginSchedule(20)
            o.Optimize()
        assert np.array_equal(a.Generators(), b.Generators())
        assert a.EvaluateLoss() == b.EvaluateLoss()
    ma, mb = a.Extract(), b.Extract()
    assert np.array_equal(ma.inside, mb.inside) and np.array_equal(ma.vertices, mb.vertices)
