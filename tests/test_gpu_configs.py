"""GPU parity at the benchmark configurations themselves, against the oracle
(the same fixed-point arithmetic), bit for bit:

- the plain fit: 2,048 generators uniform in [-1,1]^2, 16,384 targets on the
  circle r = 0.6 with N(0, 1e-3) radial noise, k = 12, cell 0.05, lr 1e-3, all
  300 steps;
- the 1M-site fit: the r = 1e-3 Poisson fill of [0,2]^2 (2829^2 cells), the
  1,048,576 generators drawn from it, 8,388,608 targets on the union of 64
  ellipses, k = 16: the fill, the whole grid, kNN lists and per-target
  decisions on every 64th target, three full steps, and the extraction of
  the fitted sites (every cell and the boundary mesh);
- the precision stress: a 512x512 lattice jittered by 1e-6 with 2,097,152
  targets on a 5-arm star, k = 16, ten steps, and the per-target decisions
  against the FP64 oracle's at the same positions.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = max(1, min(os.cpu_count() or 1, 32))


def _opt(vm, spec, iterations):
    p = vm.OptimizerParams(iterations=iterations, sampleFraction=spec.sampleFraction, lrPerSpacing=spec.lrPerSpacing,
                           lossK=spec.lossK)
    opt = vm.VoroOptimizer(spec.width, spec.height, spec.spacing, p)
    opt.SetTargets(spec.targets)
    opt.SetGenerators(spec.generators, spec.slotsW, spec.slotsH, spec.slotCellSize)
    return opt


def _ref(orc, spec, iterations):
    ref = orc.Fit(spec.width, spec.height, spec.spacing, spec.lossK, spec.lrPerSpacing, spec.sampleFraction,
                  iterations, nthreads=THREADS)
    ref.set_targets(spec.targets)
    ref.set_generators(spec.generators, spec.slotsW, spec.slotsH, spec.slotCellSize)
    return ref


def _same_state(opt, ref):
    g, m, v = ref.generators()
    om, ov = opt.Moments()
    return np.array_equal(opt.Generators(), g) and np.array_equal(om, m) and np.array_equal(ov, v)


def test_plain_fit_all_300_steps(vm, orc):
    from voromesh_gb300 import synth

    spec = synth.plain_fit()
    opt, ref = _opt(vm, spec, 300), _ref(orc, spec, 300)
    done = 0
    for chunk in (1, 9, 40, 50, 100, 100):  # through all four milestones (80, 150, 200, 250)
        opt.Step(chunk)
        lref = ref.step(chunk)
        done += chunk
        assert _same_state(opt, ref), f"after {done} steps"
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    assert opt.Iteration() == ref.iteration() == 300
    assert np.float32(opt.EvaluateLoss()) == np.float32(ref.eval_loss())


@pytest.fixture(scope="module")
def fill_1e3(vm, orc):
    """The r = 1e-3 fill of [0,2]^2 on the GPU and on the oracle."""
    s = vm.Sampler(2.0, 2.0, 1e-3, 30, 1)
    cells, _ = orc.poisson_fill(2.0, 2.0, 1e-3, 30, 1)
    return s, cells


def test_poisson_fill_r1e3(fill_1e3):
    s, cells = fill_1e3
    assert (s.GridW(), s.GridH()) == (2829, 2829)
    assert np.array_equal(s.Cells(), cells)
    assert s.VerifyAll()
    assert (cells[:, 0] >= 0).sum() > 2_600_000


def test_scale_fit_1m(vm, orc, fill_1e3):
    from voromesh_gb300 import synth

    s, _ = fill_1e3
    spec = synth.scale_fit_from_cells(s.Cells())
    assert len(spec.generators) == 1 << 20 and len(spec.targets) == 1 << 23
    opt, ref = _opt(vm, spec, 1000), _ref(orc, spec, 1000)
    start, sidx, spos, gcell = opt.Grid()
    r = ref.grid()
    assert np.array_equal(start, r[0]) and np.array_equal(sidx, r[1])
    assert np.array_equal(spos, r[2]) and np.array_equal(gcell, r[3])
    q = np.ascontiguousarray(spec.targets[::64])
    idx, d2 = opt.Knn(q, 16)
    gw = int(round(2.0 / spec.spacing))
    ridx, rd2 = orc.Grid(spec.generators, gw, gw, spec.spacing).knn(q, 16)
    assert np.array_equal(idx, ridx) and np.array_equal(d2, rd2)
    i0, j, loss, _, cnt, _ = opt.Probe(1)
    ri0, rj, rloss = orc.loss_detail(ref, q, 16)
    assert np.array_equal(i0[::64], ri0) and np.array_equal(j[::64], rj) and np.array_equal(loss[::64], rloss)
    for step in range(3):
        opt.Step(1)
        lref = ref.step(1)
        assert _same_state(opt, ref), f"after {step + 1} steps"
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    # the cells of the fitted sites and their boundary mesh
    from test_gpu_extract import assert_cells_equal, disc_masks

    masks, tiles, voxel = disc_masks()
    opt.SetOccupancy(masks, tiles, tiles, voxel)
    mesh = opt.Extract()
    gen = ref.generators()[0]
    verts, edges, counts, inside, flags = orc.Grid(gen, gw, gw, spec.spacing).cells(
        2.0, 2.0, masks, tiles, tiles, float(np.float32(1.0) / np.float32(voxel)), nthreads=THREADS)
    assert np.array_equal(mesh.inside, inside) and inside.sum() > 100000
    assert mesh.unsafeCells == flags[0] and mesh.overflowCells == flags[1]
    assert_cells_equal(mesh, len(gen), verts, edges, counts)
    _, mv, me, wt, loops = orc.assemble(verts, edges, counts, inside)
    assert mesh.watertight == wt and mesh.loops == loops and np.array_equal(mesh.edges, me)
    assert np.array_equal(mesh.vertices.view(np.uint32), mv.view(np.uint32))


def test_precision_lattice_full_size(vm, orc):
    from voromesh_gb300 import synth

    spec = synth.precision_fit()
    assert len(spec.generators) == 512 * 512 and len(spec.targets) == 2097152
    opt, ref = _opt(vm, spec, 1000), _ref(orc, spec, 1000)
    for chunk in (1, 9):
        opt.Step(chunk)
        lref = ref.step(chunk)
        assert _same_state(opt, ref)
        assert np.float32(opt.LastBatchLoss()) == np.float32(lref)
    # per-target decisions at the fitted positions: FP32 (GPU) equals FP64
    i0, j, _, _, _, _ = opt.Probe(1)
    d = orc.Fit64(2.0, 2.0, float(np.float32(spec.spacing)), 16, spec.lrPerSpacing, 1.0, 1000, nthreads=THREADS)
    d.set_targets(spec.targets)
    d.set_generators(opt.Generators(), spec.slotsW, spec.slotsH, spec.slotCellSize)
    d64i0, d64j = d.detail()
    assert np.count_nonzero(i0 != d64i0) == 0 and np.count_nonzero(j != d64j) == 0
