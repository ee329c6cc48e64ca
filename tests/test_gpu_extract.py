"""GPU extraction parity: clipped Voronoi cells and the boundary mesh against
the CPU oracle (the reference's FP64 clipper restated).

Edge labels, vertex counts, cyclic order, vertex coordinates, occupancy and
the unsafe/overflow counts must match bit for bit: both sides clip with the
reference's FP64 interpolation along the clipped edge, one IEEE rounding per
operation, and the device's FP32 inside tests fall back to FP64 within their
error bound, so they take the FP64 test's decisions. That includes the
near-cocircular lattices, where any other arithmetic splits vertices
differently.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def disc_masks(tiles=16, radius=0.6):
    n = tiles * 8
    masks = np.zeros(tiles * tiles, np.uint64)
    for j in range(n):
        for i in range(n):
            x, y = (i + 0.5) * 2 / n - 1, (j + 0.5) * 2 / n - 1
            if x * x + y * y < radius * radius:
                masks[(j >> 3) * tiles + (i >> 3)] |= np.uint64(1) << np.uint64(((j & 7) << 3) | (i & 7))
    return masks, tiles, 2.0 / n


def cell_table(mesh, n):
    """The mesh's per-cell labels and vertices in fixed 24-wide rows."""
    cs = np.asarray(mesh.cellStart)
    cnt = np.diff(cs)
    rows = np.repeat(np.arange(n), cnt)
    cols = np.arange(cs[-1]) - np.repeat(cs[:-1], cnt)
    lab = np.full((n, 24), -9999, np.int32)
    ver = np.zeros((n, 24, 2), np.float32)
    lab[rows, cols] = mesh.cellLabels
    ver[rows, cols] = mesh.cellVerts
    return cnt, lab, ver


def assert_cells_equal(mesh, n, verts, edges, counts):
    """Every cell equals the oracle's: count, labels and vertex bits."""
    cnt, lab, ver = cell_table(mesh, n)
    assert np.array_equal(cnt, counts)
    used = np.arange(24)[None, :] < counts[:, None]
    bad = ~np.all(np.where(used, edges, -9999) == lab, axis=1)
    bad |= ~np.all(np.where(used[..., None], ver.view(np.uint32) == verts.view(np.uint32), True), axis=(1, 2))
    assert not bad.any(), f"{int(bad.sum())} cells differ, first {np.flatnonzero(bad)[:8].tolist()}"


def run_case(vm, orc, gen, spacing, tgt=None):
    from voromesh_gb300 import OptimizerParams, VoroOptimizer

    n = len(gen)
    masks, tiles, voxel = disc_masks()
    opt = VoroOptimizer(2.0, 2.0, spacing, OptimizerParams(lossK=12))
    opt.SetTargets(tgt if tgt is not None else gen[:8])
    opt.SetOccupancy(masks, tiles, tiles, voxel)
    opt.SetGenerators(gen, n, 1, 2.0)
    mesh = opt.Extract()
    gw, gh = orc.grid_dims(2.0, 2.0, spacing)
    grid = orc.Grid(gen, gw, gh, spacing)
    verts, edges, counts, inside, flags = grid.cells(2.0, 2.0, masks, tiles, tiles, float(np.float32(1.0) / np.float32(voxel)))
    assert np.array_equal(mesh.inside, inside)
    assert mesh.unsafeCells == flags[0] and mesh.overflowCells == flags[1]
    assert_cells_equal(mesh, n, verts, edges, counts)
    cs, mv, me, wt, loops = orc.assemble(verts, edges, counts, inside)
    assert mesh.watertight == wt and mesh.loops == loops
    assert np.array_equal(mesh.edges, me)
    assert np.array_equal(mesh.vertices.view(np.uint32), mv.view(np.uint32))
    return mesh


def test_uniform_sites(vm, orc):
    from voromesh_gb300 import synth

    gen = synth.uniform(31, 1, 3000)
    gen[::13] = -1.0
    mesh = run_case(vm, orc, gen, 0.05)
    assert mesh.watertight and mesh.loops >= 1


def test_lattice_near_degenerate(vm, orc):
    """Near-cocircular quadruples: a jittered lattice (the precision stress
    shape). Per-cell clipping cannot keep vertex triples consistent across
    cells there, so with 1e-6 jitter neither the reference's clipper nor this
    one need be watertight; run_case checks that both give the same mesh."""
    from voromesh_gb300 import synth

    run_case(vm, orc, synth.lattice(5, 5, 48, 48, 1e-6), 2.0 / 48)
    mesh = run_case(vm, orc, synth.lattice(5, 5, 48, 48, 1e-3), 2.0 / 48)
    assert mesh.watertight


def test_uncertified_cells(vm, orc):
    """Sparse sites around a dense cluster: cells the 32 nearest cannot certify
    take the security-radius gather (same cuts as the reference's loop)."""
    from voromesh_gb300 import synth

    dense = synth.uniform(6, 1, 900, -0.05, 0.05)
    sparse = synth.uniform(6, 2, 40, -1.0, 1.0)
    gen = np.ascontiguousarray(np.concatenate([dense, sparse]))
    mesh = run_case(vm, orc, gen, 0.02)
    assert mesh.unsafeCells > 0


@pytest.mark.parametrize("n,jitter", [(3000, None), (48 * 48, 1e-3), (60000, None)])
def test_boundary_assembly_bit_exact(vm, orc, n, jitter):
    """The device boundary assembly (vertex keys, first-seen numbering, edges,
    watertightness, loops) equals the oracle's restatement of
    voro_optimizer.cu:798-854 run on the same cells, bit for bit."""
    from voromesh_gb300 import OptimizerParams, VoroOptimizer, synth

    if jitter is None:
        gen = synth.uniform(41, 1, n)
        gen[::17] = -1.0
        spacing = float(2.0 / np.sqrt(n))
    else:
        gen = synth.lattice(7, 7, 48, 48, jitter)
        spacing = 2.0 / 48
    masks, tiles, voxel = disc_masks()
    opt = VoroOptimizer(2.0, 2.0, spacing, OptimizerParams(lossK=12))
    opt.SetTargets(gen[:8])
    opt.SetOccupancy(masks, tiles, tiles, voxel)
    opt.SetGenerators(gen, len(gen), 1, 2.0)
    m = opt.Extract()
    counts = np.diff(m.cellStart).astype(np.int32)
    K = 24
    verts = np.zeros((len(gen), K, 2), np.float32)
    labels = np.zeros((len(gen), K), np.int32)
    for i in range(len(gen)):
        a, b = m.cellStart[i], m.cellStart[i + 1]
        verts[i, :b - a] = m.cellVerts[a:b]
        labels[i, :b - a] = m.cellLabels[a:b]
    _, mv, me, wt, loops = orc.assemble(verts, labels, counts, m.inside)
    assert np.array_equal(m.edges, me)
    assert np.array_equal(m.vertices.view(np.uint32), mv.view(np.uint32))
    assert m.watertight == wt and m.loops == loops
    assert len(me) > 0


def lobe_masks(voxels=1024):
    """A 5-lobed occupancy on voxels x voxels voxels of [0,2]^2, in 8x8 tiles."""
    tiles = voxels // 8
    jj, ii = np.mgrid[0:voxels, 0:voxels]
    x, y = (ii + 0.5) * 2 / voxels - 1, (jj + 0.5) * 2 / voxels - 1
    occ = np.hypot(x, y) < 0.5 + 0.25 * np.cos(5 * np.arctan2(y, x))
    masks = np.zeros(tiles * tiles, np.uint64)
    jy, ix = np.nonzero(occ)
    bits = (np.uint64(1) << (((jy & 7) << 3) | (ix & 7)).astype(np.uint64))
    np.bitwise_or.at(masks, (jy >> 3) * tiles + (ix >> 3), bits)
    return masks, tiles, 2.0 / voxels


def test_extract_precision_lattice_full_size(vm, orc, capsys):
    """The precision-stress lattice at its stated size: 512x512 sites with
    1e-6 jitter (near-cocircular quadruples everywhere), a 5-lobed occupancy.
    Inside flags, the unsafe/overflow counts and every cell (labels and vertex
    bits) equal the oracle's."""
    from voromesh_gb300 import OptimizerParams, VoroOptimizer, synth

    gen = np.ascontiguousarray(synth.lattice(1, 5, 512, 512, 1e-6).reshape(-1, 2))
    n, spacing = len(gen), float(np.float32(2.0 / 512))
    masks, tiles, voxel = lobe_masks()
    opt = VoroOptimizer(2.0, 2.0, spacing, OptimizerParams(lossK=16))
    opt.SetTargets(gen[:8])
    opt.SetOccupancy(masks, tiles, tiles, voxel)
    opt.SetGenerators(gen, 512, 512, 2.0)
    mesh = opt.Extract()
    gw, gh = orc.grid_dims(2.0, 2.0, spacing)
    verts, edges, counts, inside, flags = orc.Grid(gen, gw, gh, spacing).cells(
        2.0, 2.0, masks, tiles, tiles, float(np.float32(1.0) / np.float32(voxel)), nthreads=8)
    assert np.array_equal(mesh.inside, inside) and inside.sum() > 50000
    assert mesh.unsafeCells == flags[0] and mesh.overflowCells == flags[1]
    assert_cells_equal(mesh, n, verts, edges, counts)
    with capsys.disabled():
        print(f"\nextraction, 512x512 jittered lattice: all {n} cells equal the oracle's bit for bit; "
              f"unsafe {mesh.unsafeCells}, watertight {mesh.watertight}")


def test_extract_after_slot_grid_shrinks(vm):
    """Extract on an optimiser whose slot grid shrank (6,000 slots, then
    1,000: a later cell-packing scan of fewer tiles on the same buffers)
    gives what a fresh optimiser gives."""
    from voromesh_gb300 import OptimizerParams, VoroOptimizer, synth

    masks, tiles, voxel = disc_masks()
    big, small = synth.uniform(43, 1, 6000), synth.uniform(43, 2, 1000)

    def fresh():
        o = VoroOptimizer(2.0, 2.0, 0.05, OptimizerParams(lossK=12))
        o.SetTargets(small[:8])
        o.SetOccupancy(masks, tiles, tiles, voxel)
        return o

    reused = fresh()
    reused.SetGenerators(big, len(big), 1, 2.0)
    reused.Extract()
    reused.SetGenerators(small, len(small), 1, 2.0)
    a = reused.Extract()
    other = fresh()
    other.SetGenerators(small, len(small), 1, 2.0)
    b = other.Extract()
    assert np.array_equal(a.cellStart, b.cellStart)
    assert np.array_equal(a.cellLabels, b.cellLabels)
    assert np.array_equal(a.cellVerts.view(np.uint32), b.cellVerts.view(np.uint32))
    assert np.array_equal(a.edges, b.edges) and a.watertight == b.watertight
