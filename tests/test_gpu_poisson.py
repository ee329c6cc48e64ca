"""GPU Poisson sampler parity: the sample set equals the oracle's bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h,r", [(1.0, 1.0, 0.02), (2.0, 1.0, 0.013), (1.0, 1.0, 0.3)])
def test_fill_bit_exact(vm, orc, w, h, r):
    s = vm.Sampler(w, h, r, 30, 1)
    cells, _ = orc.poisson_fill(w, h, r, 30, 1)
    assert np.array_equal(s.Cells(), cells)
    assert s.VerifyAll()


def test_region_resample(vm, orc):
    s = vm.Sampler(1.0, 1.0, 0.02, 30, 3)
    regions = [(5, 5, 17, 13), (0, 0, 3, 40), (30, 30, 80, 80)]
    for reg in regions:
        s.Resample(*reg)
        assert s.Verify(*reg)
    cells, _ = orc.poisson_fill(1.0, 1.0, 0.02, 30, 3, regions)
    assert np.array_equal(s.Cells(), cells)


def test_region_resample_both_paths(vm, orc):
    """Large regions run one launch per phase, small ones one block-wide
    launch; interleaved, the sample set still equals the oracle's."""
    s = vm.Sampler(2.0, 1.0, 0.013, 30, 5)
    regions = [(10, 10, 200, 100), (50, 50, 60, 58), (0, 0, 218, 109), (100, 20, 130, 45)]
    for reg in regions:
        s.Resample(*reg)
        assert s.Verify(*reg)
    cells, _ = orc.poisson_fill(2.0, 1.0, 0.013, 30, 5, regions)
    assert np.array_equal(s.Cells(), cells)


def test_resample_many_equals_one_by_one(vm, orc):
    """Many samplers' regions in one call (small regions as one block each of
    a single launch, large ones on their own) give each sampler the samples of
    its own Resample call."""
    shapes = [(1.0, 1.0, 0.02, 30, 7), (2.0, 1.0, 0.013, 30, 8), (1.0, 1.0, 0.05, 20, 9), (0.5, 0.8, 0.01, 30, 10)]
    regions = [(5, 5, 17, 13), (10, 10, 200, 100), (0, 0, 40, 40), (3, 2, 30, 20)]
    many = [vm.Sampler(*sh) for sh in shapes]
    vm.resample_many(many, regions)
    for s, sh, reg in zip(many, shapes, regions):
        cells, _ = orc.poisson_fill(sh[0], sh[1], sh[2], sh[3], sh[4], [reg])
        assert np.array_equal(s.Cells(), cells)
        assert s.Verify(*reg)
        s.close()
    with pytest.raises(vm.VmError):
        s = vm.Sampler(1.0, 1.0, 0.02)
        vm.resample_many([s, s], [(0, 0, 4, 4), (4, 4, 8, 8)])


def test_tiled_rounds_many_tiles(vm, orc):
    """A region resample over half a million cells whose origin is off the colour grid,
    then the whole-grid check."""
    s = vm.Sampler(3.0, 2.0, 0.004, 30, 11)
    region = (37, 53, 900, 650)
    s.Resample(*region)
    assert s.Verify(*region)
    cells, _ = orc.poisson_fill(3.0, 2.0, 0.004, 30, 11, [region])
    assert np.array_equal(s.Cells(), cells)
    assert s.VerifyAll()


@pytest.mark.parametrize("pdl", ["1", "0"])
def test_regions_with_outside_neighbours_and_many_rounds(vm, orc, monkeypatch, pdl):
    """Large regions whose conflict neighbourhoods reach outside them (samples
    kept from earlier calls), a whole-grid region among them, and a sampler
    with 260 rounds per call: the oracle's samples, with the phases launched
    as programmatic dependents of each other or (VM_PD_PDL=0) plainly."""
    monkeypatch.setenv("VM_PD_PDL", pdl)
    s = vm.Sampler(2.0, 1.0, 0.013, 30, 5)
    regions = [(10, 10, 200, 100), (0, 0, 218, 109), (-5, 30, 120, 200), (57, 3, 190, 71)]
    for reg in regions:
        s.Resample(*reg)
        assert s.Verify(*reg)
    cells, _ = orc.poisson_fill(2.0, 1.0, 0.013, 30, 5, regions)
    assert np.array_equal(s.Cells(), cells)
    s = vm.Sampler(1.0, 1.0, 0.02, 260, 2)
    cells, _ = orc.poisson_fill(1.0, 1.0, 0.02, 260, 2)
    assert np.array_equal(s.Cells(), cells)
