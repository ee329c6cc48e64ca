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
