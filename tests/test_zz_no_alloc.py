"""The allocation-free hash-grid build (vm_build_grid_noalloc).

Callers that cannot let the library allocate device memory -- a per-frame
edit loop where cudaMalloc would stall the frame, or a host that plans all
device memory itself -- build the grid into buffers they own, with the
library's scratch held in a fixed device array. This checks, through the C
ABI, that its output equals the grid the optimiser builds with its own
allocations (bit for bit: cell starts, slot order and positions are integer
or copied data), on two calls in a row with different sizes, so the second
call must not see the first one's leftovers in the shared scratch. The file
sorts last so a stop-at-first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_grid_matches_allocating_path(vm):
    import torch

    from voromesh_gb300 import synth
    from voromesh_gb300._lib import check, load

    lib = load()
    cases = [(21, 50000, 0.01), (22, 7000, 0.03)]  # second call: fewer points and cells
    for seed, n, spacing in cases:
        gen = synth.uniform(seed, 1, n)
        gen[::11] = -1.0  # empty slots
        tgt = synth.circle(seed, 2, 64, 0.5, 1e-2)
        opt = vm.VoroOptimizer(2.0, 2.0, spacing, vm.OptimizerParams(lossK=12))
        opt.SetTargets(tgt)
        opt.SetGenerators(gen, n, 1, 2.0)
        start, sidx, spos, _ = opt.Grid()
        info = opt.info()
        gw, gh = info.gridW, info.gridH
        opt.close()

        d_gen = torch.from_numpy(gen).cuda()
        d_start = torch.full((gw * gh + 1,), -7, dtype=torch.int32, device="cuda")
        d_sidx = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_spos = torch.full((n, 2), -7.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        check(lib.vm_build_grid_noalloc(_dev_ptr(d_gen), n, gw, gh, spacing, _dev_ptr(d_start), _dev_ptr(d_sidx),
                                        _dev_ptr(d_spos), None), "vm_build_grid_noalloc")
        torch.cuda.synchronize()
        live = int(start[-1])
        assert np.array_equal(d_start.cpu().numpy(), start)
        assert np.array_equal(d_sidx.cpu().numpy()[:live], sidx)
        assert np.array_equal(d_spos.cpu().numpy()[:live], spos)


def test_noalloc_rejects_oversize(vm):
    from voromesh_gb300._lib import load

    lib = load()
    # sizes are checked before anything touches the device
    assert lib.vm_build_grid_noalloc(C.c_void_p(8), 262145, 10, 10, 0.1, C.c_void_p(8), C.c_void_p(8),
                                     C.c_void_p(8), None) == 1
    assert lib.vm_build_grid_noalloc(None, 0, 1000, 1000, 0.1, C.c_void_p(8), None, None, None) == 1


def test_noalloc_empty_and_side_stream(vm):
    """n = 0 leaves every cell start at zero (after a call that filled them),
    and a call enqueued on a side stream gives the same grid as one on the
    legacy default stream."""
    import torch

    from voromesh_gb300 import synth
    from voromesh_gb300._lib import check, load

    lib = load()
    n, gw, gh, spacing = 30000, 100, 100, 0.02
    gen = torch.from_numpy(synth.uniform(31, 1, n)).cuda()
    outs = []
    side = torch.cuda.Stream()
    for stream in (None, side):
        d_start = torch.full((gw * gh + 1,), -7, dtype=torch.int32, device="cuda")
        d_sidx = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_spos = torch.full((n, 2), -7.0, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        handle = None if stream is None else C.c_void_p(stream.cuda_stream)
        check(lib.vm_build_grid_noalloc(_dev_ptr(gen), n, gw, gh, spacing, _dev_ptr(d_start), _dev_ptr(d_sidx),
                                        _dev_ptr(d_spos), handle), "vm_build_grid_noalloc")
        torch.cuda.synchronize()
        outs.append((d_start.cpu().numpy(), d_sidx.cpu().numpy(), d_spos.cpu().numpy()))
    assert outs[0][0][-1] == n
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    d_start = torch.full((gw * gh + 1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    check(lib.vm_build_grid_noalloc(None, 0, gw, gh, spacing, _dev_ptr(d_start), None, None, None),
          "vm_build_grid_noalloc")
    torch.cuda.synchronize()
    assert not d_start.cpu().numpy().any()
