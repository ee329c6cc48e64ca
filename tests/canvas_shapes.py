"""Canvas test shapes shared by the GPU parity tests and the oracle's pin to
the reference: (name, (width, height, voxel size), closed polygon)."""
import numpy as np


def shapes():
    from voromesh_gb300 import synth

    yield "heart_1k", (1024.0, 1024.0, 1.0), synth.heart(512.0, 512.0, 819.2, 4096)
    yield "heart_small_domain", (2.0, 2.0, 2.0 / 1024), synth.heart(1.0, 1.0, 1.6, 4096)
    yield "odd_grid", (100.0, 61.0, 0.37), synth.heart(50.0, 30.0, 70.0, 50)
    yield "triangle_outside", (64.0, 64.0, 1.0), np.array([[-10, -5], [80, 20], [20, 90]], np.float32)
    # many vertices inside one voxel: dozens of samples per voxel
    t = np.linspace(0, 2 * np.pi, 400, endpoint=False)
    yield "tiny_ring", (16.0, 16.0, 1.0), np.stack([8.3 + 0.4 * np.cos(t), 8.6 + 0.4 * np.sin(t)], 1).astype(np.float32)
    # 600 crossings on one scanline: the block-per-row path
    yield "comb", (1000.0, 1000.0, 1.0), synth.comb(10.0, 10.0, 900.0, 500.0, 300)
    # samples with coordinates of very different magnitude in one voxel: the
    # sample-order fallback of the per-voxel sums
    yield "tiny_coords", (8.0, 8.0, 1.0), np.array([[1e-30, 0.25], [0.75, 1e-25], [0.9, 0.9], [3.0, 7.0]], np.float32)
    yield "single_vertex", (8.0, 8.0, 1.0), np.array([[3.5, 4.25]], np.float32)
    # vertices on voxel centres and boundaries, a horizontal edge, a repeated vertex
    yield "grid_aligned", (32.0, 32.0, 1.0), np.array(
        [[4.5, 4.5], [20, 4.5], [20, 4.5], [20, 10], [27.5, 10], [27.5, 27.5], [4, 27.5], [4, 16], [10.5, 16],
         [10.5, 12], [4.5, 12]], np.float32)
    # self-intersecting (even-odd fill) and clockwise outlines, a near-degenerate sliver
    t = np.arange(5) * 4 * np.pi / 5 - np.pi / 2
    yield "pentagram", (64.0, 64.0, 1.0), np.stack([32 + 25 * np.cos(t), 32 + 25 * np.sin(t)], 1).astype(np.float32)
    yield "clockwise_square", (16.0, 16.0, 0.5), np.array([[2, 2], [2, 12], [12, 12], [12, 2]], np.float32)
    yield "sliver", (16.0, 16.0, 1.0), np.array([[1, 8], [15, 8.0001], [15, 8.0002], [1, 8.0003]], np.float32)
    yield "random_poly", (50.0, 40.0, 0.7), np.random.default_rng(3).uniform(-5, 55, (40, 2)).astype(np.float32)
    # one tile: a vertex at 1.5 * 2^-20 and 7,279 copies of (288, 288), so the
    # voxel of (288, 288) holds ~7,284 samples each 2^28 times the tile's
    # smallest: their integer magnitude sum needs 65 bits and, taken modulo
    # 2^64, would pass the exact-sum certificate; the ordered double sum must
    # decide
    tiny = np.float32(1.5 * 2.0 ** -20)
    yield "wrap_voxel", (512.0, 512.0, 64.0), np.array([[tiny, tiny]] + [[288.0, 288.0]] * 7279, np.float32)
    # 64 samples in voxel 0, one per vertex (every edge is shorter than the
    # quarter-voxel step): 16 of 2^-50 and 48 summing to 64 + 2^-18, so the
    # mean sits on a float rounding tie, 1 + 2^-24. Summed first, the small
    # ones add 2^-52 to the mean, which rounds up to 1 + 2^-23; summed after
    # the large ones, they vanish and the tie rounds to 1. The mean depends on
    # the sample order, which the long-run fallback must restore.
    lo = [[2.0 ** -50, 2.0 ** -50]] * 16
    hi = [[1.0, 1.0]] * 46 + [[9.0, 9.0], [9.0 + 2.0 ** -18, 9.0 + 2.0 ** -18]]
    yield "order_small_first", (512.0, 512.0, 64.0), np.array(lo + hi, np.float32)
    yield "order_small_last", (512.0, 512.0, 64.0), np.array(hi + lo, np.float32)


def shape(name):
    return next((dims, poly) for n, dims, poly in shapes() if n == name)


# static, so that collecting the tests imports nothing of the package
NAMES = ["heart_1k", "heart_small_domain", "odd_grid", "triangle_outside", "tiny_ring", "comb", "tiny_coords",
         "single_vertex", "grid_aligned", "pentagram", "clockwise_square", "sliver", "random_poly", "wrap_voxel",
         "order_small_first", "order_small_last"]
