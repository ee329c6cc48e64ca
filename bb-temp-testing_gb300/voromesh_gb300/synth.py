"""Seeded synthetic workloads (generated by portable C code, libvm_synth.so,
so the same seed gives the same bytes on every host).

Shapes are defined on [-1,1]^2 and shifted by +1 into the optimiser's
[0,2]^2 domain. Nothing here is a public dataset: every workload is a
synthetic point set of the stated shape and size.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from ._lib import load_synth as load, ptr

U64 = C.c_uint64


def uniform(seed: int, stream: int, n: int, lo: float = -1.0, hi: float = 1.0, shift: bool = True) -> np.ndarray:
    out = np.empty((n, 2), np.float32)
    load().vm_synth_uniform(U64(seed), U64(stream), n, lo, hi, int(shift), ptr(out))
    return out


def circle(seed: int, stream: int, n: int, radius: float, sigma: float, shift: bool = True) -> np.ndarray:
    out = np.empty((n, 2), np.float32)
    load().vm_synth_circle(U64(seed), U64(stream), n, radius, sigma, int(shift), ptr(out))
    return out


def lattice(seed: int, stream: int, nx: int, ny: int, jitter: float, shift: bool = True) -> np.ndarray:
    out = np.empty((nx * ny, 2), np.float32)
    load().vm_synth_lattice(U64(seed), U64(stream), nx, ny, jitter, int(shift), ptr(out))
    return out


def ellipse_union(seed: int, stream: int, n: int, count: int = 64, shift: bool = True) -> np.ndarray:
    out = np.empty((n, 2), np.float32)
    made = load().vm_synth_ellipse_union(U64(seed), U64(stream), count, n, int(shift), ptr(out))
    return out[:made]


def star(seed: int, stream: int, n: int, arms: int, radii, rot: float = 0.0, shift: bool = True) -> np.ndarray:
    r = np.ascontiguousarray(radii, dtype=np.float64)
    if len(r) != 2 * arms:
        raise ValueError("radii must hold 2 * arms values")
    out = np.empty((n, 2), np.float32)
    load().vm_synth_star(U64(seed), U64(stream), arms, ptr(r), rot, 0.0, 0.0, n, int(shift), ptr(out))
    return out


def random_star(seed: int, stream: int, n: int, shift: bool = True) -> np.ndarray:
    arms = C.c_int()
    radii = np.zeros(80, np.float64)
    rot = C.c_double()
    load().vm_synth_star_params(U64(seed), U64(stream), C.byref(arms), ptr(radii), C.byref(rot))
    return star(seed, stream + 7919, n, arms.value, radii[: 2 * arms.value], rot.value, shift)


def five_arm_star(seed: int, stream: int, n: int, outer: float = 0.8, inner: float = 0.32) -> np.ndarray:
    radii = [outer if k % 2 == 0 else inner for k in range(10)]
    return star(seed, stream, n, 5, radii, -math.pi / 2)


def subset(seed: int, stream: int, n: int, k: int) -> np.ndarray:
    out = np.empty(k, np.int64)
    rc = load().vm_synth_subset(U64(seed), U64(stream), n, k, ptr(out))
    if rc != 0:
        raise ValueError("subset: k > n")
    return out


def uniform01(seed: int, stream: int, n: int) -> np.ndarray:
    out = np.empty(n, np.float64)
    load().vm_synth_uniform01(U64(seed), U64(stream), n, ptr(out))
    return out


def log_uniform_ints(seed: int, stream: int, n: int, lo: int, hi: int) -> np.ndarray:
    """n integers log-uniform in [lo, hi] (exp/log evaluated portably)."""
    lib = load()
    u = uniform01(seed, stream, n)
    a, b = lib.vm_synth_log(float(lo)), lib.vm_synth_log(float(hi))
    return np.array([int(lib.vm_synth_exp(a + (b - a) * x) + 0.5) for x in u], np.int64)


@dataclass
class FitSpec:
    """One fit: domain, spacing, generators (slots), targets and schedule."""
    name: str
    width: float
    height: float
    spacing: float
    generators: np.ndarray
    slotsW: int
    slotsH: int
    slotCellSize: float
    targets: np.ndarray
    lossK: int
    lrPerSpacing: float
    steps: int
    sampleFraction: float = 1.0


def plain_fit(sample_fraction: float = 1.0, n_gen: int = 2048, n_tgt: int = 16384) -> FitSpec:
    """2,048 generators uniform in [-1,1]^2; 16,384 targets on the circle r=0.6
    with N(0, 1e-3) radial noise; k=12; grid cell 0.05; lr 1e-3; 300 steps."""
    gen = uniform(1, 1, n_gen)
    tgt = circle(1, 2, n_tgt, 0.6, 1e-3)
    lr_ps = float(np.float32(1e-3) / np.float32(0.05))
    return FitSpec("plain_2k", 2.0, 2.0, 0.05, gen, n_gen, 1, 2.0, tgt, 12, lr_ps, 300, sample_fraction)


def scale_targets(n_tgt: int = 8388608) -> np.ndarray:
    """Targets on the boundary of a union of 64 ellipses."""
    return ellipse_union(1, 4, n_tgt, 64)


def scale_fit_from_cells(cells: np.ndarray, n_gen: int = 1048576, n_tgt: int = 8388608,
                         targets: np.ndarray | None = None, steps: int = 1000) -> FitSpec:
    """1,048,576 generators: a seeded uniform subset of the occupied cells of a
    Poisson r=1e-3 fill of [0,2]^2 (compact 1024x1024 slots); 8M targets on
    the union of 64 ellipses; k=16; spacing 2/1024; lr 0.09 spacing."""
    live = np.nonzero(cells[:, 0] >= 0.0)[0]
    if len(live) < n_gen:
        raise ValueError(f"only {len(live)} samples, need {n_gen}")
    pick = live[subset(1, 3, len(live), n_gen)]
    gen = np.ascontiguousarray(cells[pick])
    side = int(round(math.sqrt(n_gen)))
    slots_w, slots_h = (side, n_gen // side) if side * side == n_gen else (n_gen, 1)
    tgt = scale_targets(n_tgt) if targets is None else targets
    return FitSpec("scale_1m", 2.0, 2.0, 2.0 / side if side * side == n_gen else 2.0 / math.sqrt(n_gen), gen,
                   slots_w, slots_h, 2.0, tgt, 16, 0.09, steps)


def precision_fit(n_side: int = 512, n_tgt: int = 2097152) -> FitSpec:
    """512x512 lattice with U(-1e-6, 1e-6) jitter; targets on a 5-arm star
    (outer 0.8, inner 0.32); k=16; spacing 2/512."""
    gen = lattice(1, 5, n_side, n_side, 1e-6)
    tgt = five_arm_star(1, 6, n_tgt)
    return FitSpec("precision_262k", 2.0, 2.0, 2.0 / n_side, gen, n_side, n_side, 2.0, tgt, 16, 0.09, 1000)


def uneven_batch(n_fits: int = 512, lo: int = 1024, hi: int = 262144, tgt_per_gen: int = 4, steps: int = 200,
                 seed: int = 1) -> list[FitSpec]:
    """Fits with generator counts log-uniform in [lo, hi], 4x targets on random
    star polygons (5-40 arms, radii U[.2,.9]), generators uniform in [-1,1]^2,
    spacing 2/sqrt(S), k=16."""
    sizes = log_uniform_ints(seed, 11, n_fits, lo, hi)
    fits = []
    for f, s in enumerate(sizes):
        s = int(s)
        gen = uniform(seed, 100000 + 2 * f, s)
        tgt = random_star(seed, 100001 + 2 * f, tgt_per_gen * s)
        fits.append(FitSpec(f"batch_{f}", 2.0, 2.0, 2.0 / math.sqrt(s), gen, s, 1, 2.0, tgt, 16, 0.09, steps))
    return fits


def served_request(seed: int, index: int, lo: int = 1024, hi: int = 1048576, tgt_per_gen: int = 8,
                   steps: int = 500) -> FitSpec:
    """One request of the served stream: S log-uniform in [lo, hi], 8S targets
    from the ellipse-union or the star generator (coin flip)."""
    s = int(log_uniform_ints(seed, 500000 + 3 * index, 1, lo, hi)[0])
    gen = uniform(seed, 600000 + 3 * index, s)
    coin = uniform01(seed, 700000 + 3 * index, 1)[0]
    if coin < 0.5:
        tgt = ellipse_union(seed, 800000 + 3 * index, tgt_per_gen * s, 64)
    else:
        tgt = random_star(seed, 900000 + 3 * index, tgt_per_gen * s)
    return FitSpec(f"req_{index}", 2.0, 2.0, 2.0 / math.sqrt(s), gen, s, 1, 2.0, tgt, 16, 0.09, steps)


def arrival_times(seed: int, n: int, rate: float) -> np.ndarray:
    """Poisson arrivals: cumulative exponential inter-arrival times (s)."""
    lib = load()
    u = uniform01(seed, 13, n)
    gaps = np.array([-lib.vm_synth_log(1.0 - x) / rate for x in u])
    return np.cumsum(gaps)


def heart(cx: float, cy: float, width: float, segments: int) -> np.ndarray:
    """Closed polygon of the parametric heart x = 16 sin^3 t, y = 13 cos t -
    5 cos 2t - 2 cos 3t - cos 4t, `width` wide, centred on (cx, cy), y down
    (the outline of the reference's editor demo, include/voromesh/shape2d.h:21).
    Evaluated in float64 and rounded to float32."""
    t = 2.0 * np.pi * np.arange(segments) / segments
    s = np.sin(t)
    x = 16.0 * s ** 3
    y = 13.0 * np.cos(t) - 5.0 * np.cos(2 * t) - 2.0 * np.cos(3 * t) - np.cos(4 * t)
    scale = width / 32.0
    return np.stack([cx + scale * x, cy - scale * (y + 2.5)], 1).astype(np.float32)


def comb(x0: float, y0: float, width: float, height: float, teeth: int) -> np.ndarray:
    """Closed comb polygon: `teeth` vertical teeth over [x0, x0 + width],
    joined at the bottom; every scanline through the teeth crosses 2 * teeth
    edges."""
    pts = []
    w = width / (2 * teeth)
    for k in range(teeth):
        xa, xb = x0 + 2 * k * w, x0 + (2 * k + 1) * w
        pts += [(xa, y0 + height), (xa, y0), (xb, y0), (xb, y0 + height)]
    pts += [(x0 + width, y0 + height), (x0 + width, y0 + height * 1.1), (x0, y0 + height * 1.1)]
    return np.asarray(pts, np.float32)
