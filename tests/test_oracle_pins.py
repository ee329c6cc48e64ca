"""The oracle against the reference's own kernels.

tests/golden/reference_kernels.npz was produced by tests/golden/make_golden.py
from the reference's kernel code compiled for the CPU (oracle/ref_shim); where
that build is present (oracle/_ref), the tie-heavy lattice shape is also
checked against it live. The oracle's reference mode (float sums in target
order, powf) must reproduce every array bit for bit; its fixed-point mode (the
product's arithmetic) must stay within the stated tolerances.
"""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden" / "reference_kernels.npz"


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def plain():
    from voromesh_gb300 import synth

    return synth.plain_fit()


def test_inputs_regenerate(plain, gold):
    # the fixtures' inputs come from the seeded generators; their grid pins them
    from oracle import oracle as orc

    st, si, sp, gc = orc.build_grid(plain.generators, 40, 40, 0.05)
    assert np.array_equal(st, gold["plain_grid_start"])
    assert np.array_equal(si, gold["plain_grid_idx"])
    assert np.array_equal(sp, gold["plain_grid_pos"])
    assert np.array_equal(gc, gold["plain_grid_cell"])


@pytest.mark.parametrize("K", [12, 16, 32])
def test_knn_lists(orc, plain, gold, K):
    grid = orc.Grid(plain.generators, 40, 40, 0.05)
    idx, d2 = grid.knn(plain.targets[:512], K)
    assert np.array_equal(idx, gold[f"plain_knn{K}_idx"])
    assert np.array_equal(d2, gold[f"plain_knn{K}_d2"])


def test_knn_matches_brute_force(orc, plain):
    import ctypes as C

    grid = orc.Grid(plain.generators, 40, 40, 0.05)
    q = plain.targets[:200]
    idx, d2 = grid.knn(q, 16)
    L = orc.lib()
    g = np.ascontiguousarray(plain.generators)
    for i in range(len(q)):
        bi = np.empty(16, np.int32)
        bd = np.empty(16, np.float32)
        L.vo_knn_brute(orc.P(g), len(g), orc.VoF2(q[i, 0], q[i, 1]), 16, C.c_void_p(bi.ctypes.data),
                       C.c_void_p(bd.ctypes.data))
        assert np.array_equal(bi, idx[i]) and np.array_equal(bd, d2[i])


def _ref_fit(orc, plain, fraction, acc, pw, K=12):
    f = orc.Fit(2.0, 2.0, 0.05, K, plain.lrPerSpacing, fraction, 300, acc=acc, pow_mode=pw)
    f.set_targets(plain.targets)
    f.set_generators(plain.generators, 2048, 1, 2.0)
    return f


def test_first_gradient(orc, plain, gold):
    f = _ref_fit(orc, plain, 1.0, orc.ACC_REF, orc.POW_REF)
    g, cnt, loss = f.gradient()
    assert cnt == int(gold["plain_step1_count"][0])
    assert np.float32(loss) == gold["plain_step1_loss"][0]
    assert np.array_equal(g, gold["plain_step1_grad"])


@pytest.mark.parametrize("fraction", [1.0, 0.2])
def test_forty_steps(orc, plain, gold, fraction):
    key = f"plain_f{int(fraction * 100)}"
    f = _ref_fit(orc, plain, fraction, orc.ACC_REF, orc.POW_REF)
    losses = [f.step(1) for _ in range(40)]
    g, m, v = f.generators()
    assert np.array_equal(np.float32(losses), gold[f"{key}_losses"])
    assert np.array_equal(g, gold[f"{key}_gen"])
    assert np.array_equal(m, gold[f"{key}_m"]) and np.array_equal(v, gold[f"{key}_v"])


def test_k16_gradient(orc, gold):
    from voromesh_gb300 import synth

    f = orc.Fit(2.0, 2.0, 0.06, 16, 0.09, 1.0, 300, acc=orc.ACC_REF, pow_mode=orc.POW_REF)
    f.set_targets(synth.circle(3, 2, 8192, 0.6, 1e-3))
    f.set_generators(synth.uniform(3, 1, 1024), 1024, 1, 2.0)
    g, cnt, loss = f.gradient()
    assert cnt == int(gold["k16_count"][0])
    assert np.float32(loss) == gold["k16_loss"][0]
    assert np.array_equal(g, gold["k16_grad"])


def test_fixed_point_mode_tolerance(orc, plain, gold):
    """The product's sums (exact fixed point) vs the reference's float sums:
    the first gradient within 1e-5 of the gradient's scale (max |g|) and at
    least as close to the FP64 oracle as the reference's float sum is; loss
    within 1e-5 relative; positions after 5 steps within 1e-5 of the domain
    extent. (The reference's own float-atomic order varies by more than that
    over longer horizons.)"""
    fx = _ref_fit(orc, plain, 1.0, orc.ACC_FIXED, orc.POW_DET)
    g, cnt, loss = fx.gradient()
    gref = gold["plain_step1_grad"]
    assert cnt == int(gold["plain_step1_count"][0])
    assert abs(loss - gold["plain_step1_loss"][0]) <= 1e-5 * abs(gold["plain_step1_loss"][0])
    assert np.abs(g - gref).max() <= 1e-5 * np.abs(gref).max()
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.05)), 12, plain.lrPerSpacing, 1.0, 300)
    d.set_targets(plain.targets)
    d.set_generators(plain.generators, 2048, 1, 2.0)
    g64, _, _ = d.gradient()
    assert np.abs(g - g64).max() <= np.abs(gref - g64).max()
    rf = _ref_fit(orc, plain, 1.0, orc.ACC_REF, orc.POW_REF)
    fx.step(5)
    rf.step(5)
    assert np.abs(fx.generators()[0] - rf.generators()[0]).max() <= 2e-5


def test_fp64_error_bar(orc, plain):
    """FP32 arithmetic vs the FP64 oracle after 10 steps (reported, bounded)."""
    fx = _ref_fit(orc, plain, 1.0, orc.ACC_FIXED, orc.POW_DET)
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.05)), 12, plain.lrPerSpacing, 1.0, 300)
    d.set_targets(plain.targets)
    d.set_generators(plain.generators, 2048, 1, 2.0)
    fx.step(10)
    d.step(10)
    err = np.abs(fx.generators()[0].astype(np.float64) - d.generators()).max()
    assert err < 1e-3  # a few lr; bisector flips between FP32 and FP64 are discrete


@pytest.mark.parametrize("shape", ["plain", "lattice_jitter", "lattice_exact"])
def test_decisions_equal_fp64(orc, plain, shape):
    """At the same generator positions, every target's nearest site and
    bisector neighbour in FP32 (the product's, which equals this oracle bit
    for bit) are those of the FP64 oracle: no decision flips, along the FP32
    trajectory. Later FP32/FP64 position differences come from the
    trajectories parting, not from the decisions' arithmetic."""
    from voromesh_gb300 import synth

    if shape == "plain":
        gen, sw, sh, tgt, spacing, K = plain.generators, 2048, 1, plain.targets, 0.05, 12
    else:
        gen = synth.lattice(3, 5, 128, 128, 1e-6 if shape == "lattice_jitter" else 0.0)
        sw, sh, tgt, spacing, K = 128, 128, synth.five_arm_star(3, 6, 131072), 2.0 / 128, 16
    f = orc.Fit(2.0, 2.0, spacing, K, 0.09, 1.0, 300, nthreads=4)
    f.set_targets(tgt)
    f.set_generators(gen, sw, sh, 2.0)
    for steps in (0, 10):
        f.step(steps)
        d = orc.Fit64(2.0, 2.0, float(np.float32(spacing)), K, 0.09, 1.0, 300, nthreads=4)
        d.set_targets(tgt)
        d.set_generators(f.generators()[0], sw, sh, 2.0)
        i0, j, _ = orc.loss_detail(f, tgt, K)
        i64, j64 = d.detail()
        assert (i0 >= 0).sum() > 0.99 * len(tgt)
        assert np.array_equal(i0, i64) and np.array_equal(j, j64)


def _make_golden_module():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).resolve().parent / "golden" /
                                                  "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("jitter", [1e-6, 0.0])
def test_lattice_matches_live_reference(orc, jitter):
    """The tie-heavy shape (a 128x128 lattice of sites, jittered by 1e-6 or
    exact, 131,072 targets on the 5-arm star, k=16) against the reference's own
    kernels compiled for the CPU: the grid, kNN lists, the first gradient and
    10 steps of positions and moments, with the oracle in reference mode."""
    if not orc.ref_available():
        pytest.skip("the reference kernels are not compiled here")
    from voromesh_gb300 import synth

    mg = _make_golden_module()
    ref = orc.ref()
    gen = np.ascontiguousarray(synth.lattice(3, 5, 128, 128, jitter).reshape(-1, 2))
    tgt = np.ascontiguousarray(synth.five_arm_star(3, 6, 131072))
    spacing, K, n = float(np.float32(2.0 / 128)), 16, len(gen)
    gw, gh = orc.grid_dims(2.0, 2.0, spacing)
    rst, rsi, rsp, rgc = mg.ref_grid(ref, gen, gw, gh, spacing)
    f = orc.Fit(2.0, 2.0, spacing, K, 0.09, 1.0, 300, acc=orc.ACC_REF, pow_mode=orc.POW_REF, nthreads=4)
    f.set_targets(tgt)
    f.set_generators(gen, n, 1, 2.0)
    start, sidx, spos, gcell = f.grid()
    assert np.array_equal(start, rst) and np.array_equal(sidx, rsi)
    assert np.array_equal(spos, rsp) and np.array_equal(gcell, rgc)
    q = np.ascontiguousarray(tgt[::64])
    ridx = np.zeros((len(q), K), np.int32)
    rd2 = np.zeros((len(q), K), np.float32)
    ref.ref_knn(K, mg.P(rst), mg.P(rsi), mg.P(rsp), gw, gh, C.c_float(spacing), mg.P(q), len(q), mg.P(ridx),
                mg.P(rd2))
    idx, d2 = orc.Grid(gen, gw, gh, spacing).knn(q, K)
    assert np.array_equal(idx, ridx) and np.array_equal(d2, rd2)
    rpf, rpi = mg.run_params(spacing, 0.09, n, 1, 2.0, 300, 300)
    stt = np.array([1, 0], np.int32)
    sl = np.zeros(1, np.float32)
    rgrad = np.zeros_like(gen)
    ref.ref_loss(K, mg.P(tgt), len(tgt), mg.P(rst), mg.P(rsi), mg.P(rsp), gw, gh, C.c_float(spacing), mg.P(gen),
                 mg.P(rgrad), mg.P(stt), mg.P(sl), mg.P(rpf), mg.P(rpi), C.c_float(1.0), C.c_uint(1))
    g, cnt, loss = f.gradient()
    assert cnt == int(stt[1]) and np.float32(loss) == sl[0]
    assert np.array_equal(g, rgrad)
    rg, rm, rv, _ = mg.ref_fit(ref, gen, tgt, K, spacing, 0.09, 1.0, 10)
    f.step(10)
    og, om, ov = f.generators()
    assert np.array_equal(og, rg) and np.array_equal(om, rm) and np.array_equal(ov, rv)


def _fit_case(name):
    from voromesh_gb300 import synth

    if name == "far_targets_k16":  # generators in the middle only: the exact ring-search path
        gen = synth.uniform(4, 1, 600, -0.5, 0.5)
        tgt = np.concatenate([synth.circle(4, 2, 3000, 0.9, 0.05), synth.uniform(4, 3, 500, -1.2, 1.2)])
        return gen, tgt, 0.05, 16, 1.0
    if name == "subsampled_k16":
        return synth.uniform(3, 1, 1024), synth.circle(3, 2, 8192, 0.6, 1e-3), 0.06, 16, 0.2
    if name == "lattice_k12":
        return (synth.lattice(3, 5, 64, 64, 1e-6).reshape(-1, 2), synth.five_arm_star(3, 6, 40000), 2.0 / 64, 12,
                1.0)
    raise KeyError(name)


@pytest.mark.parametrize("name", ["far_targets_k16", "subsampled_k16", "lattice_k12"])
def test_fits_match_live_reference(orc, name):
    """Fits the GPU parity tests use beyond the plain one: targets far from
    every generator, a 0.2 sample fraction, and k = 12 on a jittered lattice.
    Ten steps of the reference's kernels compiled for the CPU (losses,
    positions, moments) against the oracle in reference mode."""
    if not orc.ref_available():
        pytest.skip("the reference kernels are not compiled here")
    mg = _make_golden_module()
    gen, tgt, spacing, K, frac = _fit_case(name)
    gen, tgt = np.ascontiguousarray(gen, np.float32), np.ascontiguousarray(tgt, np.float32)
    spacing = float(np.float32(spacing))
    rg, rm, rv, rloss = mg.ref_fit(orc.ref(), gen, tgt, K, spacing, 0.09, frac, 10)
    f = orc.Fit(2.0, 2.0, spacing, K, 0.09, frac, 300, acc=orc.ACC_REF, pow_mode=orc.POW_REF, nthreads=4)
    f.set_targets(tgt)
    f.set_generators(gen, len(gen), 1, 2.0)
    losses = [f.step(1) for _ in range(10)]
    og, om, ov = f.generators()
    assert np.array_equal(np.float32(losses), rloss)
    assert np.array_equal(og, rg) and np.array_equal(om, rm) and np.array_equal(ov, rv)


@pytest.mark.parametrize("jitter", [1e-6, 0.0])
def test_lattice_cells_match_live_reference(orc, jitter):
    """The clipper on the tie-heavy lattice (64x64 sites, jittered by 1e-6 or
    exact: cocircular sites everywhere), with a 5-lobed occupancy, against the
    reference's voronoiCellKernel compiled for the CPU: counts, inside flags,
    edge labels and vertices bit for bit."""
    if not orc.ref_available():
        pytest.skip("the reference kernels are not compiled here")
    from voromesh_gb300 import synth

    mg = _make_golden_module()
    ref = orc.ref()
    gen = np.ascontiguousarray(synth.lattice(3, 5, 64, 64, jitter).reshape(-1, 2))
    n, spacing = len(gen), float(np.float32(2.0 / 64))
    gw, gh = orc.grid_dims(2.0, 2.0, spacing)
    st, si, sp, _ = mg.ref_grid(ref, gen, gw, gh, spacing)
    tiles = 16  # 128x128 voxels of size 2/128 in 8x8-voxel tiles
    masks = np.zeros(tiles * tiles, np.uint64)
    jj, ii = np.mgrid[0:128, 0:128]
    x, y = (ii + 0.5) * 2 / 128 - 1, (jj + 0.5) * 2 / 128 - 1
    occ = np.hypot(x, y) < 0.5 + 0.25 * np.cos(5 * np.arctan2(y, x))
    for j, i in zip(*np.nonzero(occ)):
        masks[(j >> 3) * tiles + (i >> 3)] |= np.uint64(1) << np.uint64(((j & 7) << 3) | (i & 7))
    verts = np.zeros((n * 24, 2), np.float32)
    edges = np.zeros(n * 24, np.int32)
    counts = np.zeros(n, np.int32)
    inside = np.zeros(n, np.uint8)
    flags = np.zeros(2, np.int32)
    ref.ref_cells(mg.P(st), mg.P(si), mg.P(sp), gw, gh, C.c_float(spacing), mg.P(gen), n, C.c_float(2.0),
                  C.c_float(2.0), mg.P(masks), tiles, tiles, C.c_float(64.0), mg.P(verts), mg.P(edges), mg.P(counts),
                  mg.P(inside), mg.P(flags))
    ov, oe, oc, oi, of = orc.Grid(gen, gw, gh, spacing).cells(2.0, 2.0, masks, tiles, tiles, 64.0)
    assert np.array_equal(oc, counts) and np.array_equal(oi, inside) and np.array_equal(of, flags)
    assert inside.sum() > 500
    verts, edges = verts.reshape(n, 24, 2), edges.reshape(n, 24)
    for i in range(n):
        c = counts[i]
        assert np.array_equal(oe[i, :c], edges[i, :c]) and np.array_equal(ov[i, :c], verts[i, :c])


def test_cells(orc, gold):
    from voromesh_gb300 import synth

    gen = synth.uniform(8, 1, 300)
    gen[::17] = -1.0
    grid = orc.Grid(gen, 17, 17, 0.12)
    verts, edges, counts, inside, flags = grid.cells(2.0, 2.0, gold["cells_masks"], 4, 4, 16.0)
    assert np.array_equal(counts, gold["cells_counts"])
    assert np.array_equal(inside, gold["cells_inside"])
    assert np.array_equal(flags, gold["cells_flags"])
    for i in range(len(gen)):
        c = counts[i]
        assert np.array_equal(edges[i, :c], gold["cells_edges"][i, :c])
        assert np.array_equal(verts[i, :c], gold["cells_verts"][i, :c])


def test_poisson(orc, gold):
    grid, p = orc.poisson_fill(1.0, 1.0, 0.02, 30, 1)
    assert np.array_equal(grid, gold["poisson_fill"])
    assert orc.poisson_verify(p, grid, 0, 0, p.gridW, p.gridH)
    grid, p = orc.poisson_fill(1.0, 1.0, 0.02, 30, 1, [(5, 5, 17, 13), (0, 0, 3, 40), (30, 30, 80, 80)])
    assert np.array_equal(grid, gold["poisson_regions"])


@pytest.mark.parametrize("case", [
    (2.0, 1.0, 0.013, 30, 5, [(10, 10, 200, 100), (50, 50, 60, 58), (0, 0, 218, 109), (-5, 30, 120, 200),
                              (57, 3, 190, 71)]),
    (1.0, 1.0, 0.02, 260, 2, []),
    (1.0, 1.0, 0.3, 30, 1, [(0, 0, 2, 2)]),
    (3.0, 2.0, 0.004, 30, 11, [(37, 53, 900, 650)]),
    (0.5, 0.8, 0.01, 30, 10, [(3, 2, 30, 20)]),
])
def test_poisson_matches_live_reference(orc, case):
    """The sampler cases the GPU tests use (non-square domains, a 4-cell grid,
    260 rounds per call, regions off the colour grid and past the edges),
    against the reference's dartPhaseKernel sequence compiled for the CPU:
    the whole grid bit for bit after the fill and after every region."""
    if not orc.ref_available():
        pytest.skip("the reference kernels are not compiled here")
    w, h, r, trials, seed, regions = case
    ref = orc.ref()
    cs = C.c_float()
    gw, gh = C.c_int(), C.c_int()
    ref.ref_poisson_dims(C.c_float(w), C.c_float(h), C.c_float(r), C.byref(cs), C.byref(gw), C.byref(gh))
    grid = np.full((gw.value * gh.value, 2), -1.0, np.float32)
    base = 0
    for k, (x0, y0, x1, y1) in enumerate([(0, 0, gw.value, gh.value)] + list(regions)):
        x0, y0, x1, y1 = max(x0, 0), max(y0, 0), min(x1, gw.value), min(y1, gh.value)
        if x0 < x1 and y0 < y1:
            ref.ref_poisson_resample(orc.P(grid), C.c_float(w), C.c_float(h), C.c_float(r), cs, gw, gh,
                                     C.c_uint(seed), x0, y0, x1, y1, trials, C.c_uint(base))
        base += trials
        cells, p = orc.poisson_fill(w, h, r, trials, seed, regions[:k])
        assert (p.gridW, p.gridH) == (gw.value, gh.value)
        assert np.array_equal(cells, grid), f"after call {k}"


def _f32_round(num: int, e: int) -> np.float32:
    """num * 2^-e rounded to the nearest float32 (ties to even), from exact integers."""
    if num == 0:
        return np.float32(0.0)
    sign = -1 if num < 0 else 1
    a = abs(num)
    shift = a.bit_length() - 24
    if shift > 0:
        q, r = divmod(a, 1 << shift)
        half = 1 << (shift - 1)
        if r > half or (r == half and q & 1):
            q += 1
        a, e = q, e - shift
    return np.float32(sign * np.ldexp(float(a), -e))


def test_split_sum_rounding(orc):
    """vo_fixed2_to_float: S = H * 2^32 + L rounded once to float, on both
    sides of the int64 range, with ties and sticky bits below the rounding
    position."""
    rng = np.random.default_rng(5)
    L = orc.lib()
    cases = [(0, 0), (-1, 0xFFFFFFFF), ((1 << 31) - 1, 0xFFFFFFFF), (1 << 31, 0), (-(1 << 31) - 1, 0),
             (1 << 40, (1 << 62) + 12345), (-(1 << 50), 1), ((1 << 62) - 7, (1 << 63) - 1), (-(1 << 62), 0)]
    for _ in range(2000):
        h = int(rng.integers(-(1 << 62), 1 << 62)) >> int(rng.integers(0, 62))
        lo = int(rng.integers(0, 1 << 63)) >> int(rng.integers(0, 63))
        cases.append((h, lo))
    # exact ties: S = (2^24 + 1) * 2^k + 2^(k-1) rounds to even
    for k in (40, 50, 60, 69):
        s = ((1 << 24) + 1) * (1 << k) + (1 << (k - 1))
        cases.append((s >> 32, s & 0xFFFFFFFF))
    for h, lo in cases:
        for e in (0, 47, 52):
            got = np.float32(L.vo_fixed2_to_float(h, lo, e))
            want = _f32_round(h * (1 << 32) + lo, e)
            assert got == want, (h, lo, e, got, want)


def test_gradient_sums_past_int64_oracle(orc):
    """Three sites pulled one way by 2^20 targets: the fixed-point gradient
    passes 2^63 in magnitude and still equals FP64 within 1e-6 (the
    reference's float sums: about 1e-3)."""
    from voromesh_gb300 import synth

    gen = np.array([[0.2, 1.0], [1.0, 1.0], [1.0, 0.2]], np.float32)
    tgt = (synth.uniform(23, 2, 1 << 20, -0.02, 0.02, shift=False) + np.float32([1.9, 1.0])).astype(np.float32)
    f = orc.Fit(2.0, 2.0, 0.1, 12, 0.09, 1.0, 300, nthreads=8)
    f.set_targets(tgt)
    f.set_generators(gen, 3, 1, 2.0)
    g, cnt, _ = f.gradient()
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.1)), 12, 0.09, 1.0, 300, nthreads=8)
    d.set_targets(tgt)
    d.set_generators(gen, 3, 1, 2.0)
    g64, c64, _ = d.gradient()
    assert cnt == c64 == len(tgt)
    assert np.log2(np.abs(g64).max()) + orc.lib().vo_fixed_grad_exp(np.float32(0.1)) > 63.5
    assert np.abs(g - g64).max() <= 1e-6 * np.abs(g64).max()


def _edit_case():
    import sys

    sys.path.insert(0, str(Path(__file__).resolve().parent))
    from edit_case import edit_case, run_oracle

    return edit_case(), run_oracle


def test_local_edit_schedule(orc, gold):
    """The editor's local edit (global schedule, UpdateTargets,
    UpdateGenerators and BeginSchedule over a slot rectangle, Optimize) on the
    oracle in reference mode against the reference kernels' fixture: every
    loss, position and moment after each phase."""
    case, run_oracle = _edit_case()
    (g1, m1, v1, l1), (g2, m2, v2, l2), _ = run_oracle(orc, case, orc.ACC_REF, orc.POW_REF)
    assert np.array_equal(l1, gold["edit_global_losses"]) and np.array_equal(l2, gold["edit_local_losses"])
    assert np.array_equal(g1, gold["edit_global_gen"]) and np.array_equal(g2, gold["edit_local_gen"])
    assert np.array_equal(m1, gold["edit_global_m"]) and np.array_equal(v1, gold["edit_global_v"])
    assert np.array_equal(m2, gold["edit_local_m"]) and np.array_equal(v2, gold["edit_local_v"])
    # slots outside the rectangle are frozen through the local schedule
    cx0, cy0, cx1, cy1 = case.rect
    frozen = np.ones((case.slots, case.slots), bool)
    frozen[cy0:cy1, cx0:cx1] = False
    frozen = frozen.reshape(-1)
    assert np.array_equal(g2[frozen], g1[frozen]) and not np.array_equal(g2[~frozen], g1[~frozen])


def test_local_edit_matches_live_reference(orc):
    """The same sequence against the reference kernels run live here."""
    if not orc.ref_available():
        pytest.skip("the reference kernels are not compiled here")
    mg = _make_golden_module()
    case, run_oracle = _edit_case()
    (rg1, rm1, rv1, rl1), (rg2, rm2, rv2, rl2) = mg.ref_local_edit(orc.ref(), case)
    (g1, m1, v1, l1), (g2, m2, v2, l2), _ = run_oracle(orc, case, orc.ACC_REF, orc.POW_REF)
    assert np.array_equal(l1, rl1) and np.array_equal(l2, rl2)
    assert np.array_equal(g1, rg1) and np.array_equal(m1, rm1) and np.array_equal(v1, rv1)
    assert np.array_equal(g2, rg2) and np.array_equal(m2, rm2) and np.array_equal(v2, rv2)


def test_fast_path_sums_past_int64_oracle(orc):
    """Two nearly coincident sites and 2^18 targets beside them: per-site
    fixed-point sums pass 2^63 and the oracle's gradient still equals FP64
    within 1e-6."""
    from voromesh_gb300 import synth

    gen = np.array([[1.0, 1.0], [1.0005, 1.0], [0.3, 0.3], [1.7, 1.7]], np.float32)
    tgt = (synth.uniform(24, 2, 1 << 18, -0.003, 0.003, shift=False) + np.float32([1.018, 1.018])).astype(np.float32)
    f = orc.Fit(2.0, 2.0, 0.05, 12, 0.09, 1.0, 300, nthreads=8)
    f.set_targets(tgt)
    f.set_generators(gen, 4, 1, 2.0)
    g, cnt, _ = f.gradient()
    d = orc.Fit64(2.0, 2.0, float(np.float32(0.05)), 12, 0.09, 1.0, 300, nthreads=8)
    d.set_targets(tgt)
    d.set_generators(gen, 4, 1, 2.0)
    g64, c64, _ = d.gradient()
    assert cnt == c64 == len(tgt)
    assert np.log2(np.abs(g64).max()) + orc.lib().vo_fixed_grad_exp(np.float32(0.05)) > 63.2
    assert np.abs(g - g64).max() <= 1e-6 * np.abs(g64).max()
