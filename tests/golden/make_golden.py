"""Generates tests/golden/*.npz from the reference's own kernels.

The reference's kernel code (src/voromesh/voro_optimizer.cu and
src/poisson/poisson_disk.cu) is compiled for the host CPU by
oracle/ref_shim/build_ref.sh into oracle/_ref/libref_kernels.so and driven
here with the reference host sequence (voro_optimizer.cu:652-744: BeginSchedule
RunParams; per step beginIteration, grid build, vorolossKernel, adamKernel).
Inputs come from the library's seeded generators, so the tests regenerate them
byte for byte. Needs the reference sources (run where they are present):

    REF=/path/to/reference bash oracle/ref_shim/build_ref.sh
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "bb-temp-testing_gb300"))
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402
from voromesh_gb300 import synth  # noqa: E402

f32 = np.float32


def P(a):
    return C.c_void_p(a.ctypes.data)


def ref_grid(ref, gen, gw, gh, cell):
    n = len(gen)
    st = np.zeros(gw * gh + 1, np.int32)
    si = np.zeros(n, np.int32)
    sp = np.zeros((n, 2), np.float32)
    gc = np.zeros(n, np.int32)
    ref.ref_build_grid(P(gen), n, gw, gh, C.c_float(cell), P(st), P(si), P(sp), P(gc))
    return st, si, sp, gc


def lround(x: float) -> int:
    """std::lround: nearest integer, halves away from zero."""
    return int(np.floor(x + 0.5)) if x >= 0 else -int(np.floor(-x + 0.5))


def run_params(spacing, lr_ps, slots_w, slots_h, slot_cell, iterations, param_iterations, W=2.0, H=2.0,
               gamma=0.5, ms=(80, 150, 200, 250), rect=None):
    """RunParams of BeginSchedule(iterations, rect) (voro_optimizer.cu:658-675);
    rect None = the full slot rectangle."""
    cx0, cy0, cx1, cy1 = rect or (0, 0, slots_w, slots_h)
    cx0, cy0, cx1, cy1 = max(cx0, 0), max(cy0, 0), min(cx1, slots_w), min(cy1, slots_h)
    mss = [lround(float(m) * iterations / param_iterations) for m in ms]
    margin = f32(2.0) * f32(spacing)
    sc = f32(slot_cell)
    rpf = np.array([f32(lr_ps) * f32(spacing), gamma, 0.9, 0.999, 1e-8, W, H, f32(cx0) * sc - margin,
                    f32(cy0) * sc - margin, f32(cx1) * sc + margin, f32(cy1) * sc + margin], np.float32)
    rpi = np.array(mss + [slots_w, cx0, cy0, cx1, cy1], np.int32)
    return rpf, rpi


class RefFit:
    """The reference's host sequence (voro_optimizer.cu:613-744) driven over its
    own kernels: SetGenerators, UpdateGenerators, BeginSchedule with a slot
    rectangle (moments of the rectangle zeroed, step counter reset) and Step
    (beginIteration, grid build, vorolossKernel, adamKernel)."""

    def __init__(self, ref, gen, slots_w, slots_h, slot_cell, targets, K, spacing, lr_ps, fraction,
                 param_iterations, seed=1):
        self.ref, self.K, self.spacing, self.lr_ps = ref, K, float(f32(spacing)), lr_ps
        self.fraction, self.seed, self.param_iterations = fraction, seed, param_iterations
        self.w, self.h, self.slot_cell = slots_w, slots_h, slot_cell
        self.gen = np.ascontiguousarray(gen, np.float32).copy()
        self.m = np.zeros_like(self.gen)
        self.v = np.zeros_like(self.gen)
        self.grad = np.zeros_like(self.gen)
        self.targets = np.ascontiguousarray(targets, np.float32)
        self.st = np.zeros(2, np.int32)
        self.gw, self.gh = orc.grid_dims(2.0, 2.0, self.spacing)
        self.begin_schedule(param_iterations)

    def begin_schedule(self, iterations, rect=None):
        self.rpf, self.rpi = run_params(self.spacing, self.lr_ps, self.w, self.h, self.slot_cell, iterations,
                                        self.param_iterations, rect=rect)
        cx0, cy0, cx1, cy1 = (int(v) for v in self.rpi[5:9])
        if cx0 < cx1 and cy0 < cy1:
            for a in (self.m, self.v):
                a.reshape(self.h, self.w, 2)[cy0:cy1, cx0:cx1] = 0.0
        self.st[:] = 0
        self.length, self.iteration = iterations, 0

    def update_generators(self, slots, rect):
        cx0, cy0, cx1, cy1 = max(rect[0], 0), max(rect[1], 0), min(rect[2], self.w), min(rect[3], self.h)
        if cx0 < cx1 and cy0 < cy1:
            s = np.ascontiguousarray(slots, np.float32).reshape(self.h, self.w, 2)
            self.gen.reshape(self.h, self.w, 2)[cy0:cy1, cx0:cx1] = s[cy0:cy1, cx0:cx1]

    def step(self, k):
        losses = []
        n = len(self.gen)
        sl = np.zeros(1, np.float32)
        for _ in range(k):
            self.st[0] += 1
            self.st[1] = 0
            sl[0] = 0
            g = ref_grid(self.ref, self.gen, self.gw, self.gh, self.spacing)
            self.ref.ref_loss(self.K, P(self.targets), len(self.targets), P(g[0]), P(g[1]), P(g[2]), self.gw,
                              self.gh, C.c_float(self.spacing), P(self.gen), P(self.grad), P(self.st), P(sl),
                              P(self.rpf), P(self.rpi), C.c_float(self.fraction), C.c_uint(self.seed))
            losses.append(sl[0] / self.st[1] if self.st[1] else f32(0))
            self.ref.ref_adam(P(self.gen), P(self.m), P(self.v), P(self.grad), n, int(self.st[0]), int(self.st[1]),
                              P(self.rpf), P(self.rpi))
        self.iteration = int(self.st[0])
        return np.array(losses, np.float32)


def ref_local_edit(ref, case):
    """The local-edit case (tests/edit_case.py) through RefFit: the global
    schedule, then the edit and the local schedule. Returns the state after
    each phase."""
    f = RefFit(ref, case.generators, case.slots, case.slots, case.slot_cell, case.targets, case.K, case.spacing,
               case.lr_per_spacing, case.fraction, case.iterations)
    l1 = f.step(case.global_steps)
    mid = (f.gen.copy(), f.m.copy(), f.v.copy(), l1)
    f.targets = np.ascontiguousarray(case.targets2, np.float32)
    f.update_generators(case.slots2, case.rect)
    f.begin_schedule(case.local_iterations, case.rect)
    l2 = f.step(f.length - f.iteration)
    return mid, (f.gen.copy(), f.m.copy(), f.v.copy(), l2)


def ref_fit(ref, gen0, tg, K, spacing, lr_ps, frac, steps, seed=1, param_iterations=300):
    n = len(gen0)
    gen = gen0.copy()
    m = np.zeros_like(gen)
    v = np.zeros_like(gen)
    grad = np.zeros_like(gen)
    rpf, rpi = run_params(spacing, lr_ps, n, 1, 2.0, param_iterations, param_iterations)
    st = np.zeros(2, np.int32)
    sl = np.zeros(1, np.float32)
    gw, gh = orc.grid_dims(2.0, 2.0, spacing)
    losses = []
    for _ in range(steps):
        st[0] += 1
        st[1] = 0
        sl[0] = 0
        g = ref_grid(ref, gen, gw, gh, spacing)
        ref.ref_loss(K, P(tg), len(tg), P(g[0]), P(g[1]), P(g[2]), gw, gh, C.c_float(spacing), P(gen), P(grad), P(st),
                     P(sl), P(rpf), P(rpi), C.c_float(frac), C.c_uint(seed))
        losses.append(sl[0] / st[1] if st[1] else f32(0))
        ref.ref_adam(P(gen), P(m), P(v), P(grad), n, int(st[0]), int(st[1]), P(rpf), P(rpi))
    return gen, m, v, np.array(losses, np.float32)


def main():
    if not orc.ref_available():
        sys.exit("oracle/_ref/libref_kernels.so missing: run oracle/ref_shim/build_ref.sh first")
    ref = orc.ref()
    out = {}
    # ---- plain fit: 2,048 generators, 16,384 circle targets, k=12, cell 0.05
    spec = synth.plain_fit()
    gen, tg = spec.generators, spec.targets
    gw, gh = orc.grid_dims(2.0, 2.0, 0.05)
    st, si, sp, gc = ref_grid(ref, gen, gw, gh, 0.05)
    out.update(plain_grid_start=st, plain_grid_idx=si, plain_grid_pos=sp, plain_grid_cell=gc)
    q = np.ascontiguousarray(tg[:512])
    for K in (12, 16, 32):
        idx = np.zeros((len(q), K), np.int32)
        d2 = np.zeros((len(q), K), np.float32)
        ref.ref_knn(K, P(st), P(si), P(sp), gw, gh, C.c_float(0.05), P(q), len(q), P(idx), P(d2))
        out[f"plain_knn{K}_idx"] = idx
        out[f"plain_knn{K}_d2"] = d2
    # one loss pass with gradient (next Step semantics, iteration 1)
    rpf, rpi = run_params(0.05, spec.lrPerSpacing, 2048, 1, 2.0, 300, 300)
    stt = np.array([1, 0], np.int32)
    sl = np.zeros(1, np.float32)
    grad = np.zeros_like(gen)
    ref.ref_loss(12, P(tg), len(tg), P(st), P(si), P(sp), gw, gh, C.c_float(0.05), P(gen), P(grad), P(stt), P(sl),
                 P(rpf), P(rpi), C.c_float(1.0), C.c_uint(1))
    out.update(plain_step1_grad=grad, plain_step1_count=np.array([stt[1]], np.int32), plain_step1_loss=sl.copy())
    for frac, steps in ((1.0, 40), (0.2, 40)):
        g, m, v, losses = ref_fit(ref, gen, tg, 12, 0.05, spec.lrPerSpacing, frac, steps)
        key = f"plain_f{int(frac * 100)}"
        out.update({f"{key}_gen": g, f"{key}_m": m, f"{key}_v": v, f"{key}_losses": losses})
    # ---- the local-edit sequence: global schedule, then UpdateTargets, UpdateGenerators(rect),
    #      BeginSchedule(localIterations, rect) and Optimize (tests/edit_case.py)
    sys.path.insert(0, str(HERE.parent))
    from edit_case import edit_case  # noqa: E402

    (g1, m1, v1, l1), (g2, m2, v2, l2) = ref_local_edit(ref, edit_case())
    out.update(edit_global_gen=g1, edit_global_m=m1, edit_global_v=v1, edit_global_losses=l1, edit_local_gen=g2,
               edit_local_m=m2, edit_local_v=v2, edit_local_losses=l2)
    # ---- k=16 loss pass (kLossK patched to 16)
    gen16 = synth.uniform(3, 1, 1024)
    tg16 = synth.circle(3, 2, 8192, 0.6, 1e-3)
    gw16, gh16 = orc.grid_dims(2.0, 2.0, 0.06)
    st16, si16, sp16, _ = ref_grid(ref, gen16, gw16, gh16, 0.06)
    stt = np.array([1, 0], np.int32)
    sl = np.zeros(1, np.float32)
    grad16 = np.zeros_like(gen16)
    rpf, rpi = run_params(0.06, 0.09, 1024, 1, 2.0, 300, 300)
    ref.ref_loss(16, P(tg16), len(tg16), P(st16), P(si16), P(sp16), gw16, gh16, C.c_float(0.06), P(gen16), P(grad16),
                 P(stt), P(sl), P(rpf), P(rpi), C.c_float(1.0), C.c_uint(1))
    out.update(k16_grad=grad16, k16_count=np.array([stt[1]], np.int32), k16_loss=sl.copy())
    # ---- extraction: 300 generators, occupancy of a disc
    gen_c = synth.uniform(8, 1, 300)
    gen_c[::17] = -1.0
    gwc, ghc = orc.grid_dims(2.0, 2.0, 0.12)
    stc, sic, spc, _ = ref_grid(ref, gen_c, gwc, ghc, 0.12)
    tiles = 4  # 32x32 voxels of size 2/32 in 4x4 tiles of 8x8
    masks = np.zeros(tiles * tiles, np.uint64)
    for j in range(32):
        for i in range(32):
            x, y = (i + 0.5) * 2 / 32 - 1, (j + 0.5) * 2 / 32 - 1
            if x * x + y * y < 0.6 ** 2:
                masks[(j >> 3) * tiles + (i >> 3)] |= np.uint64(1) << np.uint64(((j & 7) << 3) | (i & 7))
    n = len(gen_c)
    verts = np.zeros((n * 24, 2), np.float32)
    edges = np.zeros(n * 24, np.int32)
    counts = np.zeros(n, np.int32)
    inside = np.zeros(n, np.uint8)
    flags = np.zeros(2, np.int32)
    ref.ref_cells(P(stc), P(sic), P(spc), gwc, ghc, C.c_float(0.12), P(gen_c), n, C.c_float(2.0), C.c_float(2.0),
                  P(masks), tiles, tiles, C.c_float(16.0), P(verts), P(edges), P(counts), P(inside), P(flags))
    out.update(cells_masks=masks, cells_verts=verts.reshape(n, 24, 2), cells_edges=edges.reshape(n, 24),
               cells_counts=counts, cells_inside=inside, cells_flags=flags)
    # ---- Poisson: unit square, r=0.02, trials 30, seed 1; then three region resamples
    cs = C.c_float()
    pgw, pgh = C.c_int(), C.c_int()
    ref.ref_poisson_dims(C.c_float(1.0), C.c_float(1.0), C.c_float(0.02), C.byref(cs), C.byref(pgw), C.byref(pgh))
    grid = np.full((pgw.value * pgh.value, 2), -1.0, np.float32)
    ref.ref_poisson_resample(P(grid), C.c_float(1.0), C.c_float(1.0), C.c_float(0.02), cs, pgw, pgh, C.c_uint(1), 0, 0,
                             pgw, pgh, 30, C.c_uint(0))
    out["poisson_fill"] = grid.copy()
    base = 30
    for (x0, y0, x1, y1) in ((5, 5, 17, 13), (0, 0, 3, 40), (30, 30, 80, 80)):
        ref.ref_poisson_resample(P(grid), C.c_float(1.0), C.c_float(1.0), C.c_float(0.02), cs, pgw, pgh, C.c_uint(1),
                                 max(x0, 0), max(y0, 0), min(x1, pgw.value), min(y1, pgh.value), 30, C.c_uint(base))
        base += 30
    out["poisson_regions"] = grid
    np.savez_compressed(HERE / "reference_kernels.npz", **out)
    print("wrote", HERE / "reference_kernels.npz", sum(v.nbytes for v in out.values()), "bytes raw")


if __name__ == "__main__":
    main()
