"""ctypes front end of the CPU oracle (oracle/vm_oracle.c) and, when it has
been built here, of the reference's own kernels run on the CPU
(oracle/_ref/libref_kernels.so, built by oracle/ref_shim/build_ref.sh).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker. The product never loads it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libvm_oracle.so"
REF_LIB = HERE / "_ref" / "libref_kernels.so"

ACC_REF, ACC_FIXED = 0, 1
POW_REF, POW_DET = 0, 1

_lib = None
_ref = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _lib.vo_fit_create.restype = C.c_void_p
        _lib.vo_fit_create.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_float,
                                       C.c_void_p, C.c_int, C.c_uint, C.c_int, C.c_int, C.c_int]
        _lib.vo_fit_step.restype = C.c_float
        _lib.vo_fit_step.argtypes = [C.c_void_p, C.c_int]
        _lib.vo_fit_eval_loss.restype = C.c_float
        _lib.vo_fit_eval_loss.argtypes = [C.c_void_p]
        for n in ("vo_fit_destroy",):
            getattr(_lib, n).argtypes = [C.c_void_p]
        _lib.vo_fit_set_targets.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.vo_fit_set_generators.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float]
        _lib.vo_fit_begin_schedule.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.vo_fit_update_generators.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.vo_fit_get.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fit_grid.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fit_grid_size.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fit_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fit_iteration.argtypes = [C.c_void_p]
        _lib.vo_fit_schedule_length.argtypes = [C.c_void_p]
        _lib.vo_fit64_create.restype = C.c_void_p
        _lib.vo_fit64_create.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                                         C.c_double, C.c_void_p, C.c_int, C.c_uint, C.c_int]
        _lib.vo_fit64_destroy.argtypes = [C.c_void_p]
        _lib.vo_fit64_set_targets.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _lib.vo_fit64_set_generators.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double]
        _lib.vo_fit64_step.restype = C.c_double
        _lib.vo_fit64_step.argtypes = [C.c_void_p, C.c_int]
        _lib.vo_fit64_eval_loss.restype = C.c_double
        _lib.vo_fit64_eval_loss.argtypes = [C.c_void_p]
        _lib.vo_fit64_get.argtypes = [C.c_void_p, C.c_void_p]
        _lib.vo_fit64_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fit64_detail.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_poisson_resample.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.vo_poisson_resample_mt.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.vo_poisson_verify.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        _lib.vo_poisson_init.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_int, C.c_uint]
        _lib.vo_extract_cells.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_int,
                                          C.c_int, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_int]
        _lib.vo_assemble.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_free.argtypes = [C.c_void_p]
        _lib.vo_build_grid.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]
        _lib.vo_knn.argtypes = [C.c_void_p, VoF2, C.c_int, C.c_void_p, C.c_void_p]
        _lib.vo_knn_many.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        _lib.vo_knn_brute.argtypes = [C.c_void_p, C.c_int, VoF2, C.c_int, C.c_void_p, C.c_void_p]
        _lib.vo_loss_detail.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_float,
                                        C.c_uint, C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.vo_fixed_loss_to_float.restype = C.c_float
        _lib.vo_fixed_loss_to_float.argtypes = [C.c_uint64, C.c_uint64, C.c_int]
        _lib.vo_fixed_to_float.restype = C.c_float
        _lib.vo_fixed_to_float.argtypes = [C.c_int64, C.c_int]
        _lib.vo_fixed2_to_float.restype = C.c_float
        _lib.vo_fixed2_to_float.argtypes = [C.c_int64, C.c_uint64, C.c_int]
        _lib.vo_fixed_from_float.restype = C.c_int64
        _lib.vo_fixed_from_float.argtypes = [C.c_float, C.c_int]
        _lib.vo_fixed_grad_exp.argtypes = [C.c_float]
        _lib.vo_fixed_loss_exp.argtypes = [C.c_float]
        _lib.vo_fixed_loss_add.argtypes = [C.c_float, C.c_int, C.c_void_p, C.c_void_p]
        _lib.vo_pow_det.restype = C.c_float
        _lib.vo_pow_det.argtypes = [C.c_float, C.c_int]
        _lib.vo_rand01.restype = C.c_float
        _lib.vo_rand01.argtypes = [C.c_uint, C.c_uint, C.c_uint]
    return _lib


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        _ref = C.CDLL(str(REF_LIB))
    return _ref


class VoF2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class VoGrid(C.Structure):
    _fields_ = [("w", C.c_int), ("h", C.c_int), ("cellSize", C.c_float), ("start", C.c_void_p),
                ("idx", C.c_void_p), ("pos", C.c_void_p)]


class VoPoisson(C.Structure):
    _fields_ = [("width", C.c_float), ("height", C.c_float), ("radius", C.c_float), ("cellSize", C.c_float),
                ("gridW", C.c_int), ("gridH", C.c_int), ("trials", C.c_int), ("seed", C.c_uint),
                ("roundBase", C.c_uint)]


def P(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def grid_dims(width: float, height: float, spacing: float):
    f = np.float32
    gw = max(1, int(np.ceil(f(width) / f(spacing))))
    gh = max(1, int(np.ceil(f(height) / f(spacing))))
    return gw, gh


def build_grid(gen: np.ndarray, gw: int, gh: int, cell: float):
    n = len(gen)
    start = np.zeros(gw * gh + 1, np.int32)
    sidx = np.zeros(max(n, 1), np.int32)
    spos = np.zeros((max(n, 1), 2), np.float32)
    gcell = np.zeros(max(n, 1), np.int32)
    lib().vo_build_grid(P(gen), n, gw, gh, C.c_float(cell), P(gcell), P(start), P(sidx), P(spos))
    live = int(start[-1])
    return start, sidx[:live], spos[:live], gcell[:n]


class Grid:
    """A cell-sorted hash grid held for vo_knn / vo_extract_cells calls."""

    def __init__(self, gen: np.ndarray, gw: int, gh: int, cell: float):
        self.gen = np.ascontiguousarray(gen, np.float32)
        self.start, self.sidx, self.spos, self.gcell = build_grid(self.gen, gw, gh, cell)
        self.sidx = np.ascontiguousarray(self.sidx)
        self.spos = np.ascontiguousarray(self.spos)
        self.c = VoGrid(gw, gh, cell, P(self.start).value, P(self.sidx).value, P(self.spos).value)

    def knn(self, queries: np.ndarray, K: int, nthreads: int = 1):
        q = np.ascontiguousarray(queries, np.float32)
        idx = np.empty((len(q), K), np.int32)
        d2 = np.empty((len(q), K), np.float32)
        lib().vo_knn_many(C.byref(self.c), P(q), len(q), K, P(idx), P(d2), nthreads)
        return idx, d2

    def cells(self, width: float, height: float, masks=None, tilesX=0, tilesY=0, invVoxel=0.0, nthreads=1):
        n = len(self.gen)
        verts = np.zeros((n * 24, 2), np.float32)
        edges = np.zeros(n * 24, np.int32)
        count = np.zeros(n, np.int32)
        inside = np.zeros(n, np.uint8)
        flags = np.zeros(2, np.int32)
        m = None if masks is None else np.ascontiguousarray(masks, np.uint64)
        lib().vo_extract_cells(C.byref(self.c), P(self.gen), n, C.c_float(width), C.c_float(height), P(m), tilesX,
                               tilesY, C.c_float(invVoxel), P(verts), P(edges), P(count), P(inside), P(flags), nthreads)
        return verts.reshape(n, 24, 2), edges.reshape(n, 24), count, inside, flags


def assemble(verts, labels, counts, inside):
    n = len(counts)
    v = np.ascontiguousarray(verts.reshape(-1, 2), np.float32)
    lab = np.ascontiguousarray(labels.reshape(-1), np.int32)
    cnt = np.ascontiguousarray(counts, np.int32)
    ins = np.ascontiguousarray(inside, np.uint8)
    cs = np.zeros(n + 1, np.int32)
    mv = C.c_void_p()
    ed = C.c_void_p()
    ne, wt, lp = C.c_int(), C.c_int(), C.c_int()
    L = lib()
    L.vo_assemble.restype = C.c_int
    nv = L.vo_assemble(P(v), P(lab), P(cnt), P(ins), n, P(cs), C.byref(mv), C.byref(ed), C.byref(ne), C.byref(wt),
                       C.byref(lp))
    verts_out = np.ctypeslib.as_array((C.c_float * (2 * nv)).from_address(mv.value)).reshape(nv, 2).copy() \
        if nv else np.zeros((0, 2), np.float32)
    edges_out = np.ctypeslib.as_array((C.c_int * (2 * ne.value)).from_address(ed.value)).reshape(-1, 2).copy() \
        if ne.value else np.zeros((0, 2), np.int32)
    L.vo_free(mv)
    L.vo_free(ed)
    return cs, verts_out, edges_out, bool(wt.value), lp.value


class Fit:
    """The optimiser restated on the CPU (FP32, reference operation order)."""

    def __init__(self, width, height, spacing, K, lrPerSpacing, sampleFraction, params_iterations, gamma=0.5,
                 milestones=(80, 150, 200, 250), seed=1, acc=ACC_FIXED, pow_mode=POW_DET, nthreads=1):
        ms = (C.c_int * 4)(*milestones)
        self.h = C.c_void_p(lib().vo_fit_create(width, height, spacing, K, lrPerSpacing, sampleFraction, gamma, ms,
                                                params_iterations, seed, acc, pow_mode, nthreads))
        self.n = 0
        self.spacing = np.float32(spacing)

    def __del__(self):
        try:
            lib().vo_fit_destroy(self.h)
        except Exception:
            pass

    def set_targets(self, t):
        t = np.ascontiguousarray(t, np.float32)
        lib().vo_fit_set_targets(self.h, P(t), len(t))

    def set_generators(self, g, slotsW, slotsH, slotCellSize):
        g = np.ascontiguousarray(g, np.float32)
        self.n = slotsW * slotsH
        lib().vo_fit_set_generators(self.h, P(g), slotsW, slotsH, slotCellSize)

    def update_generators(self, g, cx0, cy0, cx1, cy1):
        g = np.ascontiguousarray(g, np.float32)
        lib().vo_fit_update_generators(self.h, P(g), cx0, cy0, cx1, cy1)

    def begin_schedule(self, it, cx0, cy0, cx1, cy1):
        lib().vo_fit_begin_schedule(self.h, it, cx0, cy0, cx1, cy1)

    def schedule_length(self) -> int:
        return lib().vo_fit_schedule_length(self.h)

    def step(self, k=1) -> float:
        return lib().vo_fit_step(self.h, k)

    def eval_loss(self) -> float:
        return lib().vo_fit_eval_loss(self.h)

    def iteration(self) -> int:
        return lib().vo_fit_iteration(self.h)

    def generators(self):
        g = np.empty((self.n, 2), np.float32)
        m = np.empty((self.n, 2), np.float32)
        v = np.empty((self.n, 2), np.float32)
        lib().vo_fit_get(self.h, P(g), P(m), P(v))
        return g, m, v

    def grid(self):
        gw, gh = C.c_int(), C.c_int()
        lib().vo_fit_grid_size(self.h, C.byref(gw), C.byref(gh))
        start = np.empty(gw.value * gh.value + 1, np.int32)
        sidx = np.empty(max(self.n, 1), np.int32)
        spos = np.empty((max(self.n, 1), 2), np.float32)
        gcell = np.empty(max(self.n, 1), np.int32)
        lib().vo_fit_grid(self.h, P(start), P(sidx), P(spos), P(gcell))
        live = int(start[-1])
        return start, sidx[:live], spos[:live], gcell[:self.n]

    def gradient(self):
        g = np.empty((self.n, 2), np.float32)
        cnt = C.c_int()
        loss = C.c_float()
        lib().vo_fit_gradient(self.h, P(g), C.byref(cnt), C.byref(loss))
        return g, cnt.value, loss.value


def loss_detail(fit: Fit, targets, K: int, with_box=False, fraction=1.0, seed=1, iteration=0):
    """Per-target (nearest site, bisector neighbour, loss) of EvaluateLoss's
    pass over `targets` for the fit's current generators (-1/-1/0 = unused)."""
    t = np.ascontiguousarray(targets, np.float32)
    start, sidx, spos, _ = fit.grid()
    gen = fit.generators()[0]
    gw, gh = C.c_int(), C.c_int()
    lib().vo_fit_grid_size(fit.h, C.byref(gw), C.byref(gh))
    sidx = np.ascontiguousarray(sidx)
    spos = np.ascontiguousarray(spos)
    g = VoGrid(gw.value, gh.value, float(fit.spacing), P(start).value, P(sidx).value, P(spos).value)
    i0 = np.empty(len(t), np.int32)
    j = np.empty(len(t), np.int32)
    loss = np.empty(len(t), np.float32)
    lib().vo_loss_detail(P(t), len(t), C.byref(g), P(gen), K, None, C.c_float(fraction), seed, iteration, P(i0),
                         P(j), P(loss))
    return i0, j, loss


class Fit64:
    """The same optimiser in FP64 (error bars)."""

    def __init__(self, width, height, spacing, K, lrPerSpacing, sampleFraction, params_iterations, gamma=0.5,
                 milestones=(80, 150, 200, 250), seed=1, nthreads=1):
        ms = (C.c_int * 4)(*milestones)
        self.h = C.c_void_p(lib().vo_fit64_create(width, height, spacing, K, lrPerSpacing, sampleFraction, gamma, ms,
                                                  params_iterations, seed, nthreads))
        self.n = 0
        self.nt = 1

    def __del__(self):
        try:
            lib().vo_fit64_destroy(self.h)
        except Exception:
            pass

    def set_targets(self, t):
        t = np.ascontiguousarray(t, np.float32)
        self.nt = max(len(t), 1)
        lib().vo_fit64_set_targets(self.h, P(t), len(t))

    def set_generators(self, g, slotsW, slotsH, slotCellSize):
        g = np.ascontiguousarray(g, np.float32)
        self.n = slotsW * slotsH
        lib().vo_fit64_set_generators(self.h, P(g), slotsW, slotsH, slotCellSize)

    def step(self, k=1) -> float:
        return lib().vo_fit64_step(self.h, k)

    def eval_loss(self) -> float:
        return lib().vo_fit64_eval_loss(self.h)

    def generators(self):
        g = np.empty((self.n, 2), np.float64)
        lib().vo_fit64_get(self.h, P(g))
        return g

    def gradient(self):
        g = np.empty((self.n, 2), np.float64)
        cnt = C.c_int()
        loss = C.c_double()
        lib().vo_fit64_gradient(self.h, P(g), C.byref(cnt), C.byref(loss))
        return g, cnt.value, loss.value

    def detail(self):
        """Per target (nearest site, bisector neighbour) of the full-target
        pass at the current generators, in double (-1 = unused)."""
        i0 = np.empty(self.nt, np.int32)
        j = np.empty(self.nt, np.int32)
        lib().vo_fit64_detail(self.h, P(i0), P(j))
        return i0, j


def poisson_fill(width, height, radius, trials=30, seed=1, regions=(), nthreads=1):
    """Sampler construction (full fill) followed by Resample() of each region."""
    p = VoPoisson()
    L = lib()
    L.vo_poisson_init(C.byref(p), width, height, radius, trials, seed)
    grid = np.full((p.gridW * p.gridH, 2), -1.0, np.float32)
    L.vo_poisson_resample_mt(C.byref(p), P(grid), 0, 0, p.gridW, p.gridH, nthreads)
    for (x0, y0, x1, y1) in regions:
        L.vo_poisson_resample_mt(C.byref(p), P(grid), x0, y0, x1, y1, nthreads)
    return grid, p


def poisson_verify(p: VoPoisson, grid, x0, y0, x1, y1) -> bool:
    return bool(lib().vo_poisson_verify(C.byref(p), P(np.ascontiguousarray(grid, np.float32)), x0, y0, x1, y1))


# ---------------------------------------------------------------------------
# Canvas (src/voromesh/canvas.cpp): the oracle restatement (vo_canvas.c) and,
# where it was built here, the reference's own class (oracle/_ref).
# ---------------------------------------------------------------------------
REF_CANVAS_LIB = HERE / "_ref" / "libref_canvas.so"
_refc = None


def ref_canvas_available() -> bool:
    return REF_CANVAS_LIB.exists()


def _canvas_lib() -> C.CDLL:
    L = lib()
    if not hasattr(L, "_canvas_ready"):
        L.vo_canvas_create.restype = C.c_void_p
        L.vo_canvas_create.argtypes = [C.c_float, C.c_float, C.c_float]
        L.vo_canvas_destroy.argtypes = [C.c_void_p]
        L.vo_canvas_rasterize.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.vo_canvas_stamp.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]
        L.vo_canvas_dims.argtypes = [C.c_void_p, C.c_void_p]
        L.vo_canvas_counts.argtypes = [C.c_void_p, C.c_void_p]
        L.vo_canvas_get.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        L._canvas_ready = True
    return L


def ref_canvas() -> C.CDLL:
    global _refc
    if _refc is None:
        _refc = C.CDLL(str(REF_CANVAS_LIB))
        _refc.rc_canvas_create.restype = C.c_void_p
        _refc.rc_canvas_create.argtypes = [C.c_float, C.c_float, C.c_float]
        _refc.rc_canvas_destroy.argtypes = [C.c_void_p]
        _refc.rc_canvas_rasterize.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        _refc.rc_canvas_stamp.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_int]
        _refc.rc_canvas_counts.argtypes = [C.c_void_p, C.c_void_p]
        _refc.rc_canvas_get.argtypes = [C.c_void_p] + [C.c_void_p] * 6
        _refc.rc_make_heart.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]
    return _refc


def canvas_dims(width: float, height: float, voxel: float):
    """voxelsX, voxelsY, tilesX, tilesY (canvas.cpp:33-38)."""
    f = np.float32
    vx = int(np.ceil(f(width) / f(voxel)))
    vy = int(np.ceil(f(height) / f(voxel)))
    return vx, vy, (vx + 7) // 8, (vy + 7) // 8


class CanvasEdit:
    def __init__(self, tx0=0, ty0=0, tx1=0, ty1=0, removed=0, added=0, flipped=0, dirty=()):
        self.tx0, self.ty0, self.tx1, self.ty1 = tx0, ty0, tx1, ty1
        self.removed, self.added, self.flipped = removed, added, flipped
        self.dirty = np.asarray(dirty, np.int32)

    def rect(self):
        return (self.tx0, self.ty0, self.tx1, self.ty1)

    def counts(self):
        return (self.removed, self.added, self.flipped)


class _CanvasBase:
    def state(self) -> dict:
        """Full canvas state in one layout: slots (n,2) f32, free (nfree,)
        i32, inside/smask (tiles,) u64, spt (tiles*64,2) f32, sslot
        (tiles*64,) i32, counts (slots, free, surface voxels, surface tiles)."""
        raise NotImplementedError


class Canvas(_CanvasBase):
    """The oracle restatement (vo_canvas.c)."""

    def __init__(self, width, height, voxel):
        self.h = _canvas_lib().vo_canvas_create(width, height, voxel)
        if not self.h:
            raise MemoryError("vo_canvas_create")
        self.dims = canvas_dims(width, height, voxel)

    def __del__(self):
        if getattr(self, "h", None):
            _canvas_lib().vo_canvas_destroy(self.h)
            self.h = None

    def rasterize(self, poly):
        poly = np.ascontiguousarray(poly, np.float32).reshape(-1, 2)
        if _canvas_lib().vo_canvas_rasterize(self.h, P(poly), len(poly)):
            raise MemoryError("vo_canvas_rasterize")

    def stamp(self, cx, cy, r, inside) -> CanvasEdit:
        e = (C.c_int * 8)()
        if _canvas_lib().vo_canvas_stamp(self.h, cx, cy, r, int(bool(inside)), C.byref(e)):
            raise MemoryError("vo_canvas_stamp")
        dirty = np.zeros(max(e[7], 1), np.int32)
        _canvas_lib().vo_canvas_get(self.h, None, None, None, None, None, None, P(dirty))
        return CanvasEdit(*e[:7], dirty=dirty[:e[7]])

    def counts(self):
        c = np.zeros(4, np.int64)
        _canvas_lib().vo_canvas_counts(self.h, P(c))
        return tuple(int(v) for v in c)

    def slots(self) -> np.ndarray:
        a = np.zeros((max(self.counts()[0], 1), 2), np.float32)
        _canvas_lib().vo_canvas_get(self.h, P(a), None, None, None, None, None, None)
        return a[:self.counts()[0]]

    def inside(self) -> np.ndarray:
        m = np.zeros(self.dims[2] * self.dims[3], np.uint64)
        _canvas_lib().vo_canvas_get(self.h, None, None, P(m), None, None, None, None)
        return m

    def state(self) -> dict:
        ns, nf, _, _ = self.counts()
        tiles = self.dims[2] * self.dims[3]
        st = dict(slots=np.zeros((max(ns, 1), 2), np.float32), free=np.zeros(max(nf, 1), np.int32),
                  inside=np.zeros(tiles, np.uint64), smask=np.zeros(tiles, np.uint64),
                  spt=np.zeros((tiles * 64, 2), np.float32), sslot=np.zeros(tiles * 64, np.int32))
        _canvas_lib().vo_canvas_get(self.h, P(st["slots"]), P(st["free"]), P(st["inside"]), P(st["smask"]),
                                    P(st["spt"]), P(st["sslot"]), None)
        st["slots"], st["free"] = st["slots"][:ns], st["free"][:nf]
        st["counts"] = self.counts()
        return st


class RefCanvas(_CanvasBase):
    """The reference's own voromesh::Canvas, compiled from its sources."""

    def __init__(self, width, height, voxel):
        self.h = ref_canvas().rc_canvas_create(width, height, voxel)
        self.dims = canvas_dims(width, height, voxel)

    def __del__(self):
        if getattr(self, "h", None):
            ref_canvas().rc_canvas_destroy(self.h)
            self.h = None

    def rasterize(self, poly):
        poly = np.ascontiguousarray(poly, np.float32).reshape(-1, 2)
        ref_canvas().rc_canvas_rasterize(self.h, P(poly), len(poly))

    def stamp(self, cx, cy, r, inside) -> CanvasEdit:
        e = (C.c_int * 8)()
        cap = 1 << 20
        dirty = np.zeros(cap, np.int32)
        ref_canvas().rc_canvas_stamp(self.h, cx, cy, r, int(bool(inside)), C.byref(e), P(dirty), cap)
        return CanvasEdit(*e[:7], dirty=dirty[:e[7]].copy())

    def counts(self):
        c = np.zeros(4, np.int64)
        ref_canvas().rc_canvas_counts(self.h, P(c))
        return tuple(int(v) for v in c)

    def state(self) -> dict:
        ns, nf, _, _ = self.counts()
        tiles = self.dims[2] * self.dims[3]
        st = dict(slots=np.zeros((max(ns, 1), 2), np.float32), free=np.zeros(max(nf, 1), np.int32),
                  inside=np.zeros(tiles, np.uint64), smask=np.zeros(tiles, np.uint64),
                  spt=np.zeros((tiles * 64, 2), np.float32), sslot=np.zeros(tiles * 64, np.int32))
        ref_canvas().rc_canvas_get(self.h, P(st["slots"]), P(st["free"]), P(st["inside"]), P(st["smask"]),
                                   P(st["spt"]), P(st["sslot"]))
        st["slots"], st["free"] = st["slots"][:ns], st["free"][:nf]
        st["counts"] = self.counts()
        return st


def ref_make_heart(cx, cy, width, segments):
    xy = np.zeros((segments, 2), np.float32)
    ref_canvas().rc_make_heart(cx, cy, width, segments, P(xy))
    return xy


def canvas_relabelling(a: dict, b: dict):
    """Checks that canvas states a and b are equal up to a relabelling of slot
    indices and returns the map (a slot -> b slot). Occupancy, surface masks
    and points, slot values, counts and free-list length must be identical;
    slot indices must correspond one to one through the surface voxels and
    the free-list positions. Raises AssertionError otherwise."""
    assert a["counts"] == b["counts"], (a["counts"], b["counts"])
    assert np.array_equal(a["inside"], b["inside"]), "occupancy differs"
    assert np.array_equal(a["smask"], b["smask"]), "surface masks differ"
    assert np.array_equal(a["spt"].view(np.uint32), b["spt"].view(np.uint32)), "surface points differ"
    ns = a["counts"][0]
    pi = np.full(ns, -1, np.int64)
    on = a["sslot"] >= 0
    assert np.array_equal(on, b["sslot"] >= 0)
    src = np.concatenate([a["sslot"][on], a["free"]]).astype(np.int64)
    dst = np.concatenate([b["sslot"][on], b["free"]]).astype(np.int64)
    assert len(src) == ns, "slots are neither live nor free"
    assert len(np.unique(src)) == ns and len(np.unique(dst)) == ns, "slot map is not one to one"
    pi[src] = dst
    assert np.array_equal(a["slots"].view(np.uint32), b["slots"][pi].view(np.uint32)), "slot values differ"
    return pi
