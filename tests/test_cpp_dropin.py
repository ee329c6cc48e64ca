"""The C++ drop-in boundary: a caller written against the reference's
include/voromesh and include/poisson headers (tests/cpp/dropin_demo.cpp)
compiles and links against libvoromesh_gb300.so unchanged, and on a GPU its
results equal the same call sequence made through the Python binding."""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "dropin_demo.cpp"
LIBDIR = ROOT / "bb-temp-testing_gb300" / "voromesh_gb300" / "_lib"


def _build(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    if not (LIBDIR / "libvoromesh_gb300.so").exists():
        pytest.skip("library not built")
    exe = tmp_path / "dropin_demo"
    # -ffp-contract=off: the caller's own float edits round like numpy's
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(SRC),
           f"-L{LIBDIR}", "-lvoromesh_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_caller_compiles_and_links(tmp_path):
    _build(tmp_path)


def _disc_masks(tiles=10, voxel=0.025):
    masks = np.zeros(tiles * tiles, np.uint64)
    for j in range(tiles * 8):
        for i in range(tiles * 8):
            x = np.float32(np.float32(i + 0.5) * np.float32(voxel)) - np.float32(1.0)
            y = np.float32(np.float32(j + 0.5) * np.float32(voxel)) - np.float32(1.0)
            if x * x + y * y < np.float32(0.36):
                masks[(j >> 3) * tiles + (i >> 3)] |= np.uint64(1) << np.uint64(((j & 7) << 3) | (i & 7))
    return masks


@pytest.mark.gpu
def test_cpp_caller_matches_python(vm, tmp_path):
    from voromesh_gb300 import synth

    exe = _build(tmp_path)
    spec = synth.plain_fit()
    gen, tgt = spec.generators.astype(np.float32), spec.targets.astype(np.float32)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(gen), len(tgt)], np.int32).tofile(f)
        gen.tofile(f)
        tgt.tofile(f)
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = out.read_bytes()
    loss0, loss1 = np.frombuffer(raw[:8], np.float32)
    samples, verified, watertight, loops, nedges = np.frombuffer(raw[8:28], np.int32)
    gens_cpp = np.frombuffer(raw[28:], np.float32).reshape(-1, 2)

    # the same sequence through the Python binding
    s = vm.Sampler(1.0, 1.0, 0.02, 30, 1)
    s.ResampleAll()
    assert samples == int((s.Cells()[:, 0] >= 0).sum()) and verified == 1
    s.close()
    p = vm.OptimizerParams(iterations=60, localIterations=20, sampleFraction=1.0, lossK=12)
    o = vm.VoroOptimizer(2.0, 2.0, 0.05, p)
    o.SetTargets(tgt)
    masks = _disc_masks()
    o.SetOccupancy(masks, 10, 10, 0.025)
    o.SetGenerators(gen, len(gen), 1, 2.0)
    o.BeginSchedule(60)
    o.Optimize()
    assert np.float32(o.EvaluateLoss()) == loss0
    slots = tgt.copy()
    slots[:64, 0] = slots[:64, 0] * np.float32(0.98) + np.float32(0.02)
    o.UpdateTargets(np.arange(64), slots)
    o.UpdateOccupancy(masks, 0, 0, 10, 10)
    moved = gen.copy()
    moved[:256, 0] = np.where(moved[:256, 0] < 0, moved[:256, 0], moved[:256, 0] * np.float32(0.999))
    o.UpdateGenerators(moved, 0, 0, 256, 1)
    o.BeginSchedule(20, 0, 0, 256, 1)
    o.Optimize()
    assert np.float32(o.EvaluateLoss()) == loss1
    m = o.Extract()
    o.close()
    assert np.array_equal(gens_cpp, m.generators)
    assert bool(watertight) == m.watertight and loops == m.loops and nedges == len(m.edges)
    assert watertight == 1 and nedges > 0


CANVAS_SRC = ROOT / "tests" / "cpp" / "canvas_demo.cpp"


def _build_canvas(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    if not (LIBDIR / "libvoromesh_gb300.so").exists():
        pytest.skip("library not built")
    exe = tmp_path / "canvas_demo"
    cmd = [gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Werror", f"-I{ROOT / 'include'}",
           str(CANVAS_SRC), f"-L{LIBDIR}", "-lvoromesh_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_canvas_caller_compiles_and_links(tmp_path):
    _build_canvas(tmp_path)


@pytest.mark.gpu
def test_cpp_canvas_caller_matches_python(vm, tmp_path):
    """The C++ Canvas (host mirrors, lazy refresh) and the canvas-to-optimiser
    hand-off give what the Python binding and the host route give."""
    from voromesh_gb300 import synth

    exe = _build_canvas(tmp_path)
    poly = synth.heart(128.0, 128.0, 200.0, 512)
    stamps = np.array([[128, 40, 20, 0], [60, 120, 15, 1], [200, 150, 25, 0], [128, 128, 10, 1],
                       [-50, -50, 5, 1], [190, 60, 30, 1]], np.float32)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([len(poly), len(stamps)], np.int32).tofile(f)
        poly.tofile(f)
        stamps.tofile(f)
    r = subprocess.run([str(exe), str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.frombuffer(out.read_bytes(), np.uint8)
    pos = 0

    def take(dtype, n):
        nonlocal pos
        a = np.frombuffer(raw[pos:pos + n * np.dtype(dtype).itemsize].tobytes(), dtype)
        pos += n * np.dtype(dtype).itemsize
        return a

    c = vm.Canvas(256.0, 256.0, 1.0)
    c.RasterizeShape(poly)
    p = vm.OptimizerParams(sampleFraction=1.0)
    o = vm.VoroOptimizer(256.0, 256.0, 8.0, p)
    o.SetTargets(c.TargetSlots())
    o.SetOccupancy(c.InsideMasks(), c.TilesX(), c.TilesY(), c.VoxelSize())
    g = np.array([((i + 0.5) * 8.0, (j + 0.5) * 8.0) for j in range(32) for i in range(32)], np.float32)
    o.SetGenerators(g, 32, 32, 8.0)
    o.BeginSchedule(20)
    o.Optimize()
    for cx, cy, rr, ins in stamps:
        e = c.StampDisc((cx, cy), rr, bool(ins))
        head = take(np.int32, 8)
        assert tuple(head[:7]) == (e.tx0, e.ty0, e.tx1, e.ty1, e.removed, e.added, e.flipped)
        assert np.array_equal(take(np.int32, int(head[7])), e.dirtySlots)
        if e.Changed():
            o.UpdateTargets(e.dirtySlots, c.TargetSlots())
            o.UpdateOccupancy(c.InsideMasks(), e.tx0, e.ty0, e.tx1, e.ty1)
            o.BeginSchedule(5)
            o.Optimize()
    ns = int(take(np.int32, 1)[0])
    assert np.array_equal(take(np.float32, 2 * ns).reshape(-1, 2), c.TargetSlots())
    nt = int(take(np.int32, 1)[0])
    assert np.array_equal(take(np.uint64, nt), c.InsideMasks())
    tail = take(np.int32, 4)
    assert tail[0] == c.SurfaceCount() and tail[1] == c.SurfaceTileCount() and tail[2] == int(c.IsInside(100, 100))
    assert tail[3] == 1
    assert take(np.float32, 1)[0] == np.float32(o.EvaluateLoss())
