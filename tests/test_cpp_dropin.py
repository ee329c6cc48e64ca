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
