"""Builds libvoromesh_gb300.so in-tree (nvcc for sm_103a, parallel, no cmake).

The library holds the CUDA kernels, the C ABI (include/vm_capi.h), the
reference-compatible C++ classes (include/voromesh, include/poisson) and the
batched/serving runtime. The seeded input generators (csrc/synth.c, host
code) are a library of their own, libvm_synth.so, so that a program that
only needs the inputs (the CPU baseline) does not load the GPU library.
Outputs: bb-temp-testing_gb300/voromesh_gb300/_lib/libvoromesh_gb300.so and
libvm_synth.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
ROOT = PKG.parent.parent
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libvoromesh_gb300.so"
SYNTH_LIB = OUT_DIR / "libvm_synth.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: a*b+c stays two IEEE roundings in device code (the reference's
# arithmetic read literally); -ffp-contract=off does the same for host code.
NVFLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                  "-I" + str(INCLUDE), "-I" + str(CSRC)]
CFLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]

CU_SOURCES = ["vm_loss.cu", "vm_step.cu", "vm_extract.cu", "vm_poisson.cu", "vm_canvas.cu", "vm_runtime.cu", "vm_batch.cu",
              "vm_noalloc.cu"]
CXX_SOURCES = ["voro_optimizer.cpp", "poisson_disk.cpp", "canvas.cpp"]
C_SOURCES = ["synth.c"]


def _nvcc() -> str:
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nv).exists():
        raise RuntimeError("nvcc not found")
    return nv


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h"))
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    objdir = OUT_DIR / "obj"
    objdir.mkdir(parents=True, exist_ok=True)
    jobs = []
    for s in CU_SOURCES + CXX_SOURCES:
        src = CSRC / s
        if not src.exists():
            continue
        obj = objdir / (s + ".o")
        if force or _stale(obj, src):
            jobs.append([nvcc] + NVFLAGS + ["-c", str(src), "-o", str(obj)])
    for s in C_SOURCES:
        src = CSRC / s
        obj = objdir / (s + ".o")
        if force or _stale(obj, src):
            jobs.append(["gcc"] + CFLAGS + ["-c", str(src), "-o", str(obj)])
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            list(ex.map(_run, jobs))
    objs = [str(objdir / (s + ".o")) for s in CU_SOURCES + CXX_SOURCES if (CSRC / s).exists()]
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc] + ARCH + ["-shared", "-o", str(tmp)] + objs + ["-lcudart"])
        os.replace(tmp, LIB)
    if force or jobs or not SYNTH_LIB.exists():
        tmp = SYNTH_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-shared", "-o", str(tmp)] + [str(objdir / (s + ".o")) for s in C_SOURCES] + ["-lm"])
        os.replace(tmp, SYNTH_LIB)
    if verbose:
        print(f"built {LIB} and {SYNTH_LIB.name}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
