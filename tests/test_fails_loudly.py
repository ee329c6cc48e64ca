"""The product has no CPU fallback: without its library, or without a GPU,
every entry point raises instead of computing anything."""
import os
import subprocess
import sys

import pytest
from conftest import ROOT


def _run(code, env):
    return subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)


def test_missing_library_raises():
    env = dict(os.environ, VOROMESH_GB300_LIB=str(ROOT / "no_such_library.so"),
               PYTHONPATH=os.pathsep.join([str(ROOT / "bb-temp-testing_gb300"), str(ROOT)]))
    r = _run("import voromesh_gb300 as vm\n"
             "try:\n"
             "    vm.VoroOptimizer(2.0, 2.0, 0.05)\n"
             "except ImportError as e:\n"
             "    print('raised', e)\n", env)
    assert r.returncode == 0 and r.stdout.startswith("raised") and "no_such_library.so" in r.stdout, r.stdout + r.stderr


def test_no_device_raises():
    """On a host without a CUDA device the optimiser, sampler and canvas
    constructors report an error status (skipped where a GPU is present)."""
    env = dict(os.environ, PYTHONPATH=os.pathsep.join([str(ROOT / "bb-temp-testing_gb300"), str(ROOT)]))
    r = _run("import voromesh_gb300 as vm\n"
             "has_gpu = __import__('torch').cuda.is_available()\n"
             "out = []\n"
             "for make in (lambda: vm.VoroOptimizer(2.0, 2.0, 0.05), lambda: vm.Sampler(1.0, 1.0, 0.02),\n"
             "             lambda: vm.Canvas(8.0, 8.0, 1.0)):\n"
             "    try:\n"
             "        make()\n"
             "        out.append('ok')\n"
             "    except vm.VmError as e:\n"
             "        out.append('error %d' % e.code)\n"
             "print('gpu' if has_gpu else 'nogpu', *out)\n", env)
    assert r.returncode == 0, r.stderr[-2000:]
    words = r.stdout.split()
    if words[0] == "gpu":
        pytest.skip("a CUDA device is present")
    assert words[1:] == ["error", "8"] * 3, r.stdout  # VM_ERR_NODEVICE from each constructor
