"""The C-ABI library loads on a host without a GPU and exports every function
include/*.h declares (no compute calls)."""
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def libpath():
    from voromesh_gb300 import build as b

    if not b.LIB.exists():
        b.build()
    return b.LIB


def _declared_c_functions():
    text = (ROOT / "include" / "vm_capi.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:vm|vmb|vms|pd|cv)_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_loads_without_gpu(libpath):
    import ctypes

    lib = ctypes.CDLL(str(libpath))
    lib.vm_error_string.restype = ctypes.c_char_p
    assert lib.vm_error_string(0) == b"ok"


def test_every_c_function_is_exported(libpath):
    import ctypes

    lib = ctypes.CDLL(str(libpath))
    names = _declared_c_functions()
    assert len(names) >= 30
    for prefix in ("vm_", "vmb_", "vms_", "pd_", "cv_"):
        assert any(n.startswith(prefix) for n in names), prefix
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_cpp_classes_are_exported(libpath):
    out = subprocess.run(["nm", "-DC", "--defined-only", str(libpath)], capture_output=True, text=True).stdout
    for sym in ["voromesh::VoroOptimizer::VoroOptimizer(float, float, float, voromesh::OptimizerParams const&)",
                "voromesh::VoroOptimizer::SetTargets(std::vector<voromesh::Vec2, std::allocator<voromesh::Vec2> > const&)",
                "voromesh::VoroOptimizer::Step(int)", "voromesh::VoroOptimizer::EvaluateLoss()",
                "voromesh::VoroOptimizer::Extract()", "voromesh::VoroOptimizer::BeginSchedule(int, int, int, int, int)",
                "poisson::Sampler::Sampler(float, float, float, int, unsigned int)",
                "poisson::Sampler::Resample(int, int, int, int)", "poisson::Sampler::Verify(int, int, int, int) const",
                "voromesh::SetDefaultLossNeighbours(int)",
                "voromesh::Canvas::Canvas(float, float, float)",
                "voromesh::Canvas::StampDisc(voromesh::Vec2, float, bool)",
                "voromesh::Canvas::RasterizeShape(std::vector<voromesh::Vec2, std::allocator<voromesh::Vec2> > const&)",
                "voromesh::UpdateFromCanvas(voromesh::VoroOptimizer&, voromesh::Canvas const&)"]:
        assert sym in out, sym


def test_status_codes_without_gpu(libpath):
    """Argument checks answer before any device call."""
    import ctypes as C

    lib = C.CDLL(str(libpath))
    assert lib.vm_create(C.c_float(-1.0), C.c_float(1.0), C.c_float(0.1), None, C.byref(C.c_void_p())) == 1
    assert lib.pd_create(C.c_float(1.0), C.c_float(1.0), C.c_float(0.0), 30, 1, C.byref(C.c_void_p())) == 1
    assert lib.cv_create(C.c_float(1.0), C.c_float(1.0), C.c_float(0.0), C.byref(C.c_void_p())) == 1
    buf = C.create_string_buffer(256)
    assert lib.vm_last_error(buf, 256) == 0 and len(buf.value) > 0


C_CALLER = r"""
#include "vm_capi.h"
#include <stdio.h>
int main(void)
{
    int major = 0, minor = 0, sm = 0;
    char msg[256];
    vm_optimizer *h = NULL;
    int rv = vm_version(&major, &minor, &sm);
    int rc = vm_create(-1.0f, 1.0f, 1.0f, NULL, &h);
    vm_last_error(msg, (int)sizeof msg);
    printf("%d %d %d %d\n", rv, major, rc, h == NULL);
    return 0;
}
"""


def test_c_header_is_plain_c(libpath, tmp_path):
    """include/vm_capi.h compiles as C99 on its own (what a cgo or C binding
    includes) and a C caller links and runs against the library."""
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
                        str(src), f"-L{libpath.parent}", "-lvoromesh_gb300", f"-Wl,-rpath,{libpath.parent}", "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.split() == ["0", "1", "1", "1"], out.stdout + out.stderr


@pytest.mark.parametrize("header", ["voromesh/voro_optimizer.h", "voromesh/canvas.h", "voromesh/gb300_ext.h",
                                    "voromesh/shape2d.h", "poisson/poisson_disk.h", "vm_capi.h"])
def test_header_self_contained(header, tmp_path):
    """Each public header compiles on its own as C++17."""
    src = tmp_path / "h.cpp"
    src.write_text(f'#include "{header}"\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only",
                        f"-I{ROOT / 'include'}", str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def _method_names(text, public_only):
    """Capitalised names followed by '(' (the reference's method style); with
    public_only, only those before the first private section."""
    text = re.sub(r"//.*", "", text)
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    if public_only:
        text = text.split("private:")[0]
    return set(re.findall(r"\b([A-Z][A-Za-z0-9]*)\s*\(", text))


@pytest.mark.parametrize("header", ["voromesh/voro_optimizer.h", "voromesh/canvas.h", "poisson/poisson_disk.h"])
def test_reference_public_api_is_complete(header):
    """Every public method the reference's header declares is declared in this
    library's header of the same name (where the reference sources are
    present)."""
    import __graft_entry__ as g

    ref = Path(g.REFERENCE_SOURCES) / "include" / header
    if not ref.exists():
        pytest.skip("the reference sources are not present")
    missing = _method_names(ref.read_text(), True) - _method_names((ROOT / "include" / header).read_text(), False)
    assert not missing, sorted(missing)
