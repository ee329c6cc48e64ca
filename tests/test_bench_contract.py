"""bench.py's reference arm on the CPU: one full oracle step of the 1M-site
workload, printed as the one JSON line of the bench contract
(same metric and unit as the GPU arm, a cpu_baseline describing the run and
an e2e object with no host-device traffic)."""
import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    sys.path.insert(0, str(ROOT))
    import bench

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "site-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["sites"] == bench.N_SITES and d["config"]["targets"] == bench.N_TARGETS


def test_reference_arm_loads_no_gpu_library():
    """The reference arm's inputs come from libvm_synth.so and its steps from
    the oracle: the GPU library is never loaded."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']; "
            "import bench; bench.main(); maps = open('/proc/self/maps').read(); "
            "print('GPU_LIB_LOADED' if 'libvoromesh_gb300' in maps else 'GPU_LIB_ABSENT'); "
            "print('SYNTH_LOADED' if 'libvm_synth' in maps else 'SYNTH_ABSENT')")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "GPU_LIB_ABSENT" in r.stdout and "SYNTH_LOADED" in r.stdout
