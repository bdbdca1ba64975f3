"""The reference arm of bench.py on the CPU: `--impl reference` times the oracle's
half-spinor DhopEO + DhopOE on the host cores and prints one JSON line on the same
metric, unit and workload as the GPU arm, with its own cpu_baseline and an end-to-end
figure that moves no bytes over the host link.  The arm loads no part of the CUDA
library."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    sys.path.insert(0, str(ROOT))
    import bench

    run = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [ln for ln in run.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 1
    assert d["config"]["workload"] == "mobius_dwf_16^4xLs16_dhop_eo_oe_fp32"
    assert d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "half-spinor" in cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_no_product_library():
    """The arm's process maps only the oracle's library, never libgbdwf.so."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "maps = open('/proc/self/maps').read();"
            "assert 'libgbdwf' not in maps, 'product library loaded';"
            "assert 'liboracle' in maps; print('clean')")
    run = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    assert "clean" in run.stdout


def test_cpu_kernel_table_times_the_oracle_only():
    """The bench's CPU kernel table (Mooee, MooeeInv of the 16^4 x 16 workload on the host
    cores) runs the oracle's FP32 loops and reports positive times and GB/s."""
    sys.path.insert(0, str(ROOT))
    import bench

    out = bench.extra_cpu_kernels(budget_s=0.05)
    assert out["cores"] >= 1
    for name in ("Mooee", "MooeeInv"):
        assert out[name]["reps"] >= 1 and out[name]["ms"] > 0 and out[name]["gbs"] > 0
