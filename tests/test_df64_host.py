"""The double-float arithmetic of the FP64 hopping term (grid_gb300/csrc/gb_df64.cuh), built
for the host with g++ (tests/cpp/test_df64.cpp): the integer split of a double into two
floats and the widening back, the Dhop's chains of sums and Dot2 products against long
double, and a hopping-term site's relative L2 error below 1e-14."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_df64_arithmetic_on_the_host(tmp_path):
    exe = tmp_path / "test_df64"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", "-ffp-contract=off",
                    f"-I{ROOT / 'grid_gb300' / 'csrc'}", str(ROOT / "tests" / "cpp" / "test_df64.cpp"), "-o",
                    str(exe)], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
