"""The Grid-shaped C++ adapter (include/gbgrid.h): a Grid-style program (tests/cpp/
test_adapter.cpp) compiles and links against the C ABI on the CPU, and on the GPU every
check it makes holds (even-odd identities, Schur and mixed-precision solves, a user
operator through the host-driven CG, surface fields, errors as exceptions)."""
import subprocess
from pathlib import Path

import pytest

import grid_gb300 as g

ROOT = Path(__file__).resolve().parents[1]


def build(tmp_path):
    exe = tmp_path / "test_adapter"
    lib_dir = Path(g.LIB_PATH).parent
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           str(ROOT / "tests" / "cpp" / "test_adapter.cpp"), "-o", str(exe), f"-L{lib_dir}", "-lgbdwf",
           f"-Wl,-rpath,{lib_dir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles_and_links(tmp_path):
    assert build(tmp_path).exists()


@pytest.mark.gpu
def test_adapter_program_passes(gpu_available, tmp_path):
    exe = build(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASSED" in r.stdout
