"""The C-ABI library loads on a machine without a GPU and exports every entry point
that include/*.h declares; calls that need a device fail with a status code, never abort."""
import ctypes as C
import re
from pathlib import Path

import grid_gb300 as g

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w \*]*?\b(gb_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) > 40
    lib = C.CDLL(str(g.LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_version():
    assert g.lib.gb_version() >= 100
    assert g.lib.gb_status_string(0) == b"ok"
    assert g.lib.gb_status_string(5) == b"not converged"


def test_create_without_device_is_a_status_not_a_crash():
    if g.device_count() > 0:
        return  # covered by the GPU tests
    h = C.c_void_p()
    dims = (C.c_int * 4)(4, 4, 4, 4)
    rc = g.lib.gb_wilson_create(dims, 0.1, None, 0, 1, None, 0, C.byref(h))
    assert rc == 7  # GB_ERR_NO_DEVICE
    assert b"device" in g.lib.gb_last_error()


def test_bad_arguments_are_rejected_before_any_device_call():
    h = C.c_void_p()
    dims = (C.c_int * 4)(4, 3, 4, 4)  # odd extent
    assert g.lib.gb_wilson_create(dims, 0.1, None, 0, 1, None, 0, C.byref(h)) == 1
    dims = (C.c_int * 4)(4, 4, 4, 4)
    assert g.lib.gb_mobius_create(dims, 1, 0.1, 1.8, 1.5, 0.5, None, 0, 1, None, 0, C.byref(h)) == 1  # Ls < 2
    assert g.lib.gb_mobius_create(dims, 16, 0.1, 1.8, 1.5, 0.5, None, 0, 100, None, 0, C.byref(h)) == 8  # L5 too big
    # the fifth dimension must be even (site pairs of the FP32/FP16 layout)
    assert g.lib.gb_mobius_create(dims, 5, 0.1, 1.8, 1.5, 0.5, None, 0, 1, None, 0, C.byref(h)) == 8


def test_header_is_c99_and_a_c_program_links_and_calls(tmp_path):
    """The boundary is a C ABI: the header compiles as strict C99 and a C program links
    the library and calls it (what a ctypes / cgo / JNI binding relies on)."""
    import shutil
    import subprocess

    gcc = shutil.which("gcc")
    if gcc is None:
        import pytest
        pytest.skip("no C compiler")
    src = tmp_path / "use_abi.c"
    src.write_text(
        '#include <stdio.h>\n#include "gbdwf.h"\n'
        'int main(void) {\n'
        '  printf("%d %s %s\\n", gb_version(), gb_status_string(0), gb_status_string(5));\n'
        '  return 0;\n}\n')
    exe = tmp_path / "use_abi"
    lib_dir = Path(g.LIB_PATH).parent
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{ROOT / 'include'}", str(src),
                    "-o", str(exe), f"-L{lib_dir}", "-lgbdwf", f"-Wl,-rpath,{lib_dir}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split(" ", 1)
    assert int(out[0]) == g.lib.gb_version()
    assert out[1].strip() == "ok not converged"
