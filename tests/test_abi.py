"""The C ABI library builds, loads and exports every symbol the header declares
(no GPU needed)."""
import os
import re

from uclchem_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "uclchem_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ucl_\w+)\s*\(", src)))


def test_library_exports_header_symbols():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 12
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= set(names)


def test_build_targets_sm103a_only():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_params_struct_matches_header_layout():
    import ctypes
    from uclchem_gb300.params import DEFAULTS, ModelParams, PARAMS_DTYPE
    lib = _lib.load()
    p = ModelParams()
    lib.ucl_params_default(ctypes.byref(p))
    for k, v in DEFAULTS.items():
        assert getattr(p, k) == v, k
    assert PARAMS_DTYPE.itemsize == ctypes.sizeof(ModelParams)


def test_header_is_plain_c_and_struct_sizes_agree(tmp_path):
    """include/uclchem_gb300.h compiles as C99 (what a Fortran/cgo/FFI host
    sees), and its struct sizes match the Python mirrors."""
    import ctypes
    import shutil
    import subprocess
    import pytest
    from uclchem_gb300.params import ModelParams
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "uclchem_gb300.h"\n'
                   'int main(void) { printf("%zu %zu\\n", sizeof(ucl_model_params), sizeof(ucl_model_stats)); '
                   'return 0; }\n')
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == ctypes.sizeof(ModelParams)
    assert int(out[1]) == ctypes.sizeof(_lib.ModelStats) == _lib.STATS_DTYPE.itemsize
