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
