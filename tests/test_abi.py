"""The C-ABI library loads and exports every function include/mmcgb.h
declares (no compute calls: this runs without a GPU)."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "mmcgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mmcgb_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from mmc_gb300 import build
    path = build.build_library()
    lib = C.CDLL(path)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_loads_without_gpu():
    from mmc_gb300 import _native
    lib = _native.load()
    assert lib.mmcgb_abi_version() == 6
    for n in _native.EXPORTS:
        getattr(lib, n)
