"""The C-ABI library loads and exports every symbol include/*.h declares."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    inc = os.path.join(ROOT, "include")
    for fn in sorted(os.listdir(inc)):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(scg_\w+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from solvcon_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIBPATH)
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(_declared()) >= 30


def test_error_reporting_without_gpu():
    from solvcon_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.check(_lib.lib.scg_mesh_create(7, 1, 0, 1, ctypes.byref(
            ctypes.c_void_p())))
    assert "ndim" in _lib.lib.scg_last_error().decode()
    assert _lib.lib.scg_version().decode().startswith("solvcon-gb300")
