"""CPU-side checks of the C ABI library: it builds, loads, and exports every
symbol include/pixels_gb300.h declares (no GPU calls)."""
import ctypes
import os
import re

from pixels_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "pixels_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*)\s+(px_\w+)\s*\(", src, re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    decl = declared_symbols()
    assert len(decl) >= 15
    for name in decl:
        assert hasattr(lib, name), name
    assert sorted(_lib.EXPORTS) == decl


def test_library_refuses_without_device_or_bad_args():
    L = _lib.load()
    h = ctypes.c_void_p()
    # dims must be positive multiples of 8
    assert L.px_world_create(12, 8, 8, 80.0, 16, ctypes.byref(h)) == 1
    assert L.px_last_error(None) == b"null world"
