"""The product path has no CPU fallback: the package imports nothing from the
oracle, and a missing library is an error, not a quieter path (CPU only)."""
import ast
import os

import pytest

from pixels_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pixels_gb300")


def package_sources():
    for d, _, files in os.walk(PKG):
        for f in files:
            if f.endswith(".py"):
                yield os.path.join(d, f)


def imported_modules(path):
    tree = ast.parse(open(path).read(), path)
    for node in ast.walk(tree):
        if isinstance(node, ast.Import):
            for a in node.names:
                yield a.name
        elif isinstance(node, ast.ImportFrom) and node.level == 0 and node.module:
            yield node.module


def test_package_imports_nothing_from_the_oracle():
    oracle_modules = {f[:-3] for f in os.listdir(os.path.join(ROOT, "oracle")) if f.endswith(".py")}
    oracle_modules.add("oracle")
    sources = list(package_sources())
    assert len(sources) >= 5
    for path in sources:
        for mod in imported_modules(path):
            assert mod.split(".")[0] not in oracle_modules, f"{path} imports {mod}"


def test_missing_library_raises(tmp_path):
    saved = _lib._L
    _lib._L = None
    try:
        with pytest.raises(RuntimeError, match="missing"):
            _lib.load(str(tmp_path / "libpixels_gb300.so"))
    finally:
        _lib._L = saved
