"""The C-ABI library loads without a GPU and exports every function that
include/gbnuts.h declares (no compute calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbnuts_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    from stan_gb300 import _lib
    lib = _lib.load()
    names = declared_functions("gbnuts.h")
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert missing == []
    # the Python binding declares exactly the exported C ABI
    assert set(names) == set(_lib.SIGNATURES)
    # the test hooks are exported too
    hooks = declared_functions("gbnuts_testing.h")
    assert hooks and [n for n in hooks if not hasattr(lib, n)] == []


def test_library_is_in_tree():
    from stan_gb300 import _lib
    assert _lib.LIB_PATH.startswith(os.path.join(ROOT, "stan_gb300"))
    ctypes.CDLL(_lib.LIB_PATH)


def test_no_cpu_fallback_in_package():
    """The product never imports the oracle."""
    pkg = os.path.join(ROOT, "stan_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith(".py"):
                src = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in src and "from oracle" not in src, f
