"""The C-ABI library loads and exports every entry point include/la_gpu.h declares
(no compute call: this runs without a GPU)."""
import os
import re

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            text = open(os.path.join(inc, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(la_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(lagpu):
    lib = lagpu.lib()
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(lagpu):
    names = declared_symbols()
    assert set(lagpu.SIGNATURES) >= {n for n in names if n.startswith("la_")} - set()


def test_abi_version_and_status_strings(lagpu):
    lib = lagpu.lib()
    assert lib.la_abi_version() == 1
    for s in range(9):
        assert lib.la_status_string(s)
