"""The C ABI library loads and exports every function include/*.h declares."""
import ctypes
import os
import re

from yapt_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"YG_API\s+[\w\s\*]+?\b(yg_\w+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(N.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built):
    assert declared_functions() == {s[0] for s in N.SIGNATURES}


def test_errors_are_codes_not_aborts(built):
    lib = N.load()
    assert lib.yg_version() >= 1
    n = ctypes.c_size_t()
    rc = lib.yg_host_table(b"/nonexistent", 0, 380, 700, None, 0, ctypes.byref(n))
    assert rc == -5 and b"cannot open" in lib.yg_last_error()
    rc = lib.yg_host_table(N.DATA_DIR.encode(), 99, 380, 700, None, 0, ctypes.byref(n))
    assert rc == -1
