"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/xnb_gpu.h and include/xnb_dump.h (no compute calls: no GPU
needed)."""
import ctypes
import os
import re

import pytest

from exanbody_gb300 import build, dump, xnb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(xnb_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_header_symbols():
    lib_path = build.build()
    lib = ctypes.CDLL(lib_path)
    names = declared("xnb_gpu.h")
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(xnb.EXPORTED) | set(names)


def test_binding_covers_header():
    assert set(declared("xnb_gpu.h")) == set(xnb.EXPORTED)


def test_binding_constants_equal_header_defines():
    """Every XNB_* value the header defines has the same value in the binding
    (xnb.NAME for XNB_NAME); the include guard and XNB_OK (0, checked by _ck)
    are the only defines without a twin."""
    text = open(os.path.join(ROOT, "include", "xnb_gpu.h")).read()
    defines = re.findall(r"^#define\s+XNB_([A-Z0-9_]+)\s+\(?\s*(-?(?:0x[0-9a-fA-F]+|\d+))u?\s*\)?", text, flags=re.M)
    assert len(defines) >= 20
    checked = 0
    for name, value in defines:
        if name == "OK":
            continue
        assert hasattr(xnb, name), "XNB_%s has no binding constant" % name
        assert getattr(xnb, name) == int(value, 0), name
        checked += 1
    assert checked == len(defines) - 1


def test_dump_header_symbols_exported_and_bound():
    lib = ctypes.CDLL(build.build())
    names = declared("xnb_dump.h")
    assert set(names) == set(dump.EXPORTED)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string_without_gpu():
    lib = xnb.load()
    assert lib.xnb_version() >= 10000
    assert isinstance(lib.xnb_last_error_string(), bytes)


def test_system_bytes_is_monotone():
    lib = xnb.load()
    a = lib.xnb_system_bytes(1000, 100, 80.0)
    b = lib.xnb_system_bytes(2000, 200, 80.0)
    assert 0 < a < b
