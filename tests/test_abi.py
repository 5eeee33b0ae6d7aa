"""The C-ABI library loads and exports every entry point include/flowx.h
declares (no GPU needed: nothing is called)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(flowx_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from flowx_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = _declared("flowx.h")
    assert "flowx_create" in names and "flowx_substep" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared("flowx.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_kernel_names_without_gpu(lib):
    lib.flowx_kernel_count.restype = ctypes.c_int
    lib.flowx_kernel_name.restype = ctypes.c_char_p
    n = lib.flowx_kernel_count()
    names = [lib.flowx_kernel_name(i).decode() for i in range(n)]
    assert "lambda" in names and "delta_apply" in names and len(set(names)) == n


def test_python_binding_signatures(lib):
    from flowx_gb300 import _lib

    loaded = _lib.load()
    assert loaded.flowx_substep.argtypes is not None
    assert ctypes.sizeof(_lib.Push) == 128
    assert ctypes.sizeof(_lib.Primitive) == 64


def test_python_flag_values_match_the_header():
    """The flag bits and the warp-pass threshold the Python binding passes are
    the ones include/flowx.h defines."""
    from flowx_gb300 import _lib

    text = open(os.path.join(ROOT, "include", "flowx.h")).read()
    for name in ("KEEP_DELTA", "EXACT", "REFERENCE_ORDER", "WARP_PASSES", "THREAD_PASSES"):
        m = re.search(rf"FLOWX_FLAG_{name}\s*=\s*(\d+)", text)
        assert m and int(m.group(1)) == getattr(_lib, f"FLAG_{name}"), name
    m = re.search(r"#define FLOWX_WARP_PASSES_MAX_PARTICLES\s+(\d+)", text)
    assert m and int(m.group(1)) == _lib.WARP_PASSES_MAX_PARTICLES
