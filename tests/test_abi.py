"""The C ABI library: builds, loads and exports every entry point declared in
include/*.h (no GPU calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wg_gpu.h")
MLP_HEADER = os.path.join(ROOT, "include", "wg_mlp.h")
PATTERN = r"^\s*(?:wg_status|int32_t|int64_t|void|const char \*)\s*(wg_\w+)\s*\("


def declared_symbols(header=HEADER):
    text = open(header).read()
    return sorted(set(re.findall(PATTERN, text, re.M)))


@pytest.fixture(scope="module")
def lib():
    from watergap2_gb300 import build, gpu
    if not os.path.exists(gpu.LIB_PATH):
        build.build()
    return ctypes.CDLL(gpu.LIB_PATH)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "wg_create" in syms and "wg_run_days" in syms and len(syms) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() + declared_symbols(MLP_HEADER) if not hasattr(lib, s)]
    assert not missing, missing


def test_mlp_header_declares_its_entry_points():
    syms = declared_symbols(MLP_HEADER)
    assert {"wg_mlp_create", "wg_mlp_forward", "wg_mlp_gradient", "wg_mlp_train"} <= set(syms)


def test_python_binding_covers_header():
    from watergap2_gb300 import gpu
    assert set(declared_symbols()) <= set(gpu.SYMBOLS) | {"wg_status_string"}


def test_status_strings(lib):
    lib.wg_status_string.restype = ctypes.c_char_p
    assert lib.wg_status_string(0) == b"ok"
    assert lib.wg_status_string(6) == b"device wait exceeded its limit"


def test_create_rejects_null_arguments(lib):
    lib.wg_create.restype = ctypes.c_int
    assert lib.wg_create(None, None, None) == 1   # WG_ERR_INVALID, before touching a device
