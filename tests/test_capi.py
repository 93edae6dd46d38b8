"""The C-ABI library: it builds, loads, and exports every entry point include/hibf_gb300.h and
include/hibf_gb300_diagnostics.h declare.  CPU only: argument validation that happens before any device work is
checked too; nothing here launches a kernel."""

import ctypes
import re
from pathlib import Path

import pytest

from hibf_gb300 import _build, _native as N

INCLUDE = Path(__file__).resolve().parents[1] / "include"
HEADERS = [INCLUDE / "hibf_gb300.h", INCLUDE / "hibf_gb300_diagnostics.h"]


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return N.lib()


def declared():
    text = "".join(h.read_text() for h in HEADERS)
    return sorted(set(re.findall(r"\b(hibf_gpu_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    assert "hibf_gpu_ibf_create" in names and "hibf_gpu_agent_query_batch_d" in names
    assert len(names) >= 35


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(N.declared_symbols()) == set(declared())


def test_abi_version(lib):
    assert lib.hibf_gpu_abi_version() == 1


def test_logic_errors_before_device(lib):
    h = ctypes.c_void_p()
    # interleaved_bloom_filter ctor logic errors (src/interleaved_bloom_filter.cpp:41-46)
    assert lib.hibf_gpu_ibf_create(0, 10, 2, 0, ctypes.byref(h)) == N.ERR_LOGIC
    assert "bins" in N.last_error()
    assert lib.hibf_gpu_ibf_create(8, 10, 0, 0, ctypes.byref(h)) == N.ERR_LOGIC
    assert lib.hibf_gpu_ibf_create(8, 10, 6, 0, ctypes.byref(h)) == N.ERR_LOGIC
    assert lib.hibf_gpu_ibf_create(8, 0, 2, 0, ctypes.byref(h)) == N.ERR_LOGIC
    with pytest.raises(N.LogicError):
        N.call("hibf_gpu_ibf_create", 0, 10, 2, 0, ctypes.byref(h))


def test_hibf_table_validation_before_device(lib):
    import numpy as np

    h = ctypes.c_void_p()
    bins = np.array([2], np.uint64)
    bsz = np.array([64], np.uint64)
    hf = np.array([2], np.uint64)
    nxt = np.array([0, 5], np.uint64)  # merged bin pointing at a missing IBF
    ub = np.array([0, N.BIN_MERGED], np.uint64)
    st = lib.hibf_gpu_hibf_create(1, 1, bins.ctypes.data, bsz.ctypes.data, hf.ctypes.data, nxt.ctypes.data,
                                  ub.ctypes.data, ctypes.byref(h))
    assert st == N.ERR_INVALID_ARG
    ub = np.array([0, 7], np.uint64)  # user bin id beyond n_user_bins
    st = lib.hibf_gpu_hibf_create(1, 1, bins.ctypes.data, bsz.ctypes.data, hf.ctypes.data, nxt.ctypes.data,
                                  ub.ctypes.data, ctypes.byref(h))
    assert st == N.ERR_INVALID_ARG


def test_no_device_is_an_error_not_a_fallback(lib):
    n = ctypes.c_int(-1)
    assert lib.hibf_gpu_device_count(ctypes.byref(n)) == N.OK
    if n.value:
        pytest.skip("a CUDA device is present")
    h = ctypes.c_void_p()
    assert lib.hibf_gpu_ibf_create(64, 1024, 2, 0, ctypes.byref(h)) == N.ERR_NO_DEVICE
    assert not h.value
