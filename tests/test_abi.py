"""The C ABI (CPU only, no compute calls): the in-tree library loads and
exports every entry point include/chimeracl_gb300.h declares, and the Python
binding declares a signature for each."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "chimeracl_gb300.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|const char \*|unsigned long long)\s*(ccl_\w+)\s*\(",
                                 src)))


def test_header_declares_entry_points():
    names = declared()
    assert len(names) >= 30
    assert "ccl_index_sort" in names and "ccl_dht_gemm" in names


def test_library_exports_every_declared_symbol():
    from chimeracl_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = _lib.load()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.ccl_version() == 100


def test_binding_covers_every_compute_entry_point():
    from chimeracl_gb300 import _lib
    compute = [n for n in declared()
               if n not in ("ccl_version", "ccl_last_error", "ccl_launch_count")]
    assert sorted(set(compute) - set(_lib.SIGNATURES)) == []


def test_invalid_arguments_rejected_without_launch():
    """Argument checks run before any launch, so they work without a GPU."""
    from chimeracl_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    assert lib.ccl_push_x(7, 10, None, None, None, None, None, None, None, 0.1, None) == 1
    assert b"dtype" in lib.ccl_last_error()
    assert lib.ccl_push_x(0, 10, None, None, None, None, None, None, None, 0.1, None) == 1
    assert b"NULL" in lib.ccl_last_error()
    assert lib.ccl_push_x(0, 0, None, None, None, None, None, None, None, 0.1, None) == 0
    assert lib.ccl_deposit_scalar(0, 9, None, None, None, None, None, None, -1, 64, 0.0, 1.0, 16,
                                  0.0, 1.0, None, None) == 3
    # the fused push + sort keys: dtype, grid, low parts all or none, NULLs
    args = [None] * 10 + [0.1, 64, 0.0, 1.0, 16, 0.0, 1.0, None, None, None, 0, None]
    assert lib.ccl_push_x_keys(7, 10, *args) == 1 and b"dtype" in lib.ccl_last_error()
    bad_grid = args[:11] + [2] + args[12:]
    assert lib.ccl_push_x_keys(0, 10, *bad_grid) == 1 and b"grid" in lib.ccl_last_error()
    one_lo = args[:3] + [8] + args[4:18] + [8, 8] + args[20:]
    assert lib.ccl_push_x_keys(0, 10, *one_lo) == 1 and b"low parts" in lib.ccl_last_error()
    assert lib.ccl_push_x_keys(0, 10, *args) == 1 and b"NULL" in lib.ccl_last_error()
    assert lib.ccl_index_sort_keyed(10, 64, 2, None, None, None, None, None, None, 0, None) == 1
    assert b"grid" in lib.ccl_last_error()
    assert lib.ccl_index_sort_keyed(-1, 64, 16, None, None, None, None, None, None, 0, None) == 1


def test_sort_wait_probe_arguments_rejected_without_launch():
    """The sort's bounded-wait probe checks its arguments before any CUDA
    call: NULL flag or scratch, a poll count outside [1, 2^20], a scratch
    not 8-byte aligned."""
    from chimeracl_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("library not built")
    lib = _lib.load()
    assert lib.ccl_scan_wait_probe(100, 0, None, 8, None) == 1
    assert b"NULL" in lib.ccl_last_error()
    assert lib.ccl_scan_wait_probe(100, 0, 8, None, None) == 1
    assert lib.ccl_scan_wait_probe(0, 0, 8, 8, None) == 1
    assert b"spins" in lib.ccl_last_error()
    assert lib.ccl_scan_wait_probe((1 << 20) + 1, 0, 8, 8, None) == 1
    assert lib.ccl_scan_wait_probe(100, 0, 8, 12, None) == 1
    assert b"aligned" in lib.ccl_last_error()
