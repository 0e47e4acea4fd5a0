"""The C-ABI library: builds, loads, exports every symbol include/att_gb300.h
declares, and rejects bad arguments with a status (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "att_gb300.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"ATT_API\s+[\w\s\*]*?\b(att_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from att_gb300 import builder, _lib
    builder.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = _declared()
    assert "att_spmm" in names and "att_block_plan" in names and "att_block_fill" in names


def test_library_exports_every_declared_symbol(lib):
    for name in _declared():
        assert hasattr(lib, name), name


def test_binding_covers_header():
    from att_gb300 import _lib
    assert set(_lib.declared_symbols()) == set(_declared())


def test_invalid_arguments_return_status(lib):
    from att_gb300 import _lib
    n_parts = ctypes.c_int64(0)
    n_cond = ctypes.c_int64(0)
    st = lib.att_block_plan(None, None, 4, 0, 4, 0, 8, 32, 0, None, 0,
                            ctypes.byref(n_parts), ctypes.byref(n_cond), None)
    assert st == 1  # ATT_ERR_INVALID
    assert b"rowptr" in lib.att_last_error() or b"window" in lib.att_last_error()
    st = lib.att_spmm(None, None, None, 1, None, None, 4, None, 1, None, 4, 64, 64, None, 8, 64,
                      12, 8, None, None)
    assert st == 4  # window 12 unsupported
    assert lib.att_status_string(4) == b"unsupported combination"


def test_workspace_query_is_host_only(lib):
    from att_gb300 import ops
    b = ops.block_workspace_bytes(1000, 5000, 1000, 8)
    assert b >= 5000 * 4


def test_ops_refuse_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("CUDA present")
    from att_gb300 import ops
    with pytest.raises(RuntimeError):
        ops.require_cuda()


def test_thread_option_overrides_only_the_calling_thread(lib):
    """att_set_thread_option changes the launch shape of the calling thread's
    calls only; -1 returns it to the process-wide default."""
    import threading
    from att_gb300 import autotune
    v = ctypes.c_int()
    assert lib.att_get_option(b"spmm_stages", ctypes.byref(v)) == 0
    default = v.value
    other = 2 if default != 2 else 4
    seen = {}

    def worker():
        assert lib.att_set_thread_option(b"spmm_stages", other) == 0
        w = ctypes.c_int()
        lib.att_get_option(b"spmm_stages", ctypes.byref(w))
        seen["worker"] = w.value
        seen["main_during"] = None
        ev_set.set()
        ev_done.wait(5)

    ev_set, ev_done = threading.Event(), threading.Event()
    t = threading.Thread(target=worker)
    t.start()
    ev_set.wait(5)
    lib.att_get_option(b"spmm_stages", ctypes.byref(v))
    assert v.value == default and seen["worker"] == other
    ev_done.set()
    t.join()
    autotune.apply_shape(("spmm", 128, other))
    lib.att_get_option(b"spmm_fc", ctypes.byref(v))
    assert v.value == 128
    autotune.clear_shape()
    lib.att_get_option(b"spmm_stages", ctypes.byref(v))
    assert v.value == default
    assert lib.att_set_thread_option(b"spmm_stages", 7) == 1  # invalid value refused
