"""The allocation-free conversion entry point, called through the C ABI.

Some callers cannot allocate device memory: hosts that hand out device memory
only from their own arena or budget, and latency-critical callers that cannot
afford cudaMalloc/cudaFree.  att_block_convert_noalloc serves them with a
scratch array the library owns.  This test calls it twice in a row on
different graphs (so the second call runs on scratch left over from the
first) and checks each result bit-for-bit -- the tolerance every conversion
test here uses -- against the regular entry points (att_block_plan +
att_block_fill with a caller workspace).  It also checks that a graph too
large for the fixed scratch is refused with a clear error.

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(rowptr, col, deg, window, wide, part, emit_empty, n_cols, cap_parts, cap_cond):
    from att_gb300 import _lib
    lib = _lib.lib()
    n_rows = rowptr.shape[0] - 1
    nnz = col.shape[0]
    dev = rowptr.device
    out = {
        "rowptr": torch.full((2 * cap_parts + 1,), -7, dtype=torch.int32, device=dev),
        "col": torch.full((cap_cond,), -7, dtype=torch.int32, device=dev),
        "val": torch.full((cap_cond * window,), 7.0, dtype=deg.dtype, device=dev),
        "map": torch.full((cap_cond * window,), -7, dtype=torch.int32, device=dev),
        "window": torch.full((cap_parts,), -7, dtype=torch.int32, device=dev),
        "atomic": torch.full((cap_parts,), -7, dtype=torch.int32, device=dev),
    }
    n_parts = ctypes.c_int64(0)
    n_cond = ctypes.c_int64(0)
    dt = _lib.F16 if deg.dtype == torch.float16 else _lib.F32
    st = lib.att_block_convert_noalloc(
        rowptr.data_ptr(), col.data_ptr(), n_rows, nnz, n_cols, window, wide, part,
        int(emit_empty), deg.data_ptr(), dt, out["rowptr"].data_ptr(), out["col"].data_ptr(),
        out["val"].data_ptr(), dt, out["map"].data_ptr(), None, None, out["window"].data_ptr(),
        out["atomic"].data_ptr(), cap_parts, cap_cond, ctypes.byref(n_parts),
        ctypes.byref(n_cond), torch.cuda.current_stream().cuda_stream)
    return st, n_parts.value, n_cond.value, out


def _check_against_workspace_path(rowptr, col, deg, window, wide, part, emit_empty):
    from att_gb300 import ops
    n_cols = int(deg.shape[0])
    ref = ops.block_convert(rowptr, col, deg, window=window, wide=wide, part=part,
                            emit_empty=emit_empty, want_map=True, n_cols=n_cols)
    cap_p, cap_c = ref.n_parts + 5, ref.n_condensed + 16
    st, P, NC, out = _noalloc(rowptr, col, deg, window, wide, part, emit_empty, n_cols, cap_p,
                              cap_c)
    torch.cuda.synchronize()
    assert st == 0, _lastmsg()
    assert (P, NC) == (ref.n_parts, ref.n_condensed)
    bits = torch.int16 if deg.dtype == torch.float16 else torch.int32
    assert torch.equal(out["rowptr"][: 2 * P + 1], ref.rowptr)
    assert torch.equal(out["col"][:NC], ref.col)
    assert torch.equal(out["window"][:P], ref.window_of_part)
    assert torch.equal(out["atomic"][:P], ref.atomic)
    assert torch.equal(out["map"][: NC * window], ref.map)
    assert torch.equal(out["val"][: NC * window].view(bits), ref.val.view(bits))


def _lastmsg():
    from att_gb300 import _lib
    return _lib.lib().att_last_error().decode()


def test_noalloc_matches_workspace_path_two_calls(cuda):
    from att_gb300 import graphs
    # first call: a power-law graph with hub windows (bitmap path, split parts)
    rp, col = graphs.chung_lu(20000, 12, 2.1, seed=5)
    rp = graphs.pad_rows(rp, 8).cuda()
    col = col.cuda()
    deg = graphs.gcn_degree(rp, torch.float16)
    deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg))
    _check_against_workspace_path(rp, col, deg, 8, 8, 32, False)
    # second call in a row: a smaller graph, fp32 values, other shape; runs on
    # the scratch the first call left behind
    rp2, col2 = graphs.random_csr(999, 999, 14, seed=8, hub_rows=2, hub_len=900, empty_frac=0.2)
    rp2 = torch.from_numpy(rp2).cuda()
    col2 = torch.from_numpy(col2).cuda()
    deg2 = torch.rand(999, device="cuda", dtype=torch.float32) + 0.1
    _check_against_workspace_path(rp2, col2, deg2, 16, 4, 3, True)


def test_noalloc_rejects_graph_beyond_scratch(cuda):
    from att_gb300 import _lib
    lib = _lib.lib()
    cap = lib.att_block_convert_noalloc_max_scratch()
    assert cap == 64 << 20
    n_rows = 1 << 20
    nnz = cap // 4 + 1  # the sorted-column scratch alone is 4 bytes per edge
    n_parts = ctypes.c_int64(0)
    n_cond = ctypes.c_int64(0)
    dummy = torch.zeros(8, dtype=torch.int32, device="cuda")
    st = lib.att_block_convert_noalloc(
        dummy.data_ptr(), dummy.data_ptr(), n_rows, nnz, n_rows, 8, 8, 32, 0, None, _lib.NONE,
        dummy.data_ptr(), dummy.data_ptr(), None, _lib.NONE, None, None, None, dummy.data_ptr(),
        dummy.data_ptr(), 1, 1, ctypes.byref(n_parts), ctypes.byref(n_cond), None)
    assert st == 3  # ATT_ERR_WORKSPACE, refused before any GPU work
    assert "scratch" in _lastmsg()


def test_noalloc_reports_small_outputs(cuda):
    from tests._fixture import ROW, COL
    rp = torch.from_numpy(ROW).cuda()
    col = torch.from_numpy(COL).cuda()
    deg = torch.ones(32, dtype=torch.float16, device="cuda")
    st, P, NC, _ = _noalloc(rp, col, deg, 8, 8, 1, False, 32, 2, 64)
    assert st == 3 and P == 6 and NC == 48
