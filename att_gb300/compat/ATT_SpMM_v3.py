"""Drop-in for the reference extension ``ATT_SpMM_v3`` (prebuilt only in the
reference; meaning pinned by benchmark-v3/spmm-benchmark/test/spmm_{fp16,tf32}/*.py
and the callers end2end_ori/gat_final/mgat_csr/mgat_conv.py:42-59,79-106,126-132).

Y_h = A(vals_h) X_h with the block values gathered from per-edge values
``vals`` [h, nnz] through the slot -> edge map; tensor cores with fp32
accumulation; fp32 outputs.  "_h_m" returns [h, M, F], "_m_h" [M, h, F]; the
row sums return [h, M, 1] / [M, h, 1].  X is [h, M, F] or [M, F].
"""
from att_gb300.compat import _gat_common as _g


def spmm_fp16_h_m(row_pointers, column_index, degrees, vals, window, automic, X):
    """test_spmm_h_m.py:45-66."""
    return [_g.spmm(row_pointers, column_index, degrees, vals, window, automic, X.half(), "h_m")]


def spmm_tf32_h_m(row_pointers, column_index, degrees, vals, window, automic, X):
    return [_g.spmm(row_pointers, column_index, degrees, vals.float(), window, automic,
                    X.float(), "h_m")]


def spmm_fp16_m_h(row_pointers, column_index, degrees, vals, window, automic, X):
    """test_spmm_m_h.py:47-80: input [h, M, F], output [M, h, F]."""
    return [_g.spmm(row_pointers, column_index, degrees, vals, window, automic, X.half(), "m_h")]


def spmm_tf32_m_h(row_pointers, column_index, degrees, vals, window, automic, X):
    return [_g.spmm(row_pointers, column_index, degrees, vals.float(), window, automic,
                    X.float(), "m_h")]


def spmm_fp16_h_m_rowsum(row_pointers, degrees, vals, window, automic, M):
    """test_spmm_h_m_ones.py:45-68: per-row sums, [h, M, 1]."""
    return [_g.rowsum(row_pointers, degrees, vals, window, automic, M, "h_m")]


def spmm_tf32_h_m_rowsum(row_pointers, degrees, vals, window, automic, M):
    return [_g.rowsum(row_pointers, degrees, vals.float(), window, automic, M, "h_m")]


def spmm_fp16_m_h_rowsum(row_pointers, degrees, vals, window, automic, M):
    return [_g.rowsum(row_pointers, degrees, vals, window, automic, M, "m_h")]


def spmm_tf32_m_h_rowsum(row_pointers, degrees, vals, window, automic, M):
    return [_g.rowsum(row_pointers, degrees, vals.float(), window, automic, M, "m_h")]
