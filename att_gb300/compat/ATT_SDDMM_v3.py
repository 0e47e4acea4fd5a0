"""Drop-in for the reference extension ``ATT_SDDMM_v3`` (prebuilt only in the
reference; meaning pinned by benchmark-v3/sddmm-benchmark/test/sddmm_{fp16,tf32}/*.py
and the callers end2end_ori/gat_final/mgat_csr/mgat_conv.py:21-30,109-117,142-149).

All functions take the GAT format of ``ATT_Block*`` (row_pointers,
column_index, degrees = slot -> edge map, window), return ``[out]`` with out
of shape [h, nnz] in CSR edge order (fp16 for *_fp16_*, fp32 for *_tf32_*),
and ignore ``max`` (a launch-size hint of the reference kernels).
Operands are [h, M, F] or [M, F] (one head).
"""
import torch

from att_gb300.compat import _gat_common as _g


def sddmm_fp16_h_nnz(row_pointers, column_index, degrees, window, A, B, max, nnz):
    """out[h][e(i,j)] = A[h][i] . B[h][j]  (test_sddmm_fp16.py:62-69)."""
    return [_g.sddmm(row_pointers, column_index, degrees, window, A.half(), B.half(), nnz,
                     torch.float16)]


def sddmm_tf32_h_nnz(row_pointers, column_index, degrees, window, A, B, max, nnz):
    return [_g.sddmm(row_pointers, column_index, degrees, window, A.float(), B.float(), nnz,
                     torch.float32)]


def att_fp16_h_nnz(row_pointers, column_index, degrees, window, X, a0, a1, max, nnz):
    """out[h][e(i,j)] = X[h][i].a0[h] + X[h][j].a1[h]  (test_sddmm_fp16_att.py)."""
    return [_g.att(row_pointers, column_index, degrees, window, X, a0, a1, nnz, torch.float16)]


def att_tf32_h_nnz(row_pointers, column_index, degrees, window, X, a0, a1, max, nnz):
    return [_g.att(row_pointers, column_index, degrees, window, X, a0, a1, nnz, torch.float32)]


def attv2_fp16_h_nnz(row_pointers, column_index, degrees, window, X0, X1, a, max, nnz):
    """out[h][e(i,j)] = X0[h][i].a[h] + X1[h][j].a[h]  (test_sddmm_fp16_att_v2.py:70-77)."""
    return [_g.attv2(row_pointers, column_index, degrees, window, X0, X1, a, nnz, torch.float16)]


def attv2_tf32_h_nnz(row_pointers, column_index, degrees, window, X0, X1, a, max, nnz):
    return [_g.attv2(row_pointers, column_index, degrees, window, X0, X1, a, nnz, torch.float32)]


def sddmm_fp16_ones_h_nnz(row_pointers, column_index, degrees, window, g, max, nnz):
    """out[h][e(i,.)] = g[i][h]; g [M, h, 1]  (test_sddmm_fp16_ones.py:62-68)."""
    return [_g.ones(row_pointers, column_index, degrees, window, g, nnz, torch.float16)]


def sddmm_tf32_ones_h_nnz(row_pointers, column_index, degrees, window, g, max, nnz):
    return [_g.ones(row_pointers, column_index, degrees, window, g, nnz, torch.float32)]
