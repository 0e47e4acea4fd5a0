"""Drop-in for the reference extension ``ATT_SDDMM_v4`` (prebuilt only; its one
caller is end2end_acc/gat_final/mgat_csr/mgat_conv.py:21-30,110-118,157-165).

Same operators as ATT_SDDMM_v3; v4's caller passes the projected features as
[M, h*F] (not permuted to [h, M, F]) and attention vectors [h, 1, F].  Those
layouts are inferred from that caller (no v4 test exists); outputs are
[h, nnz] as in v3.
"""
from att_gb300.compat.ATT_SDDMM_v3 import (att_tf32_h_nnz, attv2_fp16_h_nnz,  # noqa: F401
                                           attv2_tf32_h_nnz, sddmm_fp16_ones_h_nnz,
                                           sddmm_tf32_ones_h_nnz, sddmm_tf32_h_nnz)
import torch

from att_gb300.compat import _gat_common as _g


def att_fp16_h_nnz(row_pointers, column_index, degrees, window, X, a0, a1, max, nnz):
    return [_g.att(row_pointers, column_index, degrees, window, X, a0, a1, nnz, torch.float16)]


def _hmf(t, H):
    """[h, M, F] view of [h, M, F], [M, h, F] or [M, h*F]."""
    if t.dim() == 2:
        return t.view(t.shape[0], H, -1).permute(1, 0, 2)
    return t if t.shape[0] == H else t.permute(1, 0, 2)


def sddmm_fp16_h_nnz(row_pointers, column_index, degrees, window, A, B, max, nnz):
    """A, B each as [h, M, F], [M, h, F] or [M, h*F]; h from a 3-D operand
    (the smaller of its two leading sizes), else 1."""
    H = 1
    for t in (A, B):
        if t.dim() == 3:
            H = min(t.shape[0], t.shape[1])
    return [_g.sddmm(row_pointers, column_index, degrees, window, _hmf(A, H).half(),
                     _hmf(B, H).half(), nnz, torch.float16, H=H)]
