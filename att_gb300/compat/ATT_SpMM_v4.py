"""Drop-in for the reference extension ``ATT_SpMM_v4`` (prebuilt only; its one
caller is end2end_acc/gat_final/mgat_csr/mgat_conv.py:42-58,80-107,128-138).

Layouts inferred from that caller (no v4 test exists): features [M, h*F];
``spmm_fp16_m_h`` returns [M, h, F]; ``spmm_fp16_m_h2`` takes [M, h, F]
(or [M, h*F]) and returns [M, h*F]; row sums as in v3.  ``bmm_v_m`` and
``bmm_v_v`` are the small batched products of the attention-vector gradients
(plain GEMMs, done with torch.bmm).
"""
import torch

from att_gb300.compat import _gat_common as _g
from att_gb300.compat.ATT_SpMM_v3 import (spmm_fp16_h_m_rowsum, spmm_fp16_m_h_rowsum,  # noqa: F401
                                          spmm_tf32_h_m_rowsum, spmm_tf32_m_h_rowsum)


def _heads(vals, X):
    return vals.shape[0] if vals.dim() == 2 and X.dim() == 2 and X.shape[1] % vals.shape[0] == 0 else None


def spmm_fp16_m_h(row_pointers, column_index, degrees, vals, window, automic, X):
    H = vals.shape[0] if vals.dim() == 2 else 1
    X3 = X.view(X.shape[0], H, -1).permute(1, 0, 2) if X.dim() == 2 else X
    return [_g.spmm(row_pointers, column_index, degrees, vals, window, automic, X3.half(), "m_h",
                    H=H)]


def spmm_fp16_m_h2(row_pointers, column_index, degrees, vals, window, automic, X):
    H = vals.shape[0] if vals.dim() == 2 else 1
    M = X.shape[0]
    X3 = X.reshape(M, H, -1).permute(1, 0, 2)
    Y = _g.spmm(row_pointers, column_index, degrees, vals, window, automic, X3.half(), "m_h",
                H=H)
    return [Y.reshape(M, -1)]


def _col(v):
    """Per-head vectors of node values as [h, M, 1] (accepts [h, M, 1] or
    [h, 1, M]: the caller's comments describe the latter, this package's row
    sums return the former)."""
    return v if v.shape[-1] == 1 else v.transpose(1, 2)


def bmm_v_m(a0_tmp, a1_tmp, X):
    """Attention-vector gradients (mgat_conv.py:82): a*_grad[h, 0, f] =
    sum_m a*_tmp[h, m] X[h, f, m]; a*_tmp [h, M, 1] (or [h, 1, M]), X
    [h, F, M] -> ([h, 1, F], [h, 1, F])."""
    g0 = torch.bmm(X, _col(a0_tmp).to(X.dtype)).transpose(1, 2)
    g1 = torch.bmm(X, _col(a1_tmp).to(X.dtype)).transpose(1, 2)
    return g0, g1


def bmm_v_v(temp_grad, temp_a):
    """Feature gradient (mgat_conv.py:94): out[m, h*F + f] = temp_grad[h, m] *
    temp_a[h, 0, f]; temp_grad [h, M, 1] (or [h, 1, M]), temp_a [h, 1, F] ->
    [M, h*F]."""
    out = torch.bmm(_col(temp_grad).to(temp_a.dtype), temp_a)  # [h, M, F]
    return [out.permute(1, 0, 2).reshape(out.shape[1], -1)]
