"""Shared implementation of the ATT_Block* / ATT_SDDMM_v* / ATT_SpMM_v* drop-ins.

Formats come from ``ATT_Block*.blockProcess_sddmm_balance_gnn[_trans]``:
``[row_pointers, column_index, degrees(map), (degrees_trans,) window, automic]``
with the slot -> edge maps in the quad layout (4-column sub-blocks; see
att_gb300.gat_ops).  Every reference caller uses 8-row windows
(end2end_*/**/mdataset_*.py), so the window defaults to 8.
"""
import torch

from att_gb300 import gat_ops, ops

WINDOW = 8


def convert(row, col, window, wide, partSize, trans, device=None):
    fmt = ops.block_convert(row, col, None, window=int(window), wide=int(wide),
                            part=int(partSize), emit_empty=False, want_val=False, want_map=True,
                            want_trans=bool(trans))
    qmap = gat_ops.map_to_quad(fmt.map, int(window), int(wide))
    res = [fmt.rowptr, fmt.col, qmap]
    if trans:
        res.append(gat_ops.map_to_quad(fmt.map_t, int(window), int(wide)))
    res += [fmt.window_of_part, fmt.atomic]
    if device is not None and torch.device(device).type == "cuda":
        return res
    return [t.cpu() for t in res]


def _cuda(*ts):
    for t in ts:
        if isinstance(t, torch.Tensor) and t.device.type != "cuda":
            raise TypeError("inputs must be CUDA tensors")


def _as_hmf(X, H=None):
    """[h, M, F] view of X given as [h, M, F], [M, F] (one head) or [M, h*F]."""
    if X.dim() == 3:
        return X
    if H is None or H == 1:
        return X.unsqueeze(0)
    M = X.shape[0]
    return X.view(M, H, -1).permute(1, 0, 2)


def _as_hf(a, H):
    """[h, F] view of an attention vector given as [h, 1, F], [1, F] or [F]."""
    if a.dim() == 3:
        return a.reshape(a.shape[0], a.shape[2])
    if a.dim() == 1:
        return a.unsqueeze(0)
    return a


def att(rowptr, col, qmap, window_t, X, a0, a1, nnz, out_dtype, x_layout="auto",
        out_layout="h_e"):
    _cuda(rowptr, col, qmap, window_t, X, a0, a1)
    H = a0.shape[0] if a0.dim() == 3 else 1
    X3 = _as_hmf(X, H)
    s0 = gat_ops.node_scores(X3, _as_hf(a0, H).to(X3.dtype))
    s1 = gat_ops.node_scores(X3, _as_hf(a1, H).to(X3.dtype))
    return gat_ops.slot_scores(rowptr, col, qmap, window_t, WINDOW, s0, s1, X3.shape[1],
                               int(nnz), out_dtype, out_layout)


def attv2(rowptr, col, qmap, window_t, X0, X1, a, nnz, out_dtype, out_layout="h_e"):
    _cuda(rowptr, col, qmap, window_t, X0, X1, a)
    H = a.shape[0] if a.dim() == 3 else 1
    A0, A1 = _as_hmf(X0, H), _as_hmf(X1, H)
    av = _as_hf(a, H).to(A0.dtype)
    s0 = gat_ops.node_scores(A0, av)
    s1 = gat_ops.node_scores(A1, av)
    return gat_ops.slot_scores(rowptr, col, qmap, window_t, WINDOW, s0, s1, A0.shape[1],
                               int(nnz), out_dtype, out_layout)


def sddmm(rowptr, col, qmap, window_t, A, B, nnz, out_dtype, H=None, out_layout="h_e"):
    _cuda(rowptr, col, qmap, window_t, A, B)
    A3, B3 = _as_hmf(A, H), _as_hmf(B, H)
    return gat_ops.sddmm(rowptr, col, qmap, window_t, WINDOW, A3, B3, int(nnz), out_dtype,
                         out_layout)


def ones(rowptr, col, qmap, window_t, g, nnz, out_dtype, out_layout="h_e"):
    """g given as [M, h, 1] (or [M, h] / [M])."""
    _cuda(rowptr, col, qmap, window_t, g)
    if g.dim() == 1:
        g = g.unsqueeze(1)
    M, H = g.shape[0], g.shape[1]
    return gat_ops.slot_rows(rowptr, col, qmap, window_t, WINDOW, g, g.stride(1), g.stride(0), H,
                             M, int(nnz), out_dtype, out_layout)


def spmm(rowptr, col, qmap, vals, window_t, atomic, X, out_layout, H=None):
    _cuda(rowptr, col, qmap, vals, window_t, atomic, X)
    if H is None:
        H = 1 if vals.dim() == 1 else (vals.shape[0] if X.dim() != 3 else X.shape[0])
    X3 = _as_hmf(X, H)
    nnz = vals.shape[-1] if vals.dim() == 1 or vals.shape[0] == H else vals.shape[0]
    v, sh, se = gat_ops.edge_view(vals, H, nnz)
    if v.dtype != X3.dtype:
        v = v.to(X3.dtype)
        v, sh, se = gat_ops.edge_view(v, H, nnz)
    return gat_ops.spmm_edge(rowptr, col, qmap, window_t, atomic, WINDOW, v, sh, se, X3,
                             X3.shape[1], out_layout)


def rowsum(rowptr, qmap, vals, window_t, atomic, M, out_layout, H=None):
    _cuda(rowptr, qmap, vals, window_t, atomic)
    if H is None:
        H = 1 if vals.dim() == 1 else vals.shape[0]
    nnz = vals.shape[-1] if vals.dim() == 1 or vals.shape[0] == H else vals.shape[0]
    v, sh, se = gat_ops.edge_view(vals, H, nnz)
    return gat_ops.rowsum(rowptr, qmap, window_t, atomic, WINDOW, v, sh, se, H, int(M),
                          out_layout)
