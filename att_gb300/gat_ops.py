"""Torch-level GAT operators over the C ABI (att_node_scores, att_slot_edges,
att_sddmm, att_gather_slot_values, att_rowsum, att_spmm).

They work on the GAT block format: the row-window structure of the
conversion plus a slot -> CSR-edge map.  The map handed to these functions is
in the *quad layout*: slot (window row r, condensed column g) at
``(g - g % 4) * W + r * 4 + g % 4`` -- 4-column sub-blocks whatever the
padding width of the format.  The layout of the reference's GAT map is not
recoverable (its source is absent); a fixed sub-block width lets every op read
any (W, wide, partSize) format without being told ``wide``, which the
reference's op signatures do not carry.

Edge-valued tensors are [H, nnz] (stride_h, stride_e = nnz, 1) or [nnz, H]
(1, H); node-valued tensors [H, M, F] or [M, H, F]; all as strided views.
"""
import torch

from . import _lib
from .ops import _DT, _p, _stream, require_cuda

QUAD = 4


def map_to_quad(map_std, window, wide):
    """Permute a slot map from the block-width-``wide`` layout to the quad layout."""
    if wide == QUAD or map_std is None or map_std.numel() == 0:
        return map_std
    n = map_std.numel()
    s = torch.arange(n, device=map_std.device, dtype=torch.int64)
    blk, inb = s // (window * QUAD), s % (window * QUAD)
    r, g = inb // QUAD, blk * QUAD + inb % QUAD
    src = (g - g % wide) * window + r * wide + g % wide
    return map_std[src].contiguous()


def _pad_last(x, mult):
    F = x.shape[-1]
    Fp = (F + mult - 1) // mult * mult
    if Fp == F:
        return x, F
    return torch.nn.functional.pad(x, (0, Fp - F)), F


def node_scores(X3, a2):
    """s[h][m] = X3[h, m, :] . a2[h, :] in fp32; X3 [H, M, F] view, a2 [H, F] view."""
    require_cuda()
    H, M, F = X3.shape
    if X3.stride(2) != 1:
        X3 = X3.contiguous()
    if a2.stride(-1) != 1:
        a2 = a2.contiguous()
    s = torch.empty(H, M, dtype=torch.float32, device=X3.device)
    _lib.call("att_node_scores", _p(X3), _DT[X3.dtype], H, M, F, X3.stride(0), X3.stride(1),
              _p(a2), _DT[a2.dtype], a2.stride(0), _p(s), s.stride(0), _stream())
    return s


def node_scores_pair(X3, a0, a1):
    """(s0, s1) with s0[h][m] = X3[h, m, :] . a0[h, :] and s1 likewise, fp32,
    in one pass over X3 [H, M, F]; a0 / a1 [H, F] (used as fp32)."""
    require_cuda()
    H, M, F = X3.shape
    if X3.stride(2) != 1:
        X3 = X3.contiguous()
    a0 = a0.float().contiguous()
    a1 = a1.float().contiguous()
    s = torch.empty(2, H, M, dtype=torch.float32, device=X3.device)
    _lib.call("att_node_scores_pair", _p(X3), _DT[X3.dtype], H, M, F, X3.stride(0), X3.stride(1),
              _p(a0), _p(a1), a0.stride(0), _p(s[0]), _p(s[1]), s.stride(1), _stream())
    return s[0], s[1]


def _edge_out(H, nnz, dtype, device, layout):
    if layout == "h_e":
        out = torch.zeros(H, nnz, dtype=dtype, device=device)
        return out, out.stride(0), out.stride(1)
    out = torch.zeros(nnz, H, dtype=dtype, device=device)
    return out, out.stride(1), out.stride(0)


def slot_scores(rowptr, col, qmap, win, window, s0, s1, n_nodes, nnz, out_dtype,
                layout="h_e"):
    """out[h][e(i,j)] = s0[h][i] + s1[h][j] for every edge a slot holds."""
    require_cuda()
    H = s0.shape[0]
    out, osh, ose = _edge_out(H, nnz, out_dtype, rowptr.device, layout)
    _lib.call("att_slot_edges", _p(rowptr), _p(col), _p(qmap), _p(win), int(win.numel()),
              window, QUAD, 0, _p(s0), _p(s1), s0.stride(0), None, _lib.NONE, 0, 0, n_nodes, H,
              _p(out), _DT[out_dtype], osh, ose, _stream())
    return out


def slot_rows(rowptr, col, qmap, win, window, g, g_stride_h, g_stride_n, H, n_nodes, nnz,
              out_dtype, layout="h_e"):
    """out[h][e(i,.)] = g[h][i] (row broadcast)."""
    require_cuda()
    out, osh, ose = _edge_out(H, nnz, out_dtype, rowptr.device, layout)
    _lib.call("att_slot_edges", _p(rowptr), _p(col), _p(qmap), _p(win), int(win.numel()),
              window, QUAD, 1, None, None, 0, _p(g), _DT[g.dtype], g_stride_h, g_stride_n,
              n_nodes, H, _p(out), _DT[out_dtype], osh, ose, _stream())
    return out


def sddmm(rowptr, col, qmap, win, window, A3, B3, nnz, out_dtype, layout="h_e"):
    """out[h][e(i,j)] = A3[h, i, :] . B3[h, j, :] on tensor cores."""
    require_cuda()
    H, _, F = A3.shape
    dt = A3.dtype
    if B3.dtype != dt:
        raise TypeError("SDDMM operands must share a dtype")
    mult = 8 if dt in (torch.float16, torch.bfloat16) else 4
    limit = 256 if mult == 8 else 128
    A3, _ = _pad_last(A3.contiguous(), mult)
    B3, _ = _pad_last(B3.contiguous(), mult)
    Fp = A3.shape[-1]
    chunks = [(k, min(k + limit, Fp)) for k in range(0, Fp, limit)]
    direct = len(chunks) == 1
    acc_dtype = out_dtype if direct else torch.float32
    total = None
    for (k0, k1) in chunks:
        a = A3[:, :, k0:k1]
        b = B3[:, :, k0:k1]
        if not direct:
            a, b = a.contiguous(), b.contiguous()
        out, osh, ose = _edge_out(H, nnz, acc_dtype, rowptr.device, layout)
        _lib.call("att_sddmm", _p(rowptr), _p(col), _p(qmap), _p(win), int(win.numel()), window,
                  QUAD, _p(a), _p(b), _DT[dt], H, k1 - k0, a.stride(0), a.stride(1),
                  a.shape[1], b.stride(0), b.stride(1), b.shape[1], _p(out), _DT[acc_dtype],
                  osh, ose, None, _stream())
        total = out if total is None else total + out
    return total if direct else total.to(out_dtype)


def gather_slot_values(qmap, window, out_wide, vals, v_stride_h, v_stride_e, H, dtype):
    n_slots = qmap.numel()
    V = torch.empty(H, n_slots, dtype=dtype, device=qmap.device)
    _lib.call("att_gather_slot_values", _p(qmap), n_slots, window, QUAD, out_wide, _p(vals),
              _DT[vals.dtype], v_stride_h, v_stride_e, H, _p(V), _DT[dtype], V.stride(0),
              _stream())
    return V


def edge_view(vals, H, nnz):
    """(tensor, stride_h, stride_e) of an [H, nnz] / [nnz, H] / [nnz] edge tensor."""
    if vals.dim() == 1:
        return vals.contiguous(), 0, 1
    if vals.shape[0] == H and vals.shape[1] == nnz:
        return vals, vals.stride(0), vals.stride(1)
    if vals.shape[0] == nnz and vals.shape[1] == H:
        return vals, vals.stride(1), vals.stride(0)
    raise ValueError("edge values of shape %s do not match H=%d, nnz=%d" % (tuple(vals.shape), H, nnz))


_ALIGN_CACHE = {}


def parts_aligned(rowptr, mult):
    """True if every part of the format starts and ends on a multiple of
    ``mult`` condensed columns (cached per rowptr tensor version)."""
    key = (rowptr.data_ptr(), rowptr.numel(), rowptr._version, mult)
    hit = _ALIGN_CACHE.get(key)
    if hit is None:
        hit = bool((rowptr[0::2] % mult == 0).all().item())
        if len(_ALIGN_CACHE) > 256:
            _ALIGN_CACHE.clear()
        _ALIGN_CACHE[key] = hit
    return hit


def spmm_edge(rowptr, col, qmap, win, atomic, window, vals, v_stride_h, v_stride_e, X3, m_out,
              out_layout="h_m"):
    """Y_h = A(vals_h) X3[h] for every head; X3 [H, M, F] view.
    out_layout "h_m" -> [H, m_out, F], "m_h" -> [m_out, H, F]; fp32.
    16-bit features need 8-column-aligned parts (formats of wide 8 or 16);
    on a 4-wide format they run through the fp32 (3xTF32) kernel."""
    require_cuda()
    from . import ops
    H, _, F = X3.shape
    dt = X3.dtype
    if dt in (torch.float16, torch.bfloat16) and not parts_aligned(rowptr, 8):
        X3 = X3.float()
        dt = torch.float32
    mult = 8 if dt in (torch.float16, torch.bfloat16) else 4
    out_wide = 8 if mult == 8 else QUAD
    Xp, F0 = _pad_last(X3, mult)
    if Xp.stride(2) != 1 or Xp.stride(1) % mult or Xp.stride(0) % mult:
        Xp = Xp.contiguous()
    Fp = Xp.shape[-1]
    if out_layout == "h_m":
        Y = torch.empty(H, m_out, Fp, dtype=torch.float32, device=X3.device)
    else:
        Y = torch.empty(m_out, H, Fp, dtype=torch.float32, device=X3.device)
    vdt = dt if mult == 8 else torch.float32
    V = gather_slot_values(qmap, window, out_wide, vals, v_stride_h, v_stride_e, H, vdt)
    for h in range(H):
        x = Xp[h]
        y = Y[h] if out_layout == "h_m" else Y[:, h, :]
        ops.spmm(rowptr, col, V[h], win, atomic, x, m_out, window=window, wide=out_wide, out=y)
    if Fp != F0:
        Y = Y[..., :F0].contiguous()
    return Y


def rowsum(rowptr, qmap, win, atomic, window, vals, v_stride_h, v_stride_e, H, m_out,
           out_layout="h_m"):
    """out[h][i] = sum of vals[h][e] over the edges of row i; [H, m_out, 1] or [m_out, H, 1]."""
    require_cuda()
    if out_layout == "h_m":
        out = torch.empty(H, m_out, 1, dtype=torch.float32, device=rowptr.device)
        osh, osn = out.stride(0), out.stride(1)
    else:
        out = torch.empty(m_out, H, 1, dtype=torch.float32, device=rowptr.device)
        osh, osn = out.stride(1), out.stride(0)
    _lib.call("att_rowsum", _p(rowptr), _p(qmap), _p(win), _p(atomic), int(win.numel()), window,
              QUAD, _p(vals), _DT[vals.dtype], v_stride_h, v_stride_e, H, _p(out), osh, osn,
              m_out, _stream())
    return out
