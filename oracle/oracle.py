"""CPU oracle for the ATT sparse hot path.

TEST INFRASTRUCTURE ONLY.  Tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module as the checker; the
``att_gb300`` product path never imports it and has no CPU fallback.

Contents
--------
* ``block_convert`` -- ctypes wrapper over ``block_oracle.c``, the C
  restatement of the reference's row-window block conversion
  (gcn/Block_gcn/example.cpp:48-348) and of the GAT slot->edge maps
  (Block/include/example.h:4-6, consumed as in
  benchmark-v3/sddmm-benchmark/include/output_tile.h:15-37).
* FP64 numpy restatements of the numeric ops, each citing the reference
  call site or test that pins its meaning:
  - GCN SpMM Y = A_hat X          gcn/SpMM/test/mgcn/test_balance.py:8-18
  - SpMM on the block format itself (per part, summed per window)
                                  gcn/SpMM/src/spmmKernel.cu:158-265
  - SDDMM out[h][e(i,j)] = A_h[i].B_h[j]
                                  benchmark-v3/sddmm-benchmark/test/sddmm_fp16/test_sddmm_fp16.py:62-69
  - additive attention X_i.a0 + X_j.a1
                                  benchmark-v3/sddmm-benchmark/test/sddmm_tf32/test_sddmm_tf32_att.py
  - GATv2-style X0_i.a + X1_j.a   benchmark-v3/sddmm-benchmark/test/sddmm_fp16/test_sddmm_fp16_att_v2.py:70-77
  - broadcast out[h][e(i,.)] = g[i][h]
                                  benchmark-v3/sddmm-benchmark/test/sddmm_fp16/test_sddmm_fp16_ones.py:62-68
  - SpMM with per-edge values, row sums
                                  benchmark-v3/spmm-benchmark/test/spmm_fp16/test_spmm_h_m.py:45-66,
                                  test_spmm_h_m_ones.py:45-68
  - GAT layer forward (v1 chain)  end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198
  - GATv2 layer (differentiable)  end2end_head/gatv2_final/mgat_csr/mgat_conv.py:151-196
* Row-sampled FP64 restatements for full-size graphs (sub_csr, sample_rows,
  spmm_rows_fp64, gat_dot_rows_fp64, gat_add_rows_torch) and the 2-layer GCN
  of the serving loop (gcn2_fp64).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
_SRC = os.path.join(HERE, "block_oracle.c")
_lib = None


class _Blocks(ctypes.Structure):
    _fields_ = [
        ("n_parts", ctypes.c_int64),
        ("n_cols", ctypes.c_int64),
        ("rowptr", ctypes.POINTER(ctypes.c_int32)),
        ("col", ctypes.POINTER(ctypes.c_int32)),
        ("val16", ctypes.POINTER(ctypes.c_uint16)),
        ("val32", ctypes.POINTER(ctypes.c_float)),
        ("map", ctypes.POINTER(ctypes.c_int32)),
        ("map_t", ctypes.POINTER(ctypes.c_int32)),
        ("window", ctypes.POINTER(ctypes.c_int32)),
        ("atomic", ctypes.POINTER(ctypes.c_int32)),
    ]


def build(force=False):
    """Compile block_oracle.c with gcc into oracle/_build/liboracle.so."""
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(_SRC):
        tmp = _LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-o", tmp, _SRC])
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        lib.oracle_block_convert.restype = ctypes.c_int
        lib.oracle_block_convert.argtypes = [
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Blocks)]
        lib.oracle_free.argtypes = [ctypes.POINTER(_Blocks)]
        lib.oracle_f32_to_f16.restype = ctypes.c_uint16
        lib.oracle_f32_to_f16.argtypes = [ctypes.c_float]
        _lib = lib
    return _lib


def _arr(ptr, n, dtype):
    if n <= 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(int(n),)).astype(dtype, copy=True)


def block_convert(rowptr, col, deg=None, window=8, wide=8, part=32,
                  emit_empty=False, want_map=False, want_trans=False):
    """Row-window block conversion on the CPU.

    ``deg``: None (no values), a float16 array (fp16 values, as
    ``blockProcess_fp16_balance``) or a float32 array (``_tf32_balance``).
    Returns a dict with ``rowptr, col, val, map, map_t, window, atomic``
    (numpy arrays; ``val`` float16/float32 or None).
    """
    lib = _load()
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    col = np.ascontiguousarray(col, dtype=np.int32)
    n_rows = rowptr.shape[0] - 1
    kind, degp = 0, None
    if deg is not None:
        deg = np.ascontiguousarray(deg)
        if deg.dtype == np.float16:
            kind, deg = 1, deg.view(np.uint16)
        elif deg.dtype == np.float32:
            kind = 2
        else:
            raise TypeError("deg must be float16 or float32")
        degp = deg.ctypes.data
    out = _Blocks()
    rc = lib.oracle_block_convert(rowptr.ctypes.data, col.ctypes.data, n_rows, degp,
                                  kind, window, wide, part, int(emit_empty),
                                  int(want_map), int(want_trans), ctypes.byref(out))
    if rc != 0:
        raise RuntimeError("oracle_block_convert failed: %d" % rc)
    try:
        np_ = out.n_parts
        ns = out.n_cols * window
        res = {
            "rowptr": _arr(out.rowptr, 2 * np_ + 1, np.int32),
            "col": _arr(out.col, out.n_cols, np.int32),
            "window": _arr(out.window, np_, np.int32),
            "atomic": _arr(out.atomic, np_, np.int32),
            "val": None, "map": None, "map_t": None,
        }
        if kind == 1:
            res["val"] = _arr(out.val16, ns, np.uint16).view(np.float16)
        elif kind == 2:
            res["val"] = _arr(out.val32, ns, np.float32)
        if want_map:
            res["map"] = _arr(out.map, ns, np.int32)
        if want_trans:
            res["map_t"] = _arr(out.map_t, ns, np.int32)
        return res
    finally:
        lib.oracle_free(ctypes.byref(out))


def f32_to_f16_bits(x):
    lib = _load()
    return lib.oracle_f32_to_f16(float(x))


# --------------------------------------------------------------------------
# FP64 numeric oracles
# --------------------------------------------------------------------------

def csr_rows(rowptr):
    rowptr = np.asarray(rowptr, dtype=np.int64)
    return np.repeat(np.arange(rowptr.shape[0] - 1, dtype=np.int64), np.diff(rowptr))


def gcn_values(rowptr, col, deg):
    """Per-edge GCN value deg[row]*deg[col] rounded as the block format stores it."""
    rows = csr_rows(rowptr)
    col = np.asarray(col, dtype=np.int64)
    d = np.asarray(deg)
    if d.dtype == np.float16:
        return (d[rows].astype(np.float32) * d[col].astype(np.float32)).astype(np.float16)
    return (d[rows].astype(np.float32) * d[col].astype(np.float32)).astype(np.float32)


def spmm_csr_fp64(rowptr, col, vals, X, n_out=None, dedupe=True):
    """Y = A X in FP64 with A given as CSR; duplicate (row,col) entries count once
    when ``dedupe`` (the block format overwrites duplicates)."""
    import scipy.sparse as sp
    rowptr = np.asarray(rowptr, dtype=np.int64)
    n_rows = rowptr.shape[0] - 1
    X = np.asarray(X, dtype=np.float64)
    rows = csr_rows(rowptr)
    col = np.asarray(col, dtype=np.int64)
    v = np.asarray(vals, dtype=np.float64)
    if dedupe and col.size:
        key = rows * (X.shape[0] + 1) + col
        _, first = np.unique(key[::-1], return_index=True)
        keep = (col.size - 1) - first
        rows, col, v = rows[keep], col[keep], v[keep]
    A = sp.csr_matrix((v, (rows, col)), shape=(n_rows, X.shape[0]))
    Y = A @ X
    if n_out is not None:
        Y = Y[:n_out]
    return np.asarray(Y)


def spmm_blocks_fp64(fmt, X, m_out, window=8, wide=8):
    """Evaluate Y = A X directly from a block format (rowptr pairs, col, val,
    window): each part adds val_block^T-contracted gathered X rows into its
    window's rows; rows not covered stay zero."""
    rp = np.asarray(fmt["rowptr"], dtype=np.int64)
    col = np.asarray(fmt["col"], dtype=np.int64)
    val = np.asarray(fmt["val"], dtype=np.float64)
    win = np.asarray(fmt["window"], dtype=np.int64)
    X = np.asarray(X, dtype=np.float64)
    F = X.shape[1]
    Y = np.zeros((m_out, F), dtype=np.float64)
    for p in range(win.shape[0]):
        s, e_real = rp[2 * p], rp[2 * p + 1]
        for c in range(s, e_real):
            j = col[c]
            if j < 0:
                continue
            b, k = (c // wide) * wide, c % wide
            for r in range(window):
                v = val[b * window + r * wide + k]
                row = win[p] * window + r
                if v != 0 and row < m_out:
                    Y[row] += v * X[j]
    return Y


def sddmm_fp64(rowptr, col, A, B):
    """out[h][e] = A[h][row(e)] . B[h][col(e)]; A, B of shape [h, M, F]."""
    rows = csr_rows(rowptr)
    col = np.asarray(col, dtype=np.int64)
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    return np.einsum("hef,hef->he", A[:, rows, :], B[:, col, :])


def att_fp64(rowptr, col, X, a0, a1):
    """out[h][e] = X[h][row].a0[h] + X[h][col].a1[h]; X [h,M,F], a [h,1,F]."""
    rows = csr_rows(rowptr)
    col = np.asarray(col, dtype=np.int64)
    X = np.asarray(X, dtype=np.float64)
    s0 = np.einsum("hmf,hf->hm", X, np.asarray(a0, dtype=np.float64).reshape(X.shape[0], -1))
    s1 = np.einsum("hmf,hf->hm", X, np.asarray(a1, dtype=np.float64).reshape(X.shape[0], -1))
    return s0[:, rows] + s1[:, col]


def attv2_fp64(rowptr, col, X0, X1, a):
    rows = csr_rows(rowptr)
    col = np.asarray(col, dtype=np.int64)
    X0 = np.asarray(X0, dtype=np.float64)
    X1 = np.asarray(X1, dtype=np.float64)
    av = np.asarray(a, dtype=np.float64).reshape(X0.shape[0], -1)
    s0 = np.einsum("hmf,hf->hm", X0, av)
    s1 = np.einsum("hmf,hf->hm", X1, av)
    return s0[:, rows] + s1[:, col]


def ones_fp64(rowptr, g):
    """out[h][e] = g[row(e)][h]; g of shape [M, h, 1]."""
    rows = csr_rows(rowptr)
    g = np.asarray(g, dtype=np.float64).reshape(np.asarray(g).shape[0], -1)
    return g[rows, :].T


def spmm_edge_fp64(rowptr, col, vals, X, n_out):
    """Y[h] = A(vals[h]) X[h]; vals [h, nnz], X [h, M, F] -> [h, n_out, F].
    Duplicate edges: the last edge id of a (row,col) pair supplies the value."""
    vals = np.asarray(vals, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    out = [spmm_csr_fp64(rowptr, col, vals[h], X[h], n_out) for h in range(vals.shape[0])]
    return np.stack(out)


def rowsum_fp64(rowptr, vals, n_out, col=None):
    """Row sums of per-edge values: [h, n_out]."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    vals = np.asarray(vals, dtype=np.float64)
    rows = csr_rows(rowptr)
    out = np.zeros((vals.shape[0], rowptr.shape[0] - 1), dtype=np.float64)
    for h in range(vals.shape[0]):
        np.add.at(out[h], rows, vals[h])
    return out[:, :n_out]


def edge_softmax_fp64(rowptr, logits):
    """Row-wise softmax over each row's edges, per head: logits [h, nnz]."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    z = np.asarray(logits, dtype=np.float64)
    out = np.zeros_like(z)
    for r in range(rowptr.shape[0] - 1):
        s, e = rowptr[r], rowptr[r + 1]
        if e > s:
            m = z[:, s:e].max(axis=1, keepdims=True)
            ex = np.exp(z[:, s:e] - m)
            out[:, s:e] = ex / ex.sum(axis=1, keepdims=True)
    return out


def gat_layer_fp64(rowptr, col, Xp, a0, a1, n_out, slope=0.2):
    """GAT layer forward on projected features Xp [h, M, F]:
    e = Xp_i.a0 + Xp_j.a1 -> LeakyReLU -> row softmax -> sum_j p_ij Xp_j."""
    e = att_fp64(rowptr, col, Xp, a0, a1)
    e = np.where(e > 0, e, slope * e)
    p = edge_softmax_fp64(rowptr, e)
    return spmm_edge_fp64(rowptr, col, p, Xp, n_out)


def rel_err(got, ref):
    """max |got-ref| / max(|ref|, tiny)  (normwise relative error)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    denom = max(np.abs(ref).max() if ref.size else 0.0, 1e-30)
    return float(np.abs(got - ref).max() / denom) if ref.size else 0.0


# --------------------------------------------------------------------------
# CPU baseline: the reference's CPU path for the SpMM (torch.sparse CSR)
# --------------------------------------------------------------------------

def csr_fp32(rowptr, col, vals, n_cols):
    """torch CSR fp32 matrix on the host (the reference's CPU-path operand)."""
    import torch
    rowptr = torch.as_tensor(rowptr).long()
    return torch.sparse_csr_tensor(rowptr, torch.as_tensor(col).long(),
                                   torch.as_tensor(vals).float(),
                                   size=(rowptr.numel() - 1, int(n_cols)))


def spmm_cpu_fp32(A, X):
    """Y = A X with torch.sparse on the host cores (fp32)."""
    import torch
    return torch.sparse.mm(A, X)


def gat_dot_layer_fp64(rowptr, col, Xp, n_out, slope=0.2):
    """GAT layer with dot-product logits per head (the SDDMM of (XW)(XW)^T
    masked to the edges, as in the 232,965-node GAT-layer workload): e_ij = Xp_i . Xp_j -> LeakyReLU -> row softmax -> sum_j p_ij Xp_j.
    Xp [h, M, F]."""
    e = sddmm_fp64(rowptr, col, Xp, Xp)
    e = np.where(e > 0, e, slope * e)
    p = edge_softmax_fp64(rowptr, e)
    return spmm_edge_fp64(rowptr, col, p, Xp, n_out)


def gat_dot_layer_cpu_fp32(rowptr, col, Xp, slope=0.2):
    """CPU fp32 restatement (torch, all host threads) of the GAT layer with dot
    logits, for the CPU baseline: e = Xp_i . Xp_j on the edges, LeakyReLU,
    row softmax (max-subtracted), weighted sum of neighbour rows."""
    import torch
    rowptr = torch.as_tensor(rowptr).long()
    col = torch.as_tensor(col).long()
    n = rowptr.numel() - 1
    rows = torch.repeat_interleave(torch.arange(n), rowptr[1:] - rowptr[:-1])
    Xr = Xp[rows]
    Xc = Xp[col]
    e = (Xr * Xc).sum(1)
    e = torch.nn.functional.leaky_relu(e, slope)
    m = torch.full((n,), float("-inf")).scatter_reduce(0, rows, e, "amax")
    p = torch.exp(e - m[rows])
    l = torch.zeros(n).index_add_(0, rows, p)
    out = torch.zeros(n, Xp.shape[1]).index_add_(0, rows, p[:, None] * Xc)
    return out / l.clamp_min(1e-30)[:, None]


def gat_add_layer_torch(rowptr, col, Xp, a0, a1, slope=0.2):
    """Differentiable torch restatement (use fp64 tensors) of the additive
    multi-head GAT aggregation (end2end_ori/gat_final/mgat_csr/mgat_conv.py:
    173-198 without dropout): Xp [N, H*F], a0/a1 [H, F] -> [N, H*F].
    Its autograd gradient is the reference gradient of the backward tests."""
    import torch
    rowptr = torch.as_tensor(rowptr).long()
    col = torch.as_tensor(col).long()
    H, F = a0.shape
    N = rowptr.numel() - 1
    X3 = Xp.view(-1, H, F)[:N]
    s0 = (X3 * a0[None]).sum(-1)
    s1 = (X3 * a1[None]).sum(-1)
    rows = torch.repeat_interleave(torch.arange(N), rowptr[1:] - rowptr[:-1])
    e = torch.nn.functional.leaky_relu(s0[rows] + s1[col], slope)
    m = torch.full((N, H), float("-inf"), dtype=e.dtype).scatter_reduce(
        0, rows[:, None].expand(-1, H), e, "amax").detach()
    ex = torch.exp(e - m[rows])
    l = torch.zeros(N, H, dtype=e.dtype).index_add(0, rows, ex)
    p = ex / l[rows]
    out = torch.zeros(N, H, F, dtype=e.dtype).index_add(0, rows, p[:, :, None] * X3[col])
    return out.reshape(N, H * F)


def gatv2_layer_torch(rowptr, col, X, W0, W1, a, slope=0.2, n_out=None):
    """Differentiable torch restatement (use fp64 tensors) of the reference's
    GATv2 layer (end2end_head/gatv2_final/mgat_csr/mgat_conv.py:151-196, no
    dropout): X0' = LeakyReLU(X W0), X1' = LeakyReLU(X W1) per head;
    e_ij = X0'_i.a + X1'_j.a; per head e is scaled to [0, 1] by its minimum
    and maximum over all edges; p = exp(e) / row sum; out_i = sum_j p_ij X1'_j.
    X [N, D], W0 / W1 [D, H*F], a [H, 1, F] -> [N, H, F]."""
    import torch
    rowptr = torch.as_tensor(rowptr).long()
    col = torch.as_tensor(col).long()
    H, _, Fo = a.shape
    N = rowptr.numel() - 1
    lr = torch.nn.functional.leaky_relu
    X0 = lr((X @ W0).view(-1, H, Fo), slope)
    X1 = lr((X @ W1).view(-1, H, Fo), slope)
    rows = torch.repeat_interleave(torch.arange(N), rowptr[1:] - rowptr[:-1])
    s0 = (X0 * a[:, 0][None]).sum(-1)  # [N, H]
    s1 = (X1 * a[:, 0][None]).sum(-1)
    e = s0[rows] + s1[col]              # [nnz, H]
    mn = e.min(0, keepdim=True).values
    mx = e.max(0, keepdim=True).values
    ex = torch.exp((e - mn) / (mx - mn))
    l = torch.zeros(N, H, dtype=e.dtype).index_add(0, rows, ex)
    out = torch.zeros(N, H, Fo, dtype=e.dtype).index_add(0, rows, ex[:, :, None] * X1[col])
    out = out / l[:, :, None]
    return out if n_out is None else out[:n_out]


def rel_err_fro(got, ref):
    """||got - ref||_F / ||ref||_F (Frobenius-norm relative error)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    d = np.linalg.norm(ref)
    return float(np.linalg.norm(got - ref) / d) if d > 0 else 0.0


# --------------------------------------------------------------------------
# Row-sampled FP64 restatements (full-size graphs: only the sampled rows and
# the neighbours they read are evaluated)
# --------------------------------------------------------------------------

def sub_csr(rowptr, col, rows):
    """CSR restricted to `rows` (in the given order): (rowptr_sub int64,
    col_sub int64, edge ids int64 into the full CSR)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    rows = np.asarray(rows, dtype=np.int64)
    starts, ends = rowptr[rows], rowptr[rows + 1]
    lens = ends - starts
    rp = np.zeros(rows.shape[0] + 1, dtype=np.int64)
    np.cumsum(lens, out=rp[1:])
    eid = np.repeat(starts - rp[:-1], lens) + np.arange(rp[-1], dtype=np.int64)
    return rp, np.asarray(col, dtype=np.int64)[eid], eid


def sample_rows(rowptr, n_rows, n_random, n_top, seed, window=8):
    """Sorted unique row ids: `n_random` seeded random rows plus every row of
    the windows that hold the `n_top` longest rows (the hub windows, whose
    parts split the most)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    lens = np.diff(rowptr)[:n_rows]
    rng = np.random.default_rng(seed)
    pick = [rng.choice(n_rows, size=min(n_random, n_rows), replace=False)]
    top = np.argsort(lens, kind="stable")[::-1][:n_top]
    for r in top:
        w0 = (r // window) * window
        pick.append(np.arange(w0, min(w0 + window, n_rows)))
    return np.unique(np.concatenate(pick))


def spmm_rows_fp64(rowptr, col, vals, X, rows):
    """(A X)[rows] in FP64; `vals` are the per-edge values of the full CSR."""
    rp, c, eid = sub_csr(rowptr, col, rows)
    return spmm_csr_fp64(rp, c, np.asarray(vals)[eid], X)


def gat_dot_rows_fp64(rowptr, col, Xp, rows, slope=0.2):
    """Dot-logit GAT layer (one head) for `rows`: e_ij = Xp_i . Xp_j on the
    edges, LeakyReLU, row softmax, sum_j p_ij Xp_j.  Xp [N, F]."""
    rows = np.asarray(rows, dtype=np.int64)
    rp, c, _ = sub_csr(rowptr, col, rows)
    X = np.asarray(Xp, dtype=np.float64)
    lens = np.diff(rp)
    out = np.zeros((len(rows), X.shape[1]))
    nz = np.nonzero(lens)[0]
    if nz.size == 0:
        return out
    seg = np.repeat(np.arange(len(rows)), lens)
    Xc = X[c]
    e = np.einsum("ef,ef->e", X[rows[seg]], Xc)
    e = np.where(e > 0, e, slope * e)
    starts = rp[:-1][nz]  # segments are contiguous and in row order
    m = np.maximum.reduceat(e, starts)
    mm = np.zeros(len(rows))
    mm[nz] = m
    pe = np.exp(e - mm[seg])
    l = np.add.reduceat(pe, starts)
    acc = np.add.reduceat(pe[:, None] * Xc, starts, axis=0)
    out[nz] = acc / l[:, None]
    return out


def gat_add_rows_torch(rowptr, col, Xp, a0, a1, rows, slope=0.2):
    """Differentiable FP64 restatement of the additive multi-head GAT
    aggregation (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198, no
    dropout) for `rows` only: Xp [N, H*F] (full, requires_grad allowed),
    a0 / a1 [H, F] -> [len(rows), H*F].  Gradients flow to every Xp row the
    sampled rows read."""
    import torch
    rp, c, _ = sub_csr(rowptr, col, rows)
    H, F = a0.shape
    rows_t = torch.as_tensor(np.asarray(rows, dtype=np.int64))
    c_t = torch.as_tensor(c)
    seg = torch.repeat_interleave(torch.arange(len(rows)), torch.as_tensor(np.diff(rp)))
    X3 = Xp.view(Xp.shape[0], H, F)
    s0 = (X3[rows_t] * a0[None]).sum(-1)
    Xc = X3[c_t]
    s1 = (Xc * a1[None]).sum(-1)
    e = torch.nn.functional.leaky_relu(s0[seg] + s1, slope)
    m = torch.full((len(rows), H), float("-inf"), dtype=e.dtype).scatter_reduce(
        0, seg[:, None].expand(-1, H), e, "amax").detach()
    ex = torch.exp(e - m[seg])
    l = torch.zeros(len(rows), H, dtype=e.dtype).index_add(0, seg, ex)
    p = ex / l[seg]
    out = torch.zeros(len(rows), H, F, dtype=e.dtype).index_add(0, seg, p[:, :, None] * Xc)
    return out.reshape(len(rows), H * F)


def gcn2_fp64(rowptr, col, vals, X, W1, W2, n_out):
    """2-layer GCN inference Y = A relu(A X W1) W2 in FP64 on the host (torch
    CSR, all host threads); A from per-edge values (the GCN layer composition of
    end2end_ori/gcn_final/mgat_csr/mgat_conv.py:27-54 with ReLU between)."""
    import torch
    rowptr = torch.as_tensor(np.asarray(rowptr, dtype=np.int64))
    A = torch.sparse_csr_tensor(rowptr, torch.as_tensor(np.asarray(col, dtype=np.int64)),
                                torch.as_tensor(np.asarray(vals, dtype=np.float64)),
                                size=(rowptr.numel() - 1, X.shape[0]))
    X = torch.as_tensor(np.asarray(X, dtype=np.float64))
    W1 = torch.as_tensor(np.asarray(W1, dtype=np.float64))
    W2 = torch.as_tensor(np.asarray(W2, dtype=np.float64))
    H = torch.relu(torch.sparse.mm(A, X @ W1))
    Y = torch.sparse.mm(A, H[: X.shape[0]] @ W2)
    return Y[:n_out].numpy()
