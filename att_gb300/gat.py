"""GAT attention on the GPU: a graph object holding the resident block format
and the fused SDDMM -> LeakyReLU -> edge-softmax -> SpMM kernel.

``GATGraph(rowptr, col)`` converts the CSR once (8-row windows) and keeps, on
the device: the block structure, the per-edge slot index, an occupancy bitmap
of the slots, and the work plan of the fused kernel (chunks of up to
``parts_per_chunk`` consecutive parts of one window; windows spread over
several chunks are merged from fp32 partials).  ``attention(...)`` runs the
fused layer; the unfused reference chain (end2end_ori/gat_final/mgat_csr/
mgat_conv.py:173-198) is available through the ATT_SDDMM_v* / ATT_SpMM_v*
drop-ins.
"""
import torch

from . import _lib, ops
from .ops import _DT, _p, _stream, require_cuda

MODE_DOT, MODE_ADD = 0, 1


class GATGraph:
    def __init__(self, rowptr, col, window=8, wide=8, part=32, parts_per_chunk=4):
        require_cuda()
        if window != 8:
            raise ValueError("the fused GAT kernel uses 8-row windows")
        rowptr = torch.as_tensor(rowptr)
        n_nodes = int(rowptr.shape[0]) - 1
        if n_nodes % window:
            # whole windows only (the conversion drops a ragged last window);
            # the extra rows are empty, as in the reference loaders' padding
            pad = window - n_nodes % window
            rowptr = torch.cat([rowptr, rowptr[-1:].expand(pad)])
        self.fmt = ops.block_convert(rowptr, col, None, window=window, wide=wide, part=part,
                                     want_val=False, want_edge_slot=True, n_cols=n_nodes)
        f = self.fmt
        self.n_nodes = n_nodes
        self.window, self.wide = window, wide
        n_slots = f.n_condensed * window
        self.mask = torch.empty(max((n_slots + 31) // 32, 1), dtype=torch.int32, device="cuda")
        _lib.call("att_slot_mask", _p(f.edge_slot), f.nnz, _p(self.mask), (n_slots + 31) // 32,
                  _stream())
        self._plan(parts_per_chunk)
        self._transposed = None
        self._csr = (rowptr, torch.as_tensor(col))

    def transposed(self):
        """The graph of the reversed edges (for the backward pass); the graph
        itself when the CSR is symmetric."""
        if self._transposed is None:
            rowptr, col = self._csr
            rowptr = rowptr.to("cuda").long()
            col = col.to("cuda").long()
            n = self.n_nodes
            rows = torch.repeat_interleave(torch.arange(n, device="cuda"),
                                           rowptr[1:n + 1] - rowptr[:n])
            key_t = torch.sort(col * n + rows).values
            if torch.equal(key_t, rows * n + col):
                self._transposed = self
            else:
                rt, ct = key_t // n, key_t % n
                rp_t = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
                rp_t[1:] = torch.cumsum(torch.bincount(rt, minlength=n), 0)
                self._transposed = GATGraph(rp_t.to(torch.int32), ct.to(torch.int32),
                                            window=self.window, wide=self.wide)
        return self._transposed

    def attention_backward(self, Xp, dout, s0, s1, row_max, row_sum, c, n_heads, slope=0.2):
        """Fused backward of attention(mode=MODE_ADD): returns (dXp_agg fp32
        [n_nodes, H*F], ds0, ds1 fp32 [H, n_nodes]) with
        dXp_agg[j] = sum_i p_ij dout_i and ds0 / ds1 the gradients of the
        scores s0 / s1.  ``c[h][i] = dout_i . out_i``."""
        dout32 = dout.float()
        hi = dout32.to(Xp.dtype).contiguous()
        lo = (dout32 - hi.float()).to(Xp.dtype).contiguous()
        return self.attention_backward_split(Xp, hi, lo, s0, s1, row_max, row_sum, c, n_heads,
                                             slope)

    def attention_backward_split(self, Xp, dout, dout_lo, s0, s1, row_max, row_sum, c, n_heads,
                                 slope=0.2):
        """attention_backward with dout given as its 16-bit hi part and the
        16-bit rounding of the remainder (att_gat_grad_prepare makes both)."""
        require_cuda()
        T = self.transposed()
        f = T.fmt
        N = self.n_nodes
        F = Xp.shape[1] // n_heads
        Xp = Xp.contiguous()
        dXp = torch.zeros(N, n_heads * F, dtype=torch.float32, device=Xp.device)
        ds0 = torch.zeros(n_heads, N, dtype=torch.float32, device=Xp.device)
        ds1 = torch.zeros(n_heads, N, dtype=torch.float32, device=Xp.device)
        _lib.call("att_gat_backward", _p(f.rowptr), _p(f.col), _p(T.mask), _p(f.window_of_part),
                  f.n_parts, self.window, self.wide, _p(Xp), _p(dout), _p(dout_lo),
                  _DT[Xp.dtype], N, n_heads,
                  F, Xp.stride(0), dout.stride(0), _p(s0.contiguous()), _p(s1.contiguous()),
                  _p(row_max.contiguous()), _p(row_sum.contiguous()), _p(c.contiguous()),
                  float(slope), _p(dXp), dXp.stride(0), _p(ds0), _p(ds1), None, _stream())
        return dXp, ds0, ds1


    def _plan(self, T):
        win = self.fmt.window_of_part.long()
        P = win.numel()
        dev = win.device
        if P == 0:
            self.chunk_begin = torch.zeros(1, dtype=torch.int32, device=dev)
            self.chunk_slot = torch.zeros(0, dtype=torch.int32, device=dev)
            self.multi = torch.zeros(0, dtype=torch.int32, device=dev)
            self.n_chunks = self.n_multi = self.n_slots = 0
            return
        ar = torch.arange(P, device=dev)
        new_win = torch.ones(P, dtype=torch.bool, device=dev)
        new_win[1:] = win[1:] != win[:-1]
        first = torch.cummax(torch.where(new_win, ar, torch.zeros_like(ar)), 0).values
        starts = torch.nonzero(((ar - first) % T) == 0).flatten()
        n_chunks = starts.numel()
        chunk_win_new = new_win[starts]                      # chunk opens a window
        group = torch.cumsum(chunk_win_new.long(), 0) - 1    # window group per chunk
        counts = torch.bincount(group)
        multi_chunk = counts[group] > 1
        slot = torch.full((n_chunks,), -1, dtype=torch.int64, device=dev)
        n_slots = int(multi_chunk.sum().item())
        slot[multi_chunk] = torch.arange(n_slots, device=dev)
        gfirst = torch.nonzero(chunk_win_new).flatten()
        mg = counts > 1
        multi = torch.stack([gfirst[mg], gfirst[mg] + counts[mg]], 1).flatten()
        self.chunk_begin = torch.cat([starts, torch.tensor([P], device=dev)]).to(torch.int32)
        self.chunk_slot = slot.to(torch.int32)
        self.multi = multi.to(torch.int32).contiguous()
        self.n_chunks, self.n_slots, self.n_multi = n_chunks, n_slots, int(mg.sum().item())

    def attention(self, Xp, n_heads=1, mode=MODE_DOT, s0=None, s1=None, slope=0.2, out=None,
                  stats=True):
        """Fused GAT aggregation.  Xp: [n_nodes, n_heads*F] fp16/bf16, or fp32
        for TF32 tensor cores with 3xTF32 products (projected features).  mode MODE_DOT: logits X'_i . X'_j per head; MODE_ADD: logits
        s0[h][i] + s1[h][j] (fp32 [n_heads, n_nodes]).  Returns
        (out fp32 [n_nodes, n_heads*F], row_max, row_sum) with the fp32 softmax
        statistics [n_heads, n_nodes] (None if not ``stats``)."""
        require_cuda()
        f = self.fmt
        N = self.n_nodes
        if Xp.dim() != 2 or Xp.shape[0] < N or Xp.shape[1] % n_heads:
            raise ValueError("Xp must be [n_nodes, n_heads*F]")
        if Xp.stride(1) != 1:
            Xp = Xp.contiguous()
        F = Xp.shape[1] // n_heads
        if out is None:
            out = torch.empty(N, n_heads * F, dtype=torch.float32, device=Xp.device)
        rmax = rsum = None
        if stats:
            rmax = torch.empty(n_heads, N, dtype=torch.float32, device=Xp.device)
            rsum = torch.empty(n_heads, N, dtype=torch.float32, device=Xp.device)
        partial = None
        if self.n_slots:
            partial = torch.empty(self.n_slots * n_heads * 8 * (F + 2), dtype=torch.float32,
                                  device=Xp.device)
        if mode == MODE_ADD:
            s0 = s0.float().contiguous()
            s1 = s1.float().contiguous()
        _lib.call("att_gat_forward", _p(f.rowptr), _p(f.col), _p(self.mask),
                  _p(f.window_of_part), f.n_parts, _p(self.chunk_begin), _p(self.chunk_slot),
                  self.n_chunks, _p(self.multi), self.n_multi, self.window, self.wide, _p(Xp),
                  _DT[Xp.dtype], N, n_heads, F, Xp.stride(0), mode, _p(s0), _p(s1), float(slope),
                  _p(out), out.stride(0), _p(rmax), _p(rsum), _p(partial), None, _stream())
        return out, rmax, rsum


class GATAttention(torch.autograd.Function):
    """Additive multi-head GAT aggregation with the fused forward and backward
    kernels: out_i = sum_j softmax_j(LeakyReLU(X'_i.a0 + X'_j.a1)) X'_j per
    head (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198 without dropout).
    Xp [N, H*F] fp16/bf16, a0/a1 [H, F]; returns fp32 [N, H*F]."""

    @staticmethod
    def forward(ctx, Xp, a0, a1, graph, n_heads, slope):
        from . import gat_ops
        N = graph.n_nodes
        F = Xp.shape[1] // n_heads
        X3 = Xp.view(N, n_heads, F).permute(1, 0, 2)
        # attention vectors stay fp32: rounding them would shift every score
        s0, s1 = gat_ops.node_scores_pair(X3, a0, a1)
        out, rmax, rsum = graph.attention(Xp, n_heads=n_heads, mode=MODE_ADD, s0=s0, s1=s1,
                                          slope=slope)
        ctx.save_for_backward(Xp, a0, a1, s0, s1, rmax, rsum, out)
        ctx.graph, ctx.n_heads, ctx.slope = graph, n_heads, slope
        return out

    @staticmethod
    def backward(ctx, dout):
        Xp, a0, a1, s0, s1, rmax, rsum, out = ctx.saved_tensors
        G, H, slope = ctx.graph, ctx.n_heads, ctx.slope
        N = G.n_nodes
        F = Xp.shape[1] // H
        dev = Xp.device
        dout = dout.float().contiguous()
        out = out.contiguous()
        # c[h][i] = dout_i . out_i and the hi/lo split of dout, one pass
        hi = torch.empty(N, H * F, dtype=Xp.dtype, device=dev)
        lo = torch.empty_like(hi)
        c = torch.empty(H, N, dtype=torch.float32, device=dev)
        _lib.call("att_gat_grad_prepare", _p(dout), dout.stride(0), _p(out), out.stride(0), N, H,
                  F, _p(hi), _p(lo), _DT[Xp.dtype], hi.stride(0), _p(c), _stream())
        dXp, ds0, ds1 = G.attention_backward_split(Xp, hi, lo, s0, s1, rmax, rsum, c, H, slope)
        # dX' = dXp + ds0 a0 + ds1 a1 (cast to X' dtype), da0 / da1 = sum_n ds X', one pass
        Xp = Xp.contiguous()
        dX = torch.empty(N, H * F, dtype=Xp.dtype, device=dev)
        da0 = torch.zeros(H, F, dtype=torch.float32, device=dev)
        da1 = torch.zeros(H, F, dtype=torch.float32, device=dev)
        _lib.call("att_gat_grad_finish", _p(dXp), dXp.stride(0), _p(ds0), _p(ds1),
                  _p(a0.float().contiguous()), _p(a1.float().contiguous()), _p(Xp), _DT[Xp.dtype],
                  Xp.stride(0), N, H, F, _p(dX), dX.stride(0), _p(da0), _p(da1), _stream())
        return dX, da0.to(a0.dtype), da1.to(a1.dtype), None, None, None


class GATConv(torch.nn.Module):
    """Multi-head GAT layer on the fused kernels: X -> X W (per head F
    features) -> additive attention -> [N, H*F] fp32 (concatenated heads).
    Parameters as the reference's GATConv_multi
    (end2end_head/gat_final/mgat_csr/mgat_conv.py:154-198): W Xavier-normal,
    a0 / a1 [H, F]."""

    def __init__(self, in_dim, out_dim, heads=1, slope=0.2, dtype=torch.bfloat16):
        super().__init__()
        gain = torch.nn.init.calculate_gain("relu")
        self.W = torch.nn.Parameter(torch.empty(in_dim, heads * out_dim))
        torch.nn.init.xavier_normal_(self.W, gain=gain)
        self.a0 = torch.nn.Parameter(torch.empty(heads, out_dim))
        self.a1 = torch.nn.Parameter(torch.empty(heads, out_dim))
        torch.nn.init.xavier_normal_(self.a0, gain=gain)
        torch.nn.init.xavier_normal_(self.a1, gain=gain)
        self.heads, self.out_dim, self.slope, self.dtype = heads, out_dim, slope, dtype

    def forward(self, X, graph):
        Xp = torch.mm(X.to(self.dtype), self.W.to(self.dtype))
        return GATAttention.apply(Xp, self.a0, self.a1, graph, self.heads, self.slope)


class DotAttentionChain:
    """One dot-product GAT aggregation as the reference composes it, a chain
    of separate ops with per-edge intermediates
    (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198 with the SDDMM of
    ATT_SDDMM_v1.sddmm_*_h_nnz): per-edge logits X'_i . X'_j on tensor cores
    (att_sddmm), LeakyReLU, the row softmax (row max subtracted so exp cannot
    overflow; torch segment reductions), then the SpMM of the normalised edge
    values (att_gather_slot_values + att_spmm).  16-bit X' runs fp16/bf16
    tensor-core ops; fp32 X' runs the TF32 kernels (3xTF32, fp32-accurate).
    The fused kernel (GATGraph.attention, mode MODE_DOT) computes the same
    layer without the nnz-sized intermediates."""

    def __init__(self, rowptr, col, window=8, wide=8, part=32):
        require_cuda()
        from . import gat_ops
        rowptr = torch.as_tensor(rowptr).to("cuda")
        col = torch.as_tensor(col).to("cuda")
        n = int(rowptr.shape[0]) - 1
        if n % window:
            pad = window - n % window
            rowptr = torch.cat([rowptr, rowptr[-1:].expand(pad)])
        fmt = ops.block_convert(rowptr.to(torch.int32), col.to(torch.int32), None, window=window,
                                wide=wide, part=part, want_val=False, want_map=True, n_cols=n)
        self.fmt, self.window, self.n_nodes, self.nnz = fmt, window, n, fmt.nnz
        self.qmap = gat_ops.map_to_quad(fmt.map, window, wide)
        self.csr_rowptr = rowptr[: n + 1].to(torch.int32).contiguous()

    def __call__(self, Xp, slope=0.2):
        from . import gat_ops
        f, n = self.fmt, self.n_nodes
        X3 = Xp.unsqueeze(0)
        e = gat_ops.sddmm(f.rowptr, f.col, self.qmap, f.window_of_part, self.window, X3, X3,
                          self.nnz, torch.float32)[0]
        # LeakyReLU + row softmax (att_edge_softmax), values in X' dtype
        p = torch.empty(self.nnz, dtype=Xp.dtype, device=Xp.device)
        _lib.call("att_edge_softmax", _p(self.csr_rowptr), n, _p(e), self.nnz, 1, float(slope), 1,
                  _p(p), _DT[Xp.dtype], self.nnz, None, None, _stream())
        return gat_ops.spmm_edge(f.rowptr, f.col, self.qmap, f.window_of_part, f.atomic,
                                 self.window, p, 0, 1, X3, n)[0]
