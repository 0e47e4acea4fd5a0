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
        """Fused GAT aggregation.  Xp: [n_nodes, n_heads*F] fp16/bf16 (projected
        features).  mode MODE_DOT: logits X'_i . X'_j per head; MODE_ADD: logits
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
