"""Model-level glue on the GPU path: the reference's autograd Functions and
conv layers, restated over the drop-in modules, and the GAT network on the
fused kernels.

* ``GCNInput`` / ``GATInput`` build what the reference's dataset classes hold
  (end2end_ori/gcn_final/mgat_csr/mdataset_fp16.py:39-91,
  end2end_ori/gat_final/mgat_csr/mdataset_fp16.py:39-92) from an edge list,
  without the .npz file I/O: node count padded to N + 8 - N % 8, CSR, degree
  normalisation, block conversion (on the GPU).
* ``MGCNFunction`` / ``GCNConv`` -- end2end_ori/gcn_final/mgat_csr/mgat_conv.py:27-108.
* ``SAGEConv`` -- end2end_ori/gsage_final/mgat_csr/mgat_conv.py:85-107.
* ``MGATFunction_multi``, ``MGATSpmm_multi``, ``MGATSpmm1_multi``,
  ``GATConv_multi`` -- end2end_head/gat_final/mgat_csr/mgat_conv.py:14-198
  (the multi-head v3 chain of separate ops: the "plain" drop-in path).
* ``MGATv2Function_multi``, ``GATv2Conv_multi`` --
  end2end_head/gatv2_final/mgat_csr/mgat_conv.py:14-196 (GATv2 on the same ops).
* ``GATNet`` -- the reference's Net (end2end_ori/gat_final/mgat_csr/gat_mgnn.py:17-40)
  with either that chain or the fused kernels (att_gb300.gat.GATConv).
"""
import math

import torch
import torch.nn as nn
import torch.nn.functional as F

from . import gat as _gat
from .compat import ATT_Block_v3, ATT_SDDMM_v3, ATT_SpMM_v3, Block_sr_bcrs, SpMM_sr_bcrs


def _csr(src, dst, num_nodes_padded):
    """CSR (sorted columns, duplicates merged) of edges src -> dst."""
    src = torch.as_tensor(src).long()
    dst = torch.as_tensor(dst).long()
    key = torch.unique(src * num_nodes_padded + dst)
    rows, cols = key // num_nodes_padded, key % num_nodes_padded
    rowptr = torch.zeros(num_nodes_padded + 1, dtype=torch.int64)
    rowptr[1:] = torch.cumsum(torch.bincount(rows, minlength=num_nodes_padded), 0)
    return rowptr.to(torch.int32), cols.to(torch.int32)


class GCNInput:
    """What MGAT_dataset_csr (GCN) holds, on the GPU (mdataset_fp16.py:39-91;
    mdataset_tf32.py for ``precision="tf32"``)."""

    def __init__(self, src, dst, num_nodes, precision="fp16", features=None, labels=None):
        self.num_nodes_ori = int(num_nodes)
        self.num_nodes = self.num_nodes_ori + 8 - self.num_nodes_ori % 8
        rowptr, col = _csr(src, dst, self.num_nodes)
        self.num_edges = int(col.numel())
        dd = (rowptr[1:] - rowptr[:-1]).float()
        self.dd1 = dd[: self.num_nodes_ori, None].cuda().clamp_min(1)  # SAGE mean
        dd = torch.rsqrt(dd)
        if precision == "fp16":
            res = Block_sr_bcrs.blockProcess_fp16_balance(rowptr, col, dd.half(), 8, 8, 32,
                                                          device="cuda")
        else:
            res = Block_sr_bcrs.blockProcess_tf32_balance(rowptr, col, dd, 8, 4, 32,
                                                          device="cuda")
        (self.row_pointers, self.column_index, self.degrees, self.t_window_rowTensor,
         self.t_atomicTensor) = res
        self.precision = precision
        self.x = features
        self.y = labels


class GATInput:
    """What MGAT_dataset_csr (GAT) holds, on the GPU
    (end2end_ori/gat_final/mgat_csr/mdataset_fp16.py:39-92)."""

    def __init__(self, src, dst, num_nodes, features=None, labels=None, wide=8):
        self.num_nodes_ori = int(num_nodes)
        self.num_nodes = self.num_nodes_ori + 8 - self.num_nodes_ori % 8
        rowptr, col = _csr(src, dst, self.num_nodes)
        self.csr = (rowptr, col)
        self.num_edges = int(col.numel())
        (self.row_pointers, self.column_index, self.degrees, self.degrees_trans, self.window,
         self.automic) = ATT_Block_v3.blockProcess_sddmm_balance_gnn_trans(rowptr, col, 8, wide,
                                                                          32, device="cuda")
        self.max_vectors = torch.max(self.row_pointers[2::2] - self.row_pointers[:-2:2])
        self.max = self.max_vectors / 16
        self.x = features
        self.y = labels
        self._fused = None

    def fused_graph(self):
        """The same graph as an att_gb300.gat.GATGraph (fused kernels)."""
        if self._fused is None:
            rowptr, col = self.csr
            self._fused = _gat.GATGraph(rowptr[: self.num_nodes_ori + 1], col)
        return self._fused


# ---------------------------------------------------------------------------
# GCN / GraphSAGE (end2end_ori/gcn_final/mgat_csr/mgat_conv.py:27-108)
# ---------------------------------------------------------------------------
def _spmm(inputInfo, X):
    fn = SpMM_sr_bcrs.forward_fp16_gnn if inputInfo.precision == "fp16" else \
        SpMM_sr_bcrs.forward_tf32_gnn
    return fn(inputInfo.row_pointers, inputInfo.column_index, inputInfo.degrees,
              inputInfo.t_window_rowTensor, inputInfo.t_atomicTensor, X.contiguous(),
              inputInfo.num_nodes, X.size(1), inputInfo.num_nodes_ori)[0]


class MGCNFunction(torch.autograd.Function):
    """Y = A_hat (X W); backward reuses the forward SpMM (A_hat symmetric),
    as the reference does (mgat_conv.py:56-74)."""

    @staticmethod
    def forward(ctx, X, weights, inputInfo):
        ctx.save_for_backward(X, weights)
        ctx.inputInfo = inputInfo
        X_prime = torch.mm(X, weights)
        out = _spmm(inputInfo, X_prime)
        return out.to(X.dtype)

    @staticmethod
    def backward(ctx, d_output):
        X, weights = ctx.saved_tensors
        d_input_prime = _spmm(ctx.inputInfo, d_output.to(X.dtype)).to(X.dtype)
        return torch.mm(d_input_prime, weights.t()), torch.mm(X.t(), d_input_prime), None


class GCNConv(nn.Module):
    def __init__(self, input_dim, output_dim):
        super().__init__()
        self.weights = nn.Parameter(torch.empty(input_dim, output_dim))
        stdv = 1.0 / math.sqrt(output_dim)
        self.weights.data.uniform_(-stdv, stdv)

    def forward(self, X, inputInfo):
        dt = torch.float16 if inputInfo.precision == "fp16" else torch.float32
        return MGCNFunction.apply(X.to(dt), self.weights.to(dt), inputInfo)


class _AggOnly(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, inputInfo):
        ctx.inputInfo = inputInfo
        return _spmm(inputInfo, X).to(X.dtype)

    @staticmethod
    def backward(ctx, d):
        return _spmm(ctx.inputInfo, d.contiguous()).to(d.dtype), None


class SAGEConv(nn.Module):
    """GraphSAGE layer: A_hat (X W) / deg + X W1
    (end2end_ori/gsage_final/mgat_csr/mgat_conv.py:95-107)."""

    def __init__(self, input_dim, output_dim):
        super().__init__()
        self.weights = nn.Parameter(torch.empty(input_dim, output_dim))
        self.weights1 = nn.Parameter(torch.empty(input_dim, output_dim))
        stdv = 1.0 / math.sqrt(output_dim)
        self.weights.data.uniform_(-stdv, stdv)
        self.weights1.data.uniform_(-stdv, stdv)

    def forward(self, X, inputInfo):
        dt = torch.float16 if inputInfo.precision == "fp16" else torch.float32
        X = X.to(dt)
        agg = _AggOnly.apply(torch.mm(X, self.weights.to(dt)), inputInfo)
        agg = agg.div(inputInfo.dd1.to(dt))
        return agg + torch.mm(X, self.weights1.to(dt))


# ---------------------------------------------------------------------------
# GAT, multi-head v3 chain (end2end_head/gat_final/mgat_csr/mgat_conv.py:14-198)
# ---------------------------------------------------------------------------
class MGATFunction_multi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X_prime, a0, a1, inputInfo):
        ctx.inputInfo = inputInfo
        ctx.save_for_backward(X_prime, a0, a1)
        return ATT_SDDMM_v3.att_fp16_h_nnz(inputInfo.row_pointers, inputInfo.column_index,
                                           inputInfo.degrees, inputInfo.window, X_prime, a0, a1,
                                           inputInfo.max, inputInfo.num_edges)[0]

    @staticmethod
    def backward(ctx, att_grad):
        X_prime, a0, a1 = ctx.saved_tensors
        inputInfo = ctx.inputInfo
        att_grad = att_grad.contiguous()
        # col_sum[i] = sum of att_grad over edges (j, i) (mirrored map);
        # row_sum[i] = sum over edges (i, j).  att = X'_i.a0 + X'_j.a1, so
        # row sums pair with a0 and column sums with a1.  The reference names
        # these a0_tmp / a1_tmp and pairs them the other way round, and merges
        # both into one outer product (mgat_conv.py:42-67), which is exact only
        # for a0 == a1; this restatement keeps the exact pairing.
        col_sum = ATT_SpMM_v3.spmm_fp16_h_m_rowsum(
            inputInfo.row_pointers, inputInfo.degrees_trans, att_grad, inputInfo.window,
            inputInfo.automic, inputInfo.num_nodes_ori)[0].half()
        row_sum = ATT_SpMM_v3.spmm_fp16_h_m_rowsum(
            inputInfo.row_pointers, inputInfo.degrees, att_grad, inputInfo.window,
            inputInfo.automic, inputInfo.num_nodes_ori)[0].half()
        a0_grad = torch.bmm(row_sum.transpose(1, 2), X_prime)
        a1_grad = torch.bmm(col_sum.transpose(1, 2), X_prime)
        X_prime_grad = torch.bmm(row_sum, a0) + torch.bmm(col_sum, a1)
        return X_prime_grad, a0_grad, a1_grad, None


class MGATSpmm_multi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, att, X_prime, inputInfo):
        ctx.inputInfo = inputInfo
        ctx.save_for_backward(att, X_prime)
        return ATT_SpMM_v3.spmm_fp16_m_h(inputInfo.row_pointers, inputInfo.column_index,
                                         inputInfo.degrees, att, inputInfo.window,
                                         inputInfo.automic, X_prime)[0]

    @staticmethod
    def backward(ctx, X_prime_grad):
        att, X_prime = ctx.saved_tensors
        inputInfo = ctx.inputInfo
        X_prime_grad = X_prime_grad.half().permute(1, 0, 2).contiguous()
        d_X_prime = ATT_SpMM_v3.spmm_fp16_h_m(inputInfo.row_pointers, inputInfo.column_index,
                                              inputInfo.degrees_trans, att, inputInfo.window,
                                              inputInfo.automic, X_prime_grad)[0].half()
        d_att = ATT_SDDMM_v3.sddmm_fp16_h_nnz(inputInfo.row_pointers, inputInfo.column_index,
                                              inputInfo.degrees, inputInfo.window, X_prime_grad,
                                              X_prime, inputInfo.max, inputInfo.num_edges)[0]
        return d_att, d_X_prime, None


class MGATSpmm1_multi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, att, inputInfo):
        ctx.inputInfo = inputInfo
        return ATT_SpMM_v3.spmm_fp16_m_h_rowsum(inputInfo.row_pointers, inputInfo.degrees, att,
                                                inputInfo.window, inputInfo.automic,
                                                inputInfo.num_nodes_ori)[0]

    @staticmethod
    def backward(ctx, X_prime_grad):
        inputInfo = ctx.inputInfo
        d_att = ATT_SDDMM_v3.sddmm_fp16_ones_h_nnz(inputInfo.row_pointers,
                                                   inputInfo.column_index, inputInfo.degrees,
                                                   inputInfo.window, X_prime_grad.half(),
                                                   inputInfo.max, inputInfo.num_edges)[0]
        return d_att, None


class GATConv_multi(nn.Module):
    """The reference's multi-head GAT layer over the separate drop-in ops
    (fp16): att -> LeakyReLU -> exp -> row sums -> SpMM -> divide."""

    def __init__(self, input_dim, output_dim, dropout, alpha, head):
        super().__init__()
        gain = nn.init.calculate_gain("relu")
        self.fc = nn.Linear(input_dim, output_dim * head, bias=False)
        nn.init.xavier_normal_(self.fc.weight.data, gain=gain)
        self.a0 = nn.Parameter(torch.zeros(head, 1, output_dim))
        self.a1 = nn.Parameter(torch.zeros(head, 1, output_dim))
        nn.init.xavier_normal_(self.a0.data, gain=gain)
        nn.init.xavier_normal_(self.a1.data, gain=gain)
        self.output_dim, self.head = output_dim, head
        self.dropout = nn.Dropout(dropout)
        self.leakyrelu = nn.LeakyReLU(alpha)

    def forward(self, X, inputInfo):
        X_prime = F.linear(X.half(), self.fc.weight.half())
        X_prime = X_prime.view(-1, self.head, self.output_dim).permute(1, 0, 2).contiguous()
        att = MGATFunction_multi.apply(X_prime, self.a0.half(), self.a1.half(), inputInfo)
        att = torch.exp(self.leakyrelu(att))
        rows_sum = MGATSpmm1_multi.apply(att, inputInfo)
        att = self.dropout(att)
        h_prime = MGATSpmm_multi.apply(att, X_prime, inputInfo)
        return h_prime.div(rows_sum)  # [M, h, F]


# ---------------------------------------------------------------------------
# GATv2, multi-head (end2end_head/gatv2_final/mgat_csr/mgat_conv.py:14-196)
# ---------------------------------------------------------------------------
class MGATv2Function_multi(torch.autograd.Function):
    """att[h][e(i,j)] = X0'[h][i].a[h] + X1'[h][j].a[h] (attv2_fp16_h_nnz,
    mgat_conv.py:14-31) with its backward (mgat_conv.py:33-66): the row sums
    of the incoming gradient pair with X0' and the column sums (mirrored map)
    with X1'."""

    @staticmethod
    def forward(ctx, X_prime0, X_prime1, a0, inputInfo):
        ctx.inputInfo = inputInfo
        ctx.save_for_backward(X_prime0, X_prime1, a0)
        return ATT_SDDMM_v3.attv2_fp16_h_nnz(inputInfo.row_pointers, inputInfo.column_index,
                                             inputInfo.degrees, inputInfo.window, X_prime0,
                                             X_prime1, a0, inputInfo.max,
                                             inputInfo.num_edges)[0]

    @staticmethod
    def backward(ctx, att_grad):
        X_prime0, X_prime1, a0 = ctx.saved_tensors
        inputInfo = ctx.inputInfo
        att_grad = att_grad.contiguous()
        col_sum = ATT_SpMM_v3.spmm_fp16_h_m_rowsum(
            inputInfo.row_pointers, inputInfo.degrees_trans, att_grad, inputInfo.window,
            inputInfo.automic, inputInfo.num_nodes_ori)[0].half()
        row_sum = ATT_SpMM_v3.spmm_fp16_h_m_rowsum(
            inputInfo.row_pointers, inputInfo.degrees, att_grad, inputInfo.window,
            inputInfo.automic, inputInfo.num_nodes_ori)[0].half()
        a_grad = (torch.bmm(row_sum.transpose(1, 2), X_prime0)
                  + torch.bmm(col_sum.transpose(1, 2), X_prime1))
        return torch.bmm(row_sum, a0), torch.bmm(col_sum, a0), a_grad, None


class GATv2Conv_multi(nn.Module):
    """The reference's multi-head GATv2 layer over the separate drop-in ops
    (fp16; mgat_conv.py:151-196): two projections, each through LeakyReLU;
    attv2 logits; per-head min-max scaling over all edges; exp; row sums;
    SpMM of the edge values with X1'; divide."""

    def __init__(self, input_dim, output_dim, dropout, alpha, head):
        super().__init__()
        gain = nn.init.calculate_gain("relu")
        self.fc0 = nn.Linear(input_dim, output_dim * head, bias=False)
        nn.init.xavier_normal_(self.fc0.weight.data, gain=gain)
        self.fc1 = nn.Linear(input_dim, output_dim * head, bias=False)
        nn.init.xavier_normal_(self.fc1.weight.data, gain=gain)
        self.a0 = nn.Parameter(torch.zeros(head, 1, output_dim))
        nn.init.xavier_normal_(self.a0.data, gain=gain)
        self.output_dim, self.head = output_dim, head
        self.dropout = nn.Dropout(dropout)
        self.leakyrelu = nn.LeakyReLU(alpha)

    def forward(self, X, inputInfo):
        H, Fo = self.head, self.output_dim
        X_prime0 = F.linear(X.half(), self.fc0.weight.half())
        X_prime1 = F.linear(X.half(), self.fc1.weight.half())
        X_prime0 = self.leakyrelu(X_prime0.view(-1, H, Fo).permute(1, 0, 2).contiguous())
        X_prime1 = self.leakyrelu(X_prime1.view(-1, H, Fo).permute(1, 0, 2).contiguous())
        att = MGATv2Function_multi.apply(X_prime0, X_prime1, self.a0.half(), inputInfo)
        max_value = torch.max(att, dim=1, keepdim=True)[0]
        min_value = torch.min(att, dim=1, keepdim=True)[0]
        att = torch.exp((att - min_value) / (max_value - min_value))
        rows_sum = MGATSpmm1_multi.apply(att, inputInfo)
        att = self.dropout(att)
        h_prime = MGATSpmm_multi.apply(att, X_prime1, inputInfo)
        return h_prime.div(rows_sum)  # [M, h, F]


class FusedGATConv(nn.Module):
    """Multi-head GAT layer on the fused kernels (att_gb300.gat.GATAttention),
    any output width (padded internally to a supported 32/64/128)."""

    def __init__(self, input_dim, output_dim, heads=1, alpha=0.2, dtype=torch.bfloat16):
        super().__init__()
        gain = nn.init.calculate_gain("relu")
        self.W = nn.Parameter(torch.empty(input_dim, heads * output_dim))
        nn.init.xavier_normal_(self.W, gain=gain)
        self.a0 = nn.Parameter(torch.empty(heads, output_dim))
        self.a1 = nn.Parameter(torch.empty(heads, output_dim))
        nn.init.xavier_normal_(self.a0, gain=gain)
        nn.init.xavier_normal_(self.a1, gain=gain)
        self.heads, self.out_dim, self.alpha, self.dtype = heads, output_dim, alpha, dtype
        self.F_pad = next(f for f in (32, 64, 128, 1 << 30) if f >= output_dim)
        if self.F_pad > 128:
            raise ValueError("fused GAT layers support up to 128 features per head")

    def forward(self, X, graph):
        N, H, Fo, Fp = graph.n_nodes, self.heads, self.out_dim, self.F_pad
        Xp = torch.mm(X.to(self.dtype), self.W.to(self.dtype))
        a0, a1 = self.a0, self.a1
        if Fp != Fo:
            Xp = F.pad(Xp.view(N, H, Fo), (0, Fp - Fo)).reshape(N, H * Fp)
            a0 = F.pad(a0, (0, Fp - Fo))
            a1 = F.pad(a1, (0, Fp - Fo))
        out = _gat.GATAttention.apply(Xp.contiguous(), a0, a1, graph, H, self.alpha)
        out = out.view(N, H, Fp)
        return out[:, :, :Fo] if Fp != Fo else out  # [N, H, F]


class GATNet(nn.Module):
    """2+-layer GAT (the reference's Net, gat_mgnn.py:17-40): hidden layers
    concatenate their heads and pass through ELU; the output layer has one
    head; log_softmax.  ``impl="fused"`` runs att_gb300's fused kernels
    (bf16), ``impl="dropin"`` the reference's chain of separate ops (fp16)."""

    def __init__(self, in_feats, hidden, out_feats, heads=4, num_layers=2, alpha=0.2,
                 impl="fused", dtype=torch.bfloat16):
        super().__init__()
        self.impl = impl
        dims = [in_feats] + [hidden * heads] * (num_layers - 1)
        if impl == "fused":
            self.layers = nn.ModuleList(
                [FusedGATConv(dims[i], hidden, heads, alpha, dtype) for i in range(num_layers - 1)]
                + [FusedGATConv(dims[-1], out_feats, 1, alpha, dtype)])
        else:
            self.layers = nn.ModuleList(
                [GATConv_multi(dims[i], hidden, 0.0, alpha, heads) for i in range(num_layers - 1)]
                + [GATConv_multi(dims[-1], out_feats, 0.0, alpha, 1)])

    def forward(self, X, inputInfo):
        g = inputInfo.fused_graph() if self.impl == "fused" else inputInfo
        x = X
        for layer in self.layers[:-1]:
            x = F.elu(layer(x, g).flatten(1).float())
        x = self.layers[-1](x, g).flatten(1).float()
        return F.log_softmax(x[: inputInfo.num_nodes_ori], dim=1)
