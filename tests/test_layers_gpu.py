"""Model-level glue on the GPU: the reference's GCN / GraphSAGE / GAT layers
over the drop-ins, and the fused GAT network.  Tolerances: fp16 1e-2
normwise relative against FP64."""
import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu


def _edges(n, deg, seed):
    from att_gb300 import graphs
    rp, col = graphs.chung_lu(n, deg, 2.1, seed=seed)
    rows = torch.repeat_interleave(torch.arange(n), (rp[1:] - rp[:-1]).long())
    return rows, col.long(), rp, col


def _ahat(rp, col, n):
    d = torch.rsqrt((rp[1:] - rp[:-1]).float()).half()
    rows = oracle.csr_rows(rp.numpy())
    v = (d[rows].float() * d[col.long()].float()).half().double().numpy()
    import scipy.sparse as sp
    return sp.csr_matrix((v, (rows, col.numpy())), shape=(n, n))


def test_gcn_layer_forward_backward(cuda):
    from att_gb300 import layers
    n, Fi, Fo = 1000, 64, 32
    rows, cols, rp, col = _edges(n, 10, 1)
    info = layers.GCNInput(rows, cols, n)
    conv = layers.GCNConv(Fi, Fo).cuda()
    X = torch.rand(n, Fi, generator=torch.Generator().manual_seed(0)).half().cuda()
    X.requires_grad_(True)
    Y = conv(X, info)
    G = torch.randn(n, Fo, generator=torch.Generator().manual_seed(1)).cuda()
    (Y.float() * G).sum().backward()
    A = _ahat(rp, col, n)
    Wd = conv.weights.detach().half().double().cpu().numpy()
    Xd = X.detach().double().cpu().numpy()
    ref = A @ (Xd @ Wd)
    assert oracle.rel_err(Y.detach().float().cpu().numpy(), ref) <= 1e-2
    Gd = G.double().cpu().numpy()
    dX = (A.T @ Gd) @ Wd.T
    dW = Xd.T @ (A.T @ Gd)
    assert oracle.rel_err(X.grad.float().cpu().numpy(), dX) <= 1e-2
    assert oracle.rel_err(conv.weights.grad.float().cpu().numpy(), dW) <= 1e-2


def test_sage_layer_forward(cuda):
    from att_gb300 import layers
    n, Fi, Fo = 800, 32, 32
    rows, cols, rp, col = _edges(n, 8, 2)
    info = layers.GCNInput(rows, cols, n)
    conv = layers.SAGEConv(Fi, Fo).cuda()
    X = torch.rand(n, Fi, generator=torch.Generator().manual_seed(0)).half().cuda()
    Y = conv(X, info)
    A = _ahat(rp, col, n)
    W = conv.weights.detach().half().double().cpu().numpy()
    W1 = conv.weights1.detach().half().double().cpu().numpy()
    Xd = X.double().cpu().numpy()
    deg = np.maximum(np.diff(rp.numpy()), 1)[:, None]
    ref = (A @ (Xd @ W)) / deg + Xd @ W1
    assert oracle.rel_err(Y.detach().float().cpu().numpy(), ref) <= 1e-2


def test_dropin_and_fused_gat_layers_agree(cuda):
    from att_gb300 import layers
    n, Fi, Fo, H = 900, 64, 32, 2
    rows, cols, rp, col = _edges(n, 12, 3)
    info = layers.GATInput(rows, cols, n)
    torch.manual_seed(0)
    plain = layers.GATConv_multi(Fi, Fo, 0.0, 0.2, H).cuda()
    fused = layers.FusedGATConv(Fi, Fo, H, 0.2, dtype=torch.float16).cuda()
    with torch.no_grad():
        fused.W.copy_(plain.fc.weight.t())
        fused.a0.copy_(plain.a0[:, 0, :])
        fused.a1.copy_(plain.a1[:, 0, :])
    X = (torch.rand(n, Fi, generator=torch.Generator().manual_seed(4)) * 0.5).half().cuda()
    with torch.no_grad():
        y_plain = plain(X, info)[:n].float()
        y_fused = fused(X, info.fused_graph()).float()
        assert oracle.rel_err(y_fused.cpu().numpy(), y_plain.cpu().numpy()) <= 1e-2
        # and both against FP64
        Wh = plain.fc.weight.t().half().float()
        Xp = torch.mm(X.float(), Wh).half().double().cpu()
        ref = oracle.gat_add_layer_torch(rp, col, Xp, plain.a0[:, 0, :].half().double().cpu(),
                                         plain.a1[:, 0, :].half().double().cpu())
        assert oracle.rel_err(y_fused.reshape(n, -1).cpu().numpy(), ref.numpy()) <= 1e-2


def test_fused_gat_training_lowers_loss(cuda):
    from att_gb300 import layers
    n = 2000
    rows, cols, rp, col = _edges(n, 12, 5)
    info = layers.GATInput(rows, cols, n)
    g = torch.Generator().manual_seed(0)
    X = torch.rand(n, 128, generator=g).bfloat16().cuda()
    y = torch.randint(0, 40, (n,), generator=g).cuda()
    torch.manual_seed(0)
    net = layers.GATNet(128, 64, 40, heads=4, impl="fused").cuda()
    opt = torch.optim.Adam(net.parameters(), lr=2e-3)
    losses = []
    for _ in range(12):
        loss = torch.nn.functional.nll_loss(net(X, info), y)
        opt.zero_grad()
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
    assert all(np.isfinite(losses)) and min(losses[6:]) < losses[0], losses
