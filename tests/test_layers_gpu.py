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


def test_gatv2_layer_forward_backward_vs_fp64(cuda):
    """GATv2Conv_multi (end2end_head/gatv2_final/mgat_csr/mgat_conv.py:151-196)
    over the drop-ins: output and the gradients of both projections and of
    the attention vector against FP64 autograd of the oracle's restatement."""
    from att_gb300 import layers
    n, Fi, Fo, H = 700, 32, 32, 2
    rows, cols, rp, col = _edges(n, 10, 6)
    info = layers.GATInput(rows, cols, n)
    torch.manual_seed(1)
    conv = layers.GATv2Conv_multi(Fi, Fo, 0.0, 0.2, H).cuda()
    X = (torch.rand(n, Fi, generator=torch.Generator().manual_seed(7)) - 0.5).half().cuda()
    y = conv(X, info)
    assert y.shape == (n, H, Fo)
    G = torch.randn(n, H, Fo, generator=torch.Generator().manual_seed(8)).cuda()
    (y.float() * G).sum().backward()
    W0 = conv.fc0.weight.detach().t().half().double().cpu().requires_grad_(True)
    W1 = conv.fc1.weight.detach().t().half().double().cpu().requires_grad_(True)
    a = conv.a0.detach().half().double().cpu().requires_grad_(True)
    ref = oracle.gatv2_layer_torch(rp, col, X.double().cpu(), W0, W1, a, 0.2)
    (ref * G.double().cpu()).sum().backward()
    assert oracle.rel_err(y.detach().float().cpu().numpy(), ref.detach().numpy()) <= 1e-2
    for got, want in ((conv.fc0.weight.grad.t(), W0.grad), (conv.fc1.weight.grad.t(), W1.grad),
                      (conv.a0.grad, a.grad)):
        err = oracle.rel_err(got.float().cpu().numpy(), want.numpy())
        assert err <= 2e-2, err


def test_v4_attention_vector_helpers(cuda):
    """ATT_SpMM_v4.bmm_v_m / bmm_v_v against their caller's math
    (end2end_acc/gat_final/mgat_csr/mgat_conv.py:82,94), in both node-vector
    layouts."""
    from att_gb300.compat import ATT_SpMM_v4
    g = torch.Generator().manual_seed(3)
    h, M, F = 4, 300, 64
    a0t = torch.randn(h, M, 1, generator=g).half().cuda()
    a1t = torch.randn(h, M, 1, generator=g).half().cuda()
    X = torch.randn(h, F, M, generator=g).half().cuda()
    ta = torch.randn(h, 1, F, generator=g).half().cuda()
    want0 = torch.einsum("hm,hfm->hf", a0t[..., 0].double(), X.double())[:, None, :]
    want1 = torch.einsum("hm,hfm->hf", a1t[..., 0].double(), X.double())[:, None, :]
    tg = a0t + a1t
    want_v = (tg[..., 0].double().T[:, :, None] * ta[:, 0].double()[None]).reshape(M, h * F)
    for lay in (lambda v: v, lambda v: v.transpose(1, 2).contiguous()):
        g0, g1 = ATT_SpMM_v4.bmm_v_m(lay(a0t), lay(a1t), X)
        assert g0.shape == (h, 1, F) and g1.shape == (h, 1, F)
        assert oracle.rel_err(g0.double().cpu().numpy(), want0.cpu().numpy()) <= 1e-2
        assert oracle.rel_err(g1.double().cpu().numpy(), want1.cpu().numpy()) <= 1e-2
        v = ATT_SpMM_v4.bmm_v_v(lay(tg), ta)[0]
        assert v.shape == (M, h * F)
        assert oracle.rel_err(v.double().cpu().numpy(), want_v.cpu().numpy()) <= 1e-2
