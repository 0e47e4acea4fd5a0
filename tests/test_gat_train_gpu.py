"""Fused GAT backward: gradients of the additive multi-head layer against
(1) torch autograd of the FP64 restatement in the oracle and (2) FP64 central
finite differences along random directions.  Tolerance 1e-2 normwise relative
(bf16/fp16 operands, fp32 accumulation)."""
import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu


def _setup(n, deg, H, F, seed, dtype, symmetric=True):
    from att_gb300 import gat, graphs
    if symmetric:
        rp, col = graphs.chung_lu(n, deg, 2.0, seed=seed)
    else:
        rpn, coln = graphs.random_csr(n, n, deg, seed=seed)
        rp, col = torch.from_numpy(rpn), torch.from_numpy(coln)
    G = gat.GATGraph(rp, col, parts_per_chunk=2)
    g = torch.Generator().manual_seed(seed)
    Xp = ((torch.rand(n, H * F, generator=g) * 2 - 1)).to(dtype)
    a0 = (torch.rand(H, F, generator=g) - 0.5) * 0.5
    a1 = (torch.rand(H, F, generator=g) - 0.5) * 0.5
    Gout = torch.randn(n, H * F, generator=g)
    return G, rp, col, Xp, a0, a1, Gout


@pytest.mark.parametrize("H,F,dtype,sym", [(1, 64, torch.float16, True), (4, 64, torch.bfloat16, True),
                                           (2, 32, torch.bfloat16, False), (2, 128, torch.float16, True)])
def test_backward_matches_fp64_autograd(cuda, H, F, dtype, sym):
    from att_gb300 import gat
    n = 1200
    G, rp, col, Xp, a0, a1, Gout = _setup(n, 14, H, F, 3 + H, dtype, sym)
    x = Xp.cuda().requires_grad_(True)
    A0 = a0.cuda().requires_grad_(True)
    A1 = a1.cuda().requires_grad_(True)
    out = gat.GATAttention.apply(x, A0, A1, G, H, 0.2)
    (out * Gout.cuda()).sum().backward()
    xr = Xp.double().requires_grad_(True)
    a0r = a0.double().requires_grad_(True)
    a1r = a1.double().requires_grad_(True)
    ref = oracle.gat_add_layer_torch(rp, col, xr, a0r, a1r)
    (ref * Gout.double()).sum().backward()
    assert oracle.rel_err(out.detach().cpu().numpy(), ref.detach().numpy()) <= 1e-2
    for got, want in ((x.grad, xr.grad), (A0.grad, a0r.grad), (A1.grad, a1r.grad)):
        err = oracle.rel_err(got.float().cpu().numpy(), want.numpy())
        assert err <= 1e-2, err


def test_backward_matches_fp64_finite_differences(cuda):
    from att_gb300 import gat
    n, H, F = 400, 2, 32
    G, rp, col, Xp, a0, a1, Gout = _setup(n, 10, H, F, 11, torch.float16)
    x = Xp.cuda().requires_grad_(True)
    A0 = a0.cuda().requires_grad_(True)
    A1 = a1.cuda().requires_grad_(True)
    out = gat.GATAttention.apply(x, A0, A1, G, H, 0.2)
    (out * Gout.cuda()).sum().backward()

    def loss(xv, a0v, a1v):
        with torch.no_grad():
            return float((oracle.gat_add_layer_torch(rp, col, xv, a0v, a1v) * Gout.double()).sum())

    # reference autograd gradient, for the failure message
    xr = Xp.double().requires_grad_(True)
    a0r = a0.double().requires_grad_(True)
    a1r = a1.double().requires_grad_(True)
    (oracle.gat_add_layer_torch(rp, col, xr, a0r, a1r) * Gout.double()).sum().backward()
    g = torch.Generator().manual_seed(5)
    x0, b0, b1 = Xp.double(), a0.double(), a1.double()
    # a small step keeps the central difference off LeakyReLU's kink at 0
    eps = 1e-6
    for which in range(3):
        v = [torch.zeros_like(x0), torch.zeros_like(b0), torch.zeros_like(b1)]
        v[which] = torch.randn(v[which].shape, generator=g, dtype=torch.float64)
        fd = (loss(x0 + eps * v[0], b0 + eps * v[1], b1 + eps * v[2]) -
              loss(x0 - eps * v[0], b0 - eps * v[1], b1 - eps * v[2])) / (2 * eps)
        grads = [x.grad.double().cpu(), A0.grad.double().cpu(), A1.grad.double().cpu()]
        refg = [xr.grad, a0r.grad, a1r.grad]
        an = float((grads[which] * v[which]).sum())
        ra = float((refg[which] * v[which]).sum())
        assert abs(an - fd) <= 1e-2 * max(abs(fd), 1.0), (which, an, fd, ra)
