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


@pytest.mark.parametrize("H,F,dtype", [(1, 40, torch.bfloat16), (4, 64, torch.bfloat16),
                                       (5, 64, torch.float16), (3, 24, torch.float16)])
def test_grad_prepare_and_finish_kernels(cuda, H, F, dtype):
    """att_gat_grad_prepare / att_gat_grad_finish through the C ABI against
    their definitions in FP64: c = dout . out per head, dout = hi + lo (hi the
    16-bit rounding, lo the rounding of the remainder), dX = dtype(dXp + ds0 a0
    + ds1 a1) and da0/da1 = sum_n ds X'.  Covers H*F below, at and above the
    256-column block (40, 256, 320) and one that does not divide it (72)."""
    from att_gb300 import _lib
    from att_gb300.ops import _DT, _p, _stream
    n = 3001
    g = torch.Generator().manual_seed(H * 100 + F)
    HF = H * F
    dout = torch.randn(n, HF, generator=g).cuda()
    out = torch.randn(n, HF, generator=g).cuda()
    hi = torch.empty(n, HF, dtype=dtype, device="cuda")
    lo = torch.empty_like(hi)
    c = torch.full((H, n), float("nan"), device="cuda")
    _lib.call("att_gat_grad_prepare", _p(dout), HF, _p(out), HF, n, H, F, _p(hi), _p(lo),
              _DT[dtype], HF, _p(c), _stream())
    torch.cuda.synchronize()
    c_ref = (dout.double().view(n, H, F) * out.double().view(n, H, F)).sum(-1).t()
    assert oracle.rel_err(c.cpu().numpy(), c_ref.cpu().numpy()) <= 1e-6
    assert torch.equal(hi, dout.to(dtype))
    assert torch.equal(lo, (dout - dout.to(dtype).float()).to(dtype))
    # finish
    dXp = torch.randn(n, HF, generator=g).cuda()
    ds0 = torch.randn(H, n, generator=g).cuda()
    ds1 = torch.randn(H, n, generator=g).cuda()
    a0 = torch.randn(H, F, generator=g).cuda()
    a1 = torch.randn(H, F, generator=g).cuda()
    Xp = torch.randn(n, HF, generator=g).to(dtype).cuda()
    dX = torch.empty(n, HF, dtype=dtype, device="cuda")
    da0 = torch.zeros(H, F, device="cuda")
    da1 = torch.zeros(H, F, device="cuda")
    _lib.call("att_gat_grad_finish", _p(dXp), HF, _p(ds0), _p(ds1), _p(a0), _p(a1), _p(Xp),
              _DT[dtype], HF, n, H, F, _p(dX), HF, _p(da0), _p(da1), _stream())
    torch.cuda.synchronize()
    X3 = Xp.double().view(n, H, F)
    dX_ref = (dXp.double().view(n, H, F) + ds0.double().t()[:, :, None] * a0.double()[None]
              + ds1.double().t()[:, :, None] * a1.double()[None]).reshape(n, HF)
    # one rounding to the 16-bit type: within its half-ulp (2^-8 bf16, 2^-11 fp16) relative
    tol = 2.0 ** -8 if dtype == torch.bfloat16 else 2.0 ** -11
    d = (dX.double() - dX_ref).abs() <= tol * dX_ref.abs() + 1e-6
    assert bool(d.all())
    da0_ref = torch.einsum("hn,nhf->hf", ds0.double(), X3)
    da1_ref = torch.einsum("hn,nhf->hf", ds1.double(), X3)
    assert oracle.rel_err(da0.cpu().numpy(), da0_ref.cpu().numpy()) <= 1e-5
    assert oracle.rel_err(da1.cpu().numpy(), da1_ref.cpu().numpy()) <= 1e-5
