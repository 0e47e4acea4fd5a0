"""Parity on the benchmarked workloads at their full sizes.

Each test builds the same seeded synthetic graph, format and features as the
bench workload of that name (``bench.py``), runs the GPU path, and checks it
against the oracle:

* block conversion: every output array bit-exact against the C restatement
  (``oracle/block_oracle.c``), on the whole graph;
* numeric results: normwise relative error (max|err| / max|ref|) against FP64
  on the host, over all rows where the host finishes in seconds, else over a
  seeded row sample that includes every row of the windows holding the
  longest rows (hub windows, split into the most parts).

Tolerances: fp16 / bf16 1e-2, fp32 (3xTF32) 1e-4 against FP64 of the kernel's
own inputs.  FP8 (e4m3 features with per-row fp32 scales): 1e-2 against FP64
of the dequantized features (the kernel's arithmetic, same norm as the other
forms); against FP64 of the unquantized features 3e-2 in the Frobenius norm
and 2^-4 max-normwise -- on a row whose only edge is its self-loop Y equals X,
so the max-normwise error there is the e4m3 rounding of X itself (3 mantissa
bits: up to 1/32..1/16 of the value), which no kernel on e4m3 inputs can
undercut.
"""
import gc

import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu


def _free():
    gc.collect()
    torch.cuda.empty_cache()


def _bits(a):
    a = np.asarray(a)
    if a.dtype == np.float16:
        return a.view(np.uint16)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    return a


def _check_format(fmt, rowptr, col, deg, W, w, P, emit_empty=False):
    o = oracle.block_convert(rowptr, col, deg, W, w, P, emit_empty=emit_empty)
    for name, t in (("rowptr", fmt.rowptr), ("col", fmt.col), ("val", fmt.val),
                    ("window", fmt.window_of_part), ("atomic", fmt.atomic)):
        got = _bits(t.cpu().numpy())
        want = _bits(o[name])
        assert got.shape == want.shape, (name, got.shape, want.shape)
        assert np.array_equal(got, want), name
    return o


def _host(wl):
    rp = wl.rowptr.cpu().numpy()
    col = wl.colidx.cpu().numpy()
    deg = wl.deg.cpu().numpy()
    return rp, col, deg


# ---------------------------------------------------------------------------
# GCN aggregation, 16,384 nodes (gamma 2.1, mean degree 10, seed 0, F = 64)
# ---------------------------------------------------------------------------
def test_gcn16k_conversion_and_spmm_all_rows(cuda):
    import bench
    from att_gb300 import ops
    from att_gb300.compat import SpMM_sr_bcrs
    wl = bench.SpmmGcn16k("cuda")
    rp, col, deg = _host(wl)
    n, F = wl.n, wl.F
    assert n == 16_384 and F == 64
    _check_format(wl.fmt, rp, col, deg, 8, 8, 32)
    vals = oracle.gcn_values(rp, col, deg).astype(np.float64)
    X = wl.X.double().cpu().numpy()
    ref = oracle.spmm_csr_fp64(rp, col, vals, X, n)
    f = wl.fmt
    Y = SpMM_sr_bcrs.forward_fp16_gnn(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, wl.X,
                                      rp.shape[0] - 1, F, n)[0]
    assert Y.shape == (n, F)
    assert oracle.rel_err(Y.cpu().numpy(), ref) <= 1e-2
    # 16-row windows over the same graph
    f16 = ops.block_convert(wl.rowptr, wl.colidx, wl.deg, window=16, wide=8, part=32)
    _check_format(f16, rp, col, deg, 16, 8, 32)
    Y16 = ops.spmm(f16.rowptr, f16.col, f16.val, f16.window_of_part, f16.atomic, wl.X, n,
                   window=16, wide=8)
    assert oracle.rel_err(Y16.cpu().numpy(), ref) <= 1e-2


# ---------------------------------------------------------------------------
# SpMM precision sweep, 2,449,029 nodes (gamma 2.2, mean degree 25, seed 2)
# ---------------------------------------------------------------------------
def _products_rows(wl):
    return oracle.sample_rows(wl.rowptr.cpu().numpy(), wl.n, 20_000, 64, seed=7)


def test_products_conversion_bit_exact_whole_graph(cuda):
    """All five arrays of the 63.7M-edge graph's format; its hub windows split
    into thousands of parts (example.cpp:112-152)."""
    import bench
    wl = bench.SpmmProducts("cuda")
    rp, col, deg = _host(wl)
    o = _check_format(wl.fmt, rp, col, deg, 8, 8, 32)
    parts_per_window = np.bincount(o["window"])
    assert parts_per_window.max() > 1000  # the hub windows are exercised
    del wl
    _free()


@pytest.mark.parametrize("form", ["fp16", "bf16", "fp8"])
def test_products_spmm_vs_fp64_sampled_rows(cuda, form):
    import bench
    from att_gb300 import ops
    cls = {"fp16": bench.SpmmProducts, "bf16": bench.SpmmProductsBF16,
           "fp8": bench.SpmmProductsFP8}[form]
    wl = cls("cuda")
    f = wl.fmt
    Y = ops.spmm(f.rowptr, f.col, wl.val, f.window_of_part, f.atomic, wl.Xk, wl.n,
                 x_scale=wl.x_scale)
    rows = _products_rows(wl)
    got = Y[torch.from_numpy(rows).cuda()].double().cpu().numpy()
    rp, col, deg = _host(wl)
    ev = oracle.gcn_values(rp, col, deg).astype(np.float64)
    if form == "bf16":
        ev = torch.from_numpy(ev).to(torch.bfloat16).double().numpy()
    # the kernel's own inputs
    if form == "fp8":
        Xin = (wl.Xk.float() * wl.x_scale[:, None]).double().cpu().numpy()
    else:
        Xin = wl.Xk.double().cpu().numpy()
    ref = oracle.spmm_rows_fp64(rp, col, ev, Xin, rows)
    assert oracle.rel_err(got, ref) <= 1e-2, form
    if form == "fp8":
        # against the unquantized features: Frobenius 3e-2, max-normwise
        # bounded by the e4m3 rounding of X (see the module docstring)
        ref_u = oracle.spmm_rows_fp64(rp, col, ev, wl.Xf64.cpu().numpy(), rows)
        assert oracle.rel_err_fro(got, ref_u) <= 3e-2
        assert oracle.rel_err(got, ref_u) <= 2.0 ** -4
    del wl, Y
    _free()


# ---------------------------------------------------------------------------
# GAT layer, 232,965 nodes, ~114M edges (gamma 1.9, seed 1, F = 64, 1 head)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("form", ["fp16", "tf32"])
def test_reddit_gat_layer_vs_fp64_sampled_rows(cuda, form):
    import bench
    cls = bench.GatReddit if form == "fp16" else bench.GatRedditTF32
    wl = cls("cuda")
    Xp = torch.mm(wl.X, wl.W)
    out, _, _ = wl.G.attention(Xp)
    rp = wl.rowptr.cpu().numpy()
    col = wl.colidx.cpu().numpy()
    rows = oracle.sample_rows(rp, wl.n, 2000, 32, seed=9)
    got = out[torch.from_numpy(rows).cuda()].double().cpu().numpy()
    ref = oracle.gat_dot_rows_fp64(rp, col, Xp.double().cpu().numpy(), rows)
    tol = 1e-2 if form == "fp16" else 1e-4
    assert oracle.rel_err(got, ref) <= tol, form
    del wl, out, Xp
    _free()


def test_reddit_gcn_conversion_bit_exact_whole_graph(cuda):
    """The 114M-edge graph's GCN block format, bit-exact (its densest windows
    hold tens of thousands of columns)."""
    from att_gb300 import graphs, ops
    import bench
    c = bench.GatReddit
    rp, col = graphs.chung_lu(c.N, c.MEAN_DEG, c.GAMMA, c.SEED, device="cuda")
    rp = graphs.pad_rows(rp, 8)
    deg = graphs.gcn_degree(rp, torch.float16)
    deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg))  # padding rows
    fmt = ops.block_convert(rp, col, deg, window=8, wide=8, part=32)
    _check_format(fmt, rp.cpu().numpy(), col.cpu().numpy(), deg.cpu().numpy(), 8, 8, 32)
    del fmt, rp, col, deg
    _free()


# ---------------------------------------------------------------------------
# 2-layer GAT training graph, 169,343 nodes (mean degree 14, seed 3):
# gradients of the fused layer-1 attention (4 heads x 64, bf16)
# ---------------------------------------------------------------------------
def test_arxiv_layer1_gradients_vs_fp64_sampled_rows(cuda):
    import bench
    from att_gb300 import gat, layers
    c = bench.GatArxivTrain
    wl = c("cuda", light=True)
    n, H, Fh = wl.n, c.HEADS, c.HID
    rows_all = torch.repeat_interleave(torch.arange(n, device="cuda"),
                                       (wl.rowptr[1:] - wl.rowptr[:-1]).long())
    info = layers.GATInput(rows_all.cpu(), wl.colidx.long().cpu(), n)
    G = info.fused_graph()
    torch.manual_seed(0)
    conv = layers.FusedGATConv(c.F_IN, Fh, H, 0.2, dtype=torch.bfloat16).cuda()
    Xp = torch.mm(wl.X, conv.W.detach().to(torch.bfloat16)).contiguous()
    rp = wl.rowptr.cpu().numpy()
    col = wl.colidx.cpu().numpy()
    rows = oracle.sample_rows(rp, n, 8192, 64, seed=5)
    g = torch.Generator(device="cuda").manual_seed(5)
    R = torch.zeros(n, H * Fh, device="cuda")
    R[torch.from_numpy(rows).cuda()] = torch.randn(len(rows), H * Fh, generator=g, device="cuda")
    x = Xp.clone().requires_grad_(True)
    a0 = conv.a0.detach().clone().requires_grad_(True)
    a1 = conv.a1.detach().clone().requires_grad_(True)
    out = gat.GATAttention.apply(x, a0, a1, G, H, 0.2)
    (out * R).sum().backward()

    xr = Xp.double().cpu().requires_grad_(True)
    a0r = conv.a0.detach().double().cpu().requires_grad_(True)
    a1r = conv.a1.detach().double().cpu().requires_grad_(True)
    ref = oracle.gat_add_rows_torch(rp, col, xr, a0r, a1r, rows)
    (ref * R[torch.from_numpy(rows).cuda()].double().cpu()).sum().backward()
    got_out = out[torch.from_numpy(rows).cuda()].detach().double().cpu().numpy()
    assert oracle.rel_err(got_out, ref.detach().numpy()) <= 1e-2
    for got, want in ((x.grad, xr.grad), (a0.grad, a0r.grad), (a1.grad, a1r.grad)):
        err = oracle.rel_err(got.double().cpu().numpy(), want.numpy())
        assert err <= 1e-2, err
    del wl, info, G, out, x
    _free()


# ---------------------------------------------------------------------------
# serving: 8 requests on independent graphs (sizes log-uniform in
# [1K, 500K] nodes, mean degree uniform in [5, 50], seed 4), served together
# ---------------------------------------------------------------------------
def test_served_requests_vs_fp64(cuda):
    from att_gb300 import graphs, serving
    model = serving.GCN2(seed=4)
    pool = serving.make_graph_pool(8, 4)
    reqs = [serving.Request(i, 0.0, rp, col, X, n, nnz)
            for i, (rp, col, X, n, nnz) in enumerate(pool)]
    srv = serving.Server(model, budget=120e9, max_active=64, workers=2)
    srv.run(reqs, realtime=False)
    W1 = model.W1.double().cpu().numpy()
    W2 = model.W2.double().cpu().numpy()
    for r in reqs:
        assert r.error is None and r.out is not None
        rp8 = graphs.pad_rows(r.rowptr.clone(), 8)
        deg = graphs.gcn_degree(rp8, torch.float16)
        deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg)).numpy()
        vals = oracle.gcn_values(rp8.numpy(), r.col.numpy(), deg).astype(np.float64)
        ref = oracle.gcn2_fp64(rp8.numpy(), r.col.numpy(), vals, r.X.double().numpy(), W1, W2,
                               r.n)
        err = oracle.rel_err(r.out.numpy(), ref)
        assert err <= 1e-2, (r.rid, r.n, err)
    _free()
