"""GAT operators (ATT_Block*, ATT_SDDMM_v*, ATT_SpMM_v* drop-ins) on the GPU.

First the known answers of the reference's own op tests on the 32-row fixture
(benchmark-v3/{sddmm,spmm}-benchmark/test/...), then every op on a seeded
power-law graph against the FP64 oracle.  Tolerances (normwise relative):
fp16 1e-2, fp32 1e-4; small-integer inputs must match exactly."""
import numpy as np
import pytest
import torch

from oracle import oracle
from tests._fixture import ROW, COL

pytestmark = pytest.mark.gpu

ROWS = 30  # the reference tests use 30 feature rows for the 32-row CSR


def _fmt(W=8, w=16, P=2, trans=False):
    from att_gb300.compat import ATT_Block
    fn = ATT_Block.blockProcess_sddmm_balance_gnn_trans if trans else \
        ATT_Block.blockProcess_sddmm_balance_gnn
    return [t.cuda() for t in fn(torch.from_numpy(ROW), torch.from_numpy(COL), W, w, P)]


@pytest.mark.parametrize("dt", ["fp16", "tf32"])
def test_sddmm_reference_known_answer(cuda, dt):
    """test_sddmm_{fp16,tf32}.py:50-70 (format (8,16,2), 4 heads, dimN 125)."""
    from att_gb300.compat import ATT_SDDMM_v3
    rp, col, mp, win, at = _fmt()
    h, dimN = 4, 125
    rhs = torch.randint(1, 3, (h, ROWS, dimN))
    rhs = (rhs.half() if dt == "fp16" else rhs.float()).cuda()
    mx = torch.max(rp[2::2] - rp[:-2:2]) / 16
    fn = ATT_SDDMM_v3.sddmm_fp16_h_nnz if dt == "fp16" else ATT_SDDMM_v3.sddmm_tf32_h_nnz
    res = fn(rp, col, mp, win, rhs, rhs, mx, int(ROW[-1]))[0]
    assert res.shape == (h, 38)
    assert torch.dot(rhs[0][0].float(), rhs[0][1].float()) == res[0][0].float()
    assert torch.dot(rhs[1][0].float(), rhs[1][2].float()) == res[1][1].float()
    ref = oracle.sddmm_fp64(ROW[:ROWS + 1], COL, rhs.double().cpu().numpy(),
                            rhs.double().cpu().numpy())
    assert np.array_equal(res.double().cpu().numpy(), ref)


@pytest.mark.parametrize("dt", ["fp16", "tf32"])
def test_att_and_attv2_reference_known_answer(cuda, dt):
    """test_sddmm_{fp16,tf32}_att.py, test_sddmm_{fp16,tf32}_att_v2.py."""
    from att_gb300.compat import ATT_SDDMM_v3
    rp, col, mp, win, at = _fmt()
    h, dimN = 8, 125
    tdt = torch.float16 if dt == "fp16" else torch.float32
    rhs = torch.randint(1, 3, (h, ROWS, dimN)).to(tdt).cuda()
    rhs1 = torch.randint(1, 3, (h, ROWS, dimN)).to(tdt).cuda()
    w = torch.ones(h, 1, dimN, dtype=tdt, device="cuda")
    mx = torch.max(rp[2::2] - rp[:-2:2]) / 16
    att = getattr(ATT_SDDMM_v3, "att_%s_h_nnz" % dt)(rp, col, mp, win, rhs, w, w, mx, 38)[0]
    assert torch.dot(rhs[0][0].float(), w[0][0].float()) + \
        torch.dot(rhs[0][1].float(), w[0][0].float()) == att[0][0].float()
    assert torch.dot(rhs[1][0].float(), w[1][0].float()) + \
        torch.dot(rhs[1][2].float(), w[1][0].float()) == att[1][1].float()
    ref = oracle.att_fp64(ROW[:ROWS + 1], COL, rhs.double().cpu().numpy(),
                          w.double().cpu().numpy(), w.double().cpu().numpy())
    assert np.array_equal(att.double().cpu().numpy(), ref)
    v2 = getattr(ATT_SDDMM_v3, "attv2_%s_h_nnz" % dt)(rp, col, mp, win, rhs, rhs1, w, mx, 38)[0]
    assert torch.dot(rhs[1][0].float(), w[1][0].float()) + \
        torch.dot(rhs1[1][2].float(), w[1][0].float()) == v2[1][1].float()
    ref2 = oracle.attv2_fp64(ROW[:ROWS + 1], COL, rhs.double().cpu().numpy(),
                             rhs1.double().cpu().numpy(), w.double().cpu().numpy())
    assert np.array_equal(v2.double().cpu().numpy(), ref2)


def test_ones_reference_known_answer(cuda):
    """test_sddmm_fp16_ones.py:51-68."""
    from att_gb300.compat import ATT_SDDMM_v3
    rp, col, mp, win, at = _fmt()
    h = 4
    rhs = torch.randint(1, 5, (ROWS, h, 1)).half().cuda()
    res = ATT_SDDMM_v3.sddmm_fp16_ones_h_nnz(rp, col, mp, win, rhs, 1.0, 38)[0]
    assert rhs[0][0] == res[0][0] and rhs[1][1] == res[1][6]
    ref = oracle.ones_fp64(ROW[:ROWS + 1], rhs.double().cpu().numpy())
    assert np.array_equal(res.double().cpu().numpy(), ref)


@pytest.mark.parametrize("dt,w", [("fp16", 8), ("tf32", 4)])
def test_spmm_reference_known_answers(cuda, dt, w):
    """test_spmm_{h_m,m_h,h_m_ones,m_h_ones}.py (format (8, wide, 32), csr values 1)."""
    from att_gb300.compat import ATT_SpMM_v3
    rp, col, mp, win, at = _fmt(8, w, 32)
    tdt = torch.float16 if dt == "fp16" else torch.float32
    for head, dimN, fn in ((1, 66, "h_m"), (3, 65, "m_h")):
        vals = torch.ones(head, 38, dtype=tdt, device="cuda")
        rhs = torch.randint(1, 3, (head, ROWS, dimN)).to(tdt).cuda()
        Y = getattr(ATT_SpMM_v3, "spmm_%s_%s" % (dt, fn))(rp, col, mp, vals, win, at, rhs)[0]
        for hh in range(head):
            ref = oracle.spmm_csr_fp64(ROW[:ROWS + 1], COL, np.ones(38), rhs[hh].double().cpu().numpy())
            got = Y[hh] if fn == "h_m" else Y[:, hh, :]
            assert np.array_equal(got.double().cpu().numpy(), ref)
    for fn in ("h_m", "m_h"):
        vals = torch.ones(3, 38, dtype=tdt, device="cuda")
        rs = getattr(ATT_SpMM_v3, "spmm_%s_%s_rowsum" % (dt, fn))(rp, mp, vals, win, at, ROWS)[0]
        want = np.diff(ROW[:ROWS + 1]).astype(np.float64)
        for hh in range(3):
            got = rs[hh, :, 0] if fn == "h_m" else rs[:, hh, 0]
            assert np.array_equal(got.double().cpu().numpy(), want)


def _graph(n=2000, deg=12, seed=21):
    from att_gb300 import graphs
    rp, col = graphs.chung_lu(n, deg, 2.0, seed=seed)
    rp = graphs.pad_rows(rp, 8)
    return rp.numpy(), col.numpy(), n


@pytest.mark.parametrize("fmt_cfg", [(8, 8, 32), (8, 4, 32), (8, 16, 2), (8, 8, 3)])
@pytest.mark.parametrize("dt", ["fp16", "tf32"])
def test_ops_random_graph_vs_fp64(cuda, fmt_cfg, dt):
    from att_gb300.compat import ATT_Block_v3, ATT_SDDMM_v3, ATT_SpMM_v3
    rp_np, col_np, n = _graph()
    W, w, P = fmt_cfg
    f = [t.cuda() for t in ATT_Block_v3.blockProcess_sddmm_balance_gnn_trans(
        torch.from_numpy(rp_np), torch.from_numpy(col_np), W, w, P)]
    rp, col, mp, mpt, win, at = f
    nnz = col_np.shape[0]
    H, F = 3, 64
    tdt = torch.float16 if dt == "fp16" else torch.float32
    tol = 1e-2 if dt == "fp16" else 1e-4
    g = torch.Generator().manual_seed(5)
    X = (torch.rand(H, n, F, generator=g) * 2 - 1).to(tdt).cuda()
    Z = (torch.rand(H, n, F, generator=g) * 2 - 1).to(tdt).cuda()
    a0 = (torch.rand(H, 1, F, generator=g) - 0.5).to(tdt).cuda()
    a1 = (torch.rand(H, 1, F, generator=g) - 0.5).to(tdt).cuda()
    Xd, Zd = X.double().cpu().numpy(), Z.double().cpu().numpy()
    rpc = rp_np[: n + 1]
    mx = 1.0
    # SDDMM
    s = getattr(ATT_SDDMM_v3, "sddmm_%s_h_nnz" % dt)(rp, col, mp, win, X, Z, mx, nnz)[0]
    assert oracle.rel_err(s.cpu().numpy(), oracle.sddmm_fp64(rpc, col_np, Xd, Zd)) <= tol
    # additive attention
    e = getattr(ATT_SDDMM_v3, "att_%s_h_nnz" % dt)(rp, col, mp, win, X, a0, a1, mx, nnz)[0]
    ref_e = oracle.att_fp64(rpc, col_np, Xd, a0.double().cpu().numpy(), a1.double().cpu().numpy())
    assert oracle.rel_err(e.cpu().numpy(), ref_e) <= tol
    # SpMM with edge values, both output layouts, plain and mirrored map
    vals = (torch.rand(H, nnz, generator=g)).to(tdt).cuda()
    vd = vals.double().cpu().numpy()
    ref = oracle.spmm_edge_fp64(rpc, col_np, vd, Xd, n)
    Y = getattr(ATT_SpMM_v3, "spmm_%s_h_m" % dt)(rp, col, mp, vals, win, at, X)[0]
    assert oracle.rel_err(Y.cpu().numpy(), ref) <= tol
    Y2 = getattr(ATT_SpMM_v3, "spmm_%s_m_h" % dt)(rp, col, mp, vals, win, at, X)[0]
    assert oracle.rel_err(Y2.permute(1, 0, 2).cpu().numpy(), ref) <= tol
    # mirrored map: slot (i,j) takes the value of edge (j,i) -> A^T (symmetric pattern)
    rows = oracle.csr_rows(rpc)
    key = rows * n + col_np
    tkey = col_np.astype(np.int64) * n + rows
    order = np.argsort(key)
    pos_t = order[np.searchsorted(key[order], tkey)]
    ref_t = oracle.spmm_edge_fp64(rpc, col_np, vd[:, pos_t], Xd, n)
    Yt = getattr(ATT_SpMM_v3, "spmm_%s_h_m" % dt)(rp, col, mpt, vals, win, at, X)[0]
    assert oracle.rel_err(Yt.cpu().numpy(), ref_t) <= tol
    # row sums
    rs = getattr(ATT_SpMM_v3, "spmm_%s_h_m_rowsum" % dt)(rp, mp, vals, win, at, n)[0]
    assert oracle.rel_err(rs[:, :, 0].cpu().numpy(), oracle.rowsum_fp64(rpc, vd, n)) <= tol
    # broadcast
    gg = torch.rand(n, H, 1, generator=g).to(tdt).cuda()
    o = getattr(ATT_SDDMM_v3, "sddmm_%s_ones_h_nnz" % dt)(rp, col, mp, win, gg, mx, nnz)[0]
    assert np.array_equal(o.double().cpu().numpy(), oracle.ones_fp64(rpc, gg.double().cpu().numpy()))


def test_gat_v1_chain_matches_fp64_layer(cuda):
    """The reference's GAT v1 forward (end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198,
    dropout off): att -> LeakyReLU -> exp -> rowsum -> SpMM -> divide equals a
    row-softmax GAT layer."""
    from att_gb300.compat import ATT_Block_v3, ATT_SDDMM_v1, ATT_SpMM_v1
    rp_np, col_np, n = _graph(3000, 10, 4)
    rp, col, mp, mpt, win, at = [t.cuda() for t in ATT_Block_v3.blockProcess_sddmm_balance_gnn_trans(
        torch.from_numpy(rp_np), torch.from_numpy(col_np), 8, 8, 32)]
    nnz = col_np.shape[0]
    F = 64
    g = torch.Generator().manual_seed(3)
    Xp = ((torch.rand(n, F, generator=g) * 2 - 1) * 0.5).half().cuda()
    a0 = ((torch.rand(1, F, generator=g) - 0.5) * 0.5).half().cuda()
    a1 = ((torch.rand(1, F, generator=g) - 0.5) * 0.5).half().cuda()
    att = ATT_SDDMM_v1.att_fp16_h_nnz(rp, col, mp, win, Xp, a0, a1, 1.0, nnz)[0]
    att = torch.nn.functional.leaky_relu(att, 0.2)
    att = torch.exp(att)
    rows_sum = ATT_SpMM_v1.spmm_fp16_h_m_rowsum(rp, mp, att, win, at, n)[0].half()
    h = ATT_SpMM_v1.spmm_fp16_h_m(rp, col, mp, att, win, at, Xp)[0].half()
    h = h.div(rows_sum)
    ref = oracle.gat_layer_fp64(rp_np[: n + 1], col_np, Xp.double().cpu().numpy()[None],
                                a0.double().cpu().numpy()[None], a1.double().cpu().numpy()[None], n)
    assert oracle.rel_err(h.float().cpu().numpy(), ref) <= 1e-2


@pytest.mark.parametrize("odt", [torch.float32, torch.float16, torch.bfloat16])
@pytest.mark.parametrize("H", [1, 3])
def test_edge_softmax_vs_fp64(cuda, odt, H):
    """att_edge_softmax (LeakyReLU then row softmax over CSR rows) against the
    FP64 oracle: probabilities within the output type's rounding (fp32 1e-6,
    fp16 1e-3, bf16 8e-3 relative), row max / sum in fp32 within 1e-6, rows
    without edges report max -inf and sum 0; covers a hub row (longer than a
    warp's sweep many times over) and empty rows."""
    from att_gb300 import _lib, graphs
    from att_gb300.ops import _DT, _p, _stream
    rp, col = graphs.random_csr(500, 500, 30, seed=4, empty_frac=0.3, hub_rows=1, hub_len=450)
    n, nnz = 500, int(rp[-1])
    g = torch.Generator().manual_seed(H)
    logits = (torch.randn(H, nnz, generator=g) * 6).cuda()
    out = torch.full((H, nnz), float("nan"), dtype=odt, device="cuda")
    rmax = torch.empty(H, n, device="cuda")
    rsum = torch.empty(H, n, device="cuda")
    _lib.call("att_edge_softmax", _p(torch.from_numpy(rp).cuda()), n, _p(logits), nnz, H, 0.2, 1,
              _p(out), _DT[odt], nnz, _p(rmax), _p(rsum), _stream())
    torch.cuda.synchronize()
    tol = {torch.float32: 1e-6, torch.float16: 1e-3, torch.bfloat16: 8e-3}[odt]
    lens = np.diff(rp)
    for h in range(H):
        x = logits[h].double().cpu().numpy()
        x = np.where(x > 0, x, 0.2 * x)
        ref = oracle.edge_softmax_fp64(rp, x[None])[0]
        got = out[h].double().cpu().numpy()
        assert np.all(np.abs(got - ref) <= tol * np.abs(ref) + 1e-7)
        rows = np.repeat(np.arange(n), lens)
        m_ref = np.full(n, -np.inf)
        np.maximum.at(m_ref, rows, x)
        s_ref = np.zeros(n)
        np.add.at(s_ref, rows, np.exp(x - m_ref[rows]))
        has = lens > 0
        rm, rs = rmax[h].cpu().numpy(), rsum[h].cpu().numpy()
        assert np.allclose(rm[has], m_ref[has], rtol=1e-6, atol=0)
        assert np.allclose(rs[has], s_ref[has], rtol=1e-5, atol=0)
        assert np.all(np.isneginf(rm[~has])) and np.all(rs[~has] == 0)


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16, torch.float32])
@pytest.mark.parametrize("H,F", [(1, 8), (4, 64), (2, 128), (1, 256), (3, 40)])
def test_node_scores_pair_matches_two_single_passes(cuda, dtype, H, F):
    """att_node_scores_pair (one pass, 16-byte loads where the layout allows)
    against two att_node_scores passes and FP64, on the [H, N, F] view of an
    [N, H*F] projection (the fused GAT layer's layout)."""
    from att_gb300 import gat_ops
    g = torch.Generator().manual_seed(H * 1000 + F)
    n = 1237
    Xp = (torch.rand(n, H * F, generator=g) * 2 - 1).to(dtype).cuda()
    X3 = Xp.view(n, H, F).permute(1, 0, 2)
    a0 = (torch.rand(H, F, generator=g) - 0.5).cuda()
    a1 = (torch.rand(H, F, generator=g) - 0.5).cuda()
    s0, s1 = gat_ops.node_scores_pair(X3, a0, a1)
    r0 = gat_ops.node_scores(X3, a0)
    r1 = gat_ops.node_scores(X3, a1)
    ref0 = torch.einsum("hmf,hf->hm", X3.double(), a0.double())
    ref1 = torch.einsum("hmf,hf->hm", X3.double(), a1.double())
    for got, single, ref in ((s0, r0, ref0), (s1, r1, ref1)):
        assert got.shape == (H, n)
        assert oracle.rel_err(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-5
        assert oracle.rel_err(got.cpu().numpy(), single.cpu().numpy()) <= 1e-5
