"""The CPU oracle pinned against the reference's own outputs (golden file made
by tests/golden/make_golden.py from the reference's compiled conversion) and
against the known answers of the reference's tests."""
import os

import numpy as np
import pytest

from oracle import oracle
from tests._fixture import ROW, COL

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "blocks_golden.npz")


def _golden():
    return np.load(GOLDEN)


def test_f16_rounding_matches_numpy():
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.standard_normal(20000).astype(np.float32) * 10.0 ** rng.integers(-9, 5, 20000),
                         np.array([65504, 65520, 65536, 1e-8, 2 ** -24, 2 ** -25, 3 * 2 ** -26, 0.0, -0.0],
                                  np.float32)])
    want = xs.astype(np.float16).view(np.uint16)
    got = np.array([oracle.f32_to_f16_bits(float(x)) for x in xs], np.uint16)
    assert np.array_equal(got, want)


def test_oracle_matches_reference_golden():
    g = _golden()
    n = int(g["n_graphs"])
    for gi in range(n):
        rowptr, col = g["g%d_rowptr" % gi], g["g%d_col" % gi]
        for (W, w, P) in g["configs"]:
            for kind in ("fp16", "tf32"):
                deg = g["g%d_deg16" % gi] if kind == "fp16" else g["g%d_deg32" % gi]
                o = oracle.block_convert(rowptr, col, deg, int(W), int(w), int(P),
                                         emit_empty=(kind == "tf32"))
                key = "g%d_%s_%d_%d_%d" % (gi, kind, W, w, P)
                for name in ("rowptr", "col", "window", "atomic"):
                    assert np.array_equal(o[name], g[key + "_" + name]), (key, name)
                ref_val = g[key + "_val"]
                bits = np.uint16 if kind == "fp16" else np.uint32
                assert np.array_equal(o["val"].view(bits), ref_val.view(bits)), (key, "val")


def test_known_split_of_fixture():
    # (window, wide, partSize) = (8, 8, 1): every block its own part
    o = oracle.block_convert(ROW, COL, np.ones(32, np.float16), 8, 8, 1)
    assert o["rowptr"].tolist() == [0, 8, 8, 11, 16, 21, 24, 32, 32, 35, 40, 45, 48]
    assert o["window"].tolist() == [0, 0, 1, 2, 2, 3]
    assert o["atomic"].tolist() == [1, 1, 0, 1, 1, 0]


def test_map_semantics_on_fixture():
    o = oracle.block_convert(ROW, COL, None, 8, 8, 32, want_map=True, want_trans=True)
    mp, W, w = o["map"], 8, 8
    rows = oracle.csr_rows(ROW)
    seen = np.zeros(COL.shape[0], bool)
    for slot, e in enumerate(mp):
        if e < 0:
            continue
        blk, rem = slot // (W * w), slot % (W * w)
        r, k = rem // w, rem % w
        cond = blk * w + k
        # slot's window row and condensed column hold edge e
        assert o["col"][cond] == COL[e]
        assert rows[e] % W == r
        seen[e] = True
    assert seen.all()


def test_semantic_pins_on_fixture():
    rng = np.random.default_rng(1)
    h, n, F = 4, 30, 125
    rp = ROW[: n + 1]
    col = COL[: rp[-1]]
    X = rng.integers(1, 3, size=(h, n, F)).astype(np.float64)
    out = oracle.sddmm_fp64(rp, col, X, X)
    assert out[0][0] == X[0][0] @ X[0][1]          # test_sddmm_fp16.py:62
    assert out[1][1] == X[1][0] @ X[1][2]          # test_sddmm_fp16.py:67
    a = np.ones((h, 1, F))
    att = oracle.att_fp64(rp, col, X, a, a)
    assert att[1][1] == X[1][0] @ a[1][0] + X[1][2] @ a[1][0]   # test_sddmm_tf32_att.py
    g = rng.integers(1, 5, size=(n, h, 1)).astype(np.float64)
    ones = oracle.ones_fp64(rp, g)
    assert ones[0][0] == g[0][0][0] and ones[1][6] == g[1][1][0]  # test_sddmm_fp16_ones.py:62-68
    vals = np.ones((3, col.shape[0]))
    rs = oracle.rowsum_fp64(rp, vals, n)
    assert np.array_equal(rs[0], np.diff(rp).astype(np.float64))  # test_spmm_h_m_ones.py


def test_spmm_oracles_agree():
    from att_gb300 import graphs
    rp, col = graphs.random_csr(203, 203, 9, seed=3, hub_rows=2, hub_len=150)
    deg = (1.0 / np.sqrt(np.maximum(np.diff(rp), 1))).astype(np.float16)
    X = np.random.default_rng(2).uniform(-1, 1, size=(203, 16))
    for (W, w, P) in ((8, 8, 32), (16, 8, 2), (8, 4, 3)):
        o = oracle.block_convert(rp, col, deg, W, w, P)
        a = oracle.spmm_blocks_fp64(o, X, 203, W, w)
        b = oracle.spmm_csr_fp64(rp[: (203 // W) * W + 1], col[: rp[(203 // W) * W]],
                                 oracle.gcn_values(rp, col, deg)[: rp[(203 // W) * W]], X, 203)
        b = np.vstack([b, np.zeros((203 - b.shape[0], 16))])
        assert np.allclose(a, b, rtol=0, atol=1e-12)


def test_graph_generator_hits_edge_count():
    from att_gb300 import graphs
    rp, col = graphs.chung_lu(4096, 10, 2.1, seed=0)
    assert int(rp[-1]) == 4096 * 10 + 4096
    r = np.asarray(rp)
    c = np.asarray(col)
    for i in range(0, 4096, 97):
        row = c[r[i]:r[i + 1]]
        assert np.all(np.diff(row) > 0)


def test_gat_oracles_match_dense_restatement():
    """The FP64 GAT-layer oracles (dot and additive logits) against a dense
    restatement on a small graph: masked logits, LeakyReLU, row softmax over
    the edges, aggregation -- rows without edges give zeros."""
    from att_gb300 import graphs
    n, H, F = 60, 2, 8
    rp, col = graphs.random_csr(n, n, 7, seed=5, empty_frac=0.2)
    rng = np.random.default_rng(9)
    X = rng.uniform(-1, 1, size=(H, n, F))
    a0 = rng.uniform(-0.5, 0.5, size=(H, 1, F))
    a1 = rng.uniform(-0.5, 0.5, size=(H, 1, F))
    mask = np.zeros((n, n), dtype=bool)
    for i in range(n):
        mask[i, col[rp[i]:rp[i + 1]]] = True

    def dense(e):
        e = np.where(e > 0, e, 0.2 * e)
        e = np.where(mask[None], e, -np.inf)
        m = e.max(axis=2, keepdims=True)
        m = np.where(np.isfinite(m), m, 0.0)
        p = np.where(mask[None], np.exp(e - m), 0.0)
        s = p.sum(axis=2, keepdims=True)
        p = np.divide(p, s, out=np.zeros_like(p), where=s > 0)
        return p @ X

    dot = dense(np.einsum("hif,hjf->hij", X, X))
    add = dense((X @ a0.transpose(0, 2, 1)) + (X @ a1.transpose(0, 2, 1)).transpose(0, 2, 1))
    assert np.allclose(oracle.gat_dot_layer_fp64(rp, col, X, n), dot, rtol=0, atol=1e-12)
    assert np.allclose(oracle.gat_layer_fp64(rp, col, X, a0, a1, n), add, rtol=0, atol=1e-12)


def _small_graph(seed=3, n=300):
    from att_gb300 import graphs
    import torch
    rp, col = graphs.chung_lu(n, 9, 2.1, seed=seed)
    return rp.numpy(), col.numpy()


def test_row_sampled_restatements_match_whole_graph():
    """sub_csr / sample_rows and the row-sampled FP64 functions agree with the
    whole-graph restatements on the sampled rows."""
    import torch
    rp, col = _small_graph()
    n = rp.shape[0] - 1
    rows = oracle.sample_rows(rp, n, 40, 3, seed=1)
    lens = np.diff(rp)
    top = np.argsort(lens)[::-1][:3]
    for r in top:  # every row of each hub window is in the sample
        w0 = r // 8 * 8
        assert set(range(w0, min(w0 + 8, n))) <= set(rows.tolist())
    srp, scol, eid = oracle.sub_csr(rp, col, rows)
    assert np.array_equal(np.diff(srp), lens[rows])
    assert np.array_equal(scol, col[eid])
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (n, 16))
    vals = rng.uniform(0, 1, col.shape[0])
    full = oracle.spmm_csr_fp64(rp, col, vals, X)
    assert np.allclose(oracle.spmm_rows_fp64(rp, col, vals, X, rows), full[rows], atol=1e-12)
    gat_full = oracle.gat_dot_layer_fp64(rp, col, X[None], n)[0]
    assert np.allclose(oracle.gat_dot_rows_fp64(rp, col, X, rows), gat_full[rows], atol=1e-12)
    H, F = 2, 8
    Xp = torch.from_numpy(rng.uniform(-1, 1, (n, H * F)))
    a0 = torch.from_numpy(rng.uniform(-0.5, 0.5, (H, F)))
    a1 = torch.from_numpy(rng.uniform(-0.5, 0.5, (H, F)))
    whole = oracle.gat_add_layer_torch(rp, col, Xp, a0, a1)
    part = oracle.gat_add_rows_torch(rp, col, Xp, a0, a1, rows)
    assert torch.allclose(part, whole[torch.from_numpy(rows)], atol=1e-12)


def test_gcn2_restatement_is_two_layers_of_spmm():
    rp, col = _small_graph(seed=5, n=200)
    n = rp.shape[0] - 1
    rng = np.random.default_rng(1)
    X = rng.uniform(-1, 1, (n, 8))
    W1 = rng.uniform(-1, 1, (8, 6))
    W2 = rng.uniform(-1, 1, (6, 4))
    vals = rng.uniform(0, 1, col.shape[0])
    h = np.maximum(oracle.spmm_csr_fp64(rp, col, vals, X @ W1), 0)
    want = oracle.spmm_csr_fp64(rp, col, vals, h @ W2)
    assert np.allclose(oracle.gcn2_fp64(rp, col, vals, X, W1, W2, n), want, atol=1e-12)


def test_gatv2_restatement_gradients_by_finite_differences():
    """The GATv2 restatement's autograd gradients agree with FP64 central
    differences (torch.autograd.gradcheck) on a small graph."""
    import torch
    rp, col = _small_graph(seed=1, n=40)
    g = torch.Generator().manual_seed(0)
    X = torch.rand(40, 6, generator=g, dtype=torch.float64)
    W0 = torch.rand(6, 8, generator=g, dtype=torch.float64).requires_grad_(True)
    W1 = torch.rand(6, 8, generator=g, dtype=torch.float64).requires_grad_(True)
    a = torch.rand(2, 1, 4, generator=g, dtype=torch.float64).requires_grad_(True)
    assert torch.autograd.gradcheck(
        lambda w0, w1, aa: oracle.gatv2_layer_torch(rp, col, X, w0, w1, aa), (W0, W1, a))
