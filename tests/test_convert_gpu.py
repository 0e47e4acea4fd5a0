"""GPU conversion vs the reference's outputs (golden) and the C oracle:
bit-exact on every output array."""
import os

import numpy as np
import pytest
import torch

from oracle import oracle
from tests._fixture import ROW, COL

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "blocks_golden.npz")


def _bits(a):
    a = np.asarray(a)
    if a.dtype == np.float16:
        return a.view(np.uint16)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    return a


def _gpu(rowptr, col, deg, W, w, P, emit_empty, **kw):
    from att_gb300 import ops
    d = None if deg is None else torch.from_numpy(np.ascontiguousarray(deg))
    return ops.block_convert(torch.from_numpy(rowptr), torch.from_numpy(col), d, window=W, wide=w,
                             part=P, emit_empty=emit_empty, **kw)


def test_matches_reference_golden(cuda):
    g = np.load(GOLDEN)
    for gi in range(int(g["n_graphs"])):
        rowptr, col = g["g%d_rowptr" % gi], g["g%d_col" % gi]
        for (W, w, P) in g["configs"]:
            for kind in ("fp16", "tf32"):
                deg = g["g%d_deg16" % gi] if kind == "fp16" else g["g%d_deg32" % gi]
                f = _gpu(rowptr, col, deg, int(W), int(w), int(P), kind == "tf32")
                key = "g%d_%s_%d_%d_%d" % (gi, kind, W, w, P)
                got = dict(rowptr=f.rowptr, col=f.col, val=f.val, window=f.window_of_part,
                           atomic=f.atomic)
                for name, t in got.items():
                    assert np.array_equal(_bits(t.cpu().numpy()), _bits(g[key + "_" + name])), \
                        (key, name)


def test_compat_module_returns_reference_tuple(cuda):
    from att_gb300.compat import Block_sr_bcrs
    res = Block_sr_bcrs.blockProcess_fp16_balance(torch.from_numpy(ROW), torch.from_numpy(COL),
                                                  torch.ones(32, dtype=torch.float16), 8, 8, 1)
    assert len(res) == 5 and all(t.device.type == "cpu" for t in res)
    assert res[0].tolist() == [0, 8, 8, 11, 16, 21, 24, 32, 32, 35, 40, 45, 48]
    assert res[3].tolist() == [0, 0, 1, 2, 2, 3]
    assert res[4].tolist() == [1, 1, 0, 1, 1, 0]


@pytest.mark.parametrize("case", range(10))
def test_random_graphs_vs_oracle_with_maps(cuda, case):
    from att_gb300 import graphs
    specs = [
        dict(n_rows=300, n_cols=300, max_len=12, seed=1),
        dict(n_rows=517, n_cols=517, max_len=6, seed=2, hub_rows=3, hub_len=450),
        dict(n_rows=240, n_cols=240, max_len=10, seed=3, empty_frac=0.6),
        dict(n_rows=129, n_cols=2000, max_len=40, seed=4, dup=True, sort_rows=False),
        dict(n_rows=64, n_cols=9000, max_len=3, seed=5, hub_rows=4, hub_len=5000),  # > smem cap
        dict(n_rows=1001, n_cols=1001, max_len=30, seed=6, hub_rows=1, hub_len=1000),
        # windows of tens of thousands of edges through the merge path
        dict(n_rows=48, n_cols=300000, max_len=20, seed=7, hub_rows=3, hub_len=45000),
        # unsorted rows with duplicates in windows of 1025..4096 edges and of
        # more than 4096 (the sorting and bitmap fallbacks of the merge path)
        dict(n_rows=80, n_cols=5000, max_len=300, seed=8, dup=True, sort_rows=False),
        dict(n_rows=40, n_cols=60000, max_len=5, seed=9, hub_rows=2, hub_len=40000, dup=True,
             sort_rows=False),
        # sorted rows with repeated columns, in windows of a few hundred edges
        dict(n_rows=64, n_cols=3000, max_len=200, seed=10, dup=True),
    ]
    sp = specs[case]
    rowptr, col = graphs.random_csr(**sp)
    n_cols = sp["n_cols"]
    rng = np.random.default_rng(case)
    d32 = (1.0 / np.sqrt(rng.integers(1, 50, size=max(n_cols, rowptr.shape[0])))).astype(np.float32)
    d16 = d32.astype(np.float16)
    sorted_rows = sp.get("sort_rows", True)
    for (W, w, P) in ((8, 8, 32), (8, 4, 32), (16, 8, 4), (8, 16, 2), (16, 16, 1)):
        for deg, emit in ((d16, False), (d32, True)):
            o = oracle.block_convert(rowptr, col, deg, W, w, P, emit_empty=emit, want_map=True,
                                     want_trans=sorted_rows)
            f = _gpu(rowptr, col, deg, W, w, P, emit, want_map=True, want_trans=sorted_rows,
                     want_edge_slot=True, n_cols=deg.shape[0])
            for name, t in (("rowptr", f.rowptr), ("col", f.col), ("val", f.val),
                            ("window", f.window_of_part), ("atomic", f.atomic), ("map", f.map)):
                assert np.array_equal(_bits(t.cpu().numpy()), _bits(o[name])), (case, W, w, P, name)
            if sorted_rows:
                assert np.array_equal(f.map_t.cpu().numpy(), o["map_t"]), (case, W, w, P)
            # edge_slot inverts the map for the last duplicate of each slot
            es = f.edge_slot.cpu().numpy()
            mp = f.map.cpu().numpy()
            used = es >= 0
            assert np.all(mp[es[used]] >= np.nonzero(used)[0])


def _windows_of_sizes(sizes, n_cols, seed, sort_rows=True):
    """CSR whose 8-row windows hold exactly `sizes[i]` edges each, split at
    random over their rows, columns drawn from a range narrow enough that
    rows of a window share columns."""
    rng = np.random.default_rng(seed)
    lens, cols = [], []
    for E in sizes:
        cuts = np.sort(rng.integers(0, E + 1, size=7))
        per = np.diff(np.concatenate([[0], cuts, [E]]))
        span = max(8, min(n_cols, 2 * E))
        lo = int(rng.integers(0, n_cols - span + 1))
        for L in per:
            c = rng.integers(lo, lo + span, size=int(L)).astype(np.int32)
            cols.append(np.sort(c) if sort_rows else c)
            lens.append(int(L))
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    return rowptr, np.concatenate(cols).astype(np.int32)


@pytest.mark.parametrize("sort_rows", [True, False])
def test_window_sizes_at_every_kernel_boundary(cuda, sort_rows):
    """Windows of exactly 1, 31-33, 63-65, 127-129, 255-257, 1023-1025 and
    4095-4097 edges: the edges either side of every size class of the plan
    (register sorts up to 32, 64, 128 and 256 keys, then the row merge and
    its sorting / bitmap fallbacks for unsorted rows), with rows sharing
    columns (duplicates within a window).  Bit-exact with the C oracle."""
    sizes = [1, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257, 1023, 1024, 1025, 4095,
             4096, 4097, 0, 7]
    rowptr, col = _windows_of_sizes(sizes, 20000, seed=31 + sort_rows, sort_rows=sort_rows)
    d = (1.0 / np.sqrt(np.arange(1, 20001))).astype(np.float32)
    for (W, w, P, deg, emit) in ((8, 8, 32, d.astype(np.float16), False), (8, 4, 32, d, True)):
        o = oracle.block_convert(rowptr, col, deg, W, w, P, emit_empty=emit, want_map=True)
        f = _gpu(rowptr, col, deg, W, w, P, emit, want_map=True, n_cols=deg.shape[0])
        for name, t in (("rowptr", f.rowptr), ("col", f.col), ("val", f.val),
                        ("window", f.window_of_part), ("atomic", f.atomic), ("map", f.map)):
            assert np.array_equal(_bits(t.cpu().numpy()), _bits(o[name])), (sort_rows, W, w, name)


def test_unsorted_rows_rejected_for_mirror_map(cuda):
    from att_gb300 import graphs, _lib
    rowptr, col = graphs.random_csr(64, 64, 8, seed=9, sort_rows=False)
    with pytest.raises(_lib.AttError):
        _gpu(rowptr, col, None, 8, 8, 32, False, want_map=True, want_trans=True)


def test_bad_column_rejected(cuda):
    from att_gb300 import _lib
    col = COL.copy()
    col[5] = 40
    with pytest.raises(_lib.AttError):
        _gpu(ROW, col, np.ones(32, np.float16), 8, 8, 32, False)


def test_empty_graph(cuda):
    rowptr = np.zeros(17, np.int32)
    col = np.zeros(0, np.int32)
    f = _gpu(rowptr, col, np.ones(16, np.float16), 8, 8, 32, False)
    assert f.n_parts == 0 and f.rowptr.tolist() == [0]
    f = _gpu(rowptr, col, np.ones(16, np.float32), 8, 4, 32, True)
    assert f.n_parts == 2 and f.rowptr.tolist() == [0, 0, 0, 0, 0]


def test_async_convert_matches_sync(cuda):
    """block_convert_async + block_convert_finish (no host synchronisation in
    the plan) give the same format as block_convert, bit for bit."""
    import torch
    from att_gb300 import graphs, ops
    for seed, (n, L, hubs) in enumerate([(64, 8, 0), (3001, 30, 4), (20000, 12, 10)]):
        rp, col = graphs.random_csr(n, n, L, seed, hub_rows=hubs, hub_len=min(n, 2000))
        deg = torch.rand(n, dtype=torch.float32).half()
        a = ops.block_convert(torch.from_numpy(rp), torch.from_numpy(col), deg, window=8, wide=8,
                              part=32, want_map=True)
        p = ops.block_convert_async(torch.from_numpy(rp), torch.from_numpy(col), deg, window=8,
                                    wide=8, part=32, want_map=True)
        p.event.synchronize()
        b = ops.block_convert_finish(p)
        for name in ("rowptr", "col", "window_of_part", "atomic", "val", "map"):
            assert torch.equal(getattr(a, name), getattr(b, name)), (seed, name)


def test_async_fill_matches_sync(cuda):
    """block_convert_finish(check_later=True) (att_block_fill_async: no host
    synchronisation, checks copied to pinned memory) gives the synchronous
    format bit for bit, every output included, and its deferred check passes."""
    import torch
    from att_gb300 import graphs, ops
    for seed, (n, L, hubs) in enumerate([(64, 8, 0), (3001, 30, 4), (20000, 12, 10)]):
        rp, col = graphs.random_csr(n, n, L, seed + 7, hub_rows=hubs, hub_len=min(n, 2000))
        deg = torch.rand(n, dtype=torch.float32).half()
        kw = dict(window=8, wide=8, part=32, want_map=True, want_trans=True, want_edge_slot=True)
        a = ops.block_convert(torch.from_numpy(rp), torch.from_numpy(col), deg, **kw)
        p = ops.block_convert_async(torch.from_numpy(rp), torch.from_numpy(col), deg, **kw)
        p.event.synchronize()
        b = ops.block_convert_finish(p, check_later=True)
        torch.cuda.synchronize()
        ops.block_fill_check(b)
        assert "fill_flags" not in b.extra
        for name in ("rowptr", "col", "window_of_part", "atomic", "val", "map", "map_t",
                     "edge_slot"):
            assert torch.equal(getattr(a, name), getattr(b, name)), (seed, name)


def test_async_fill_reports_unsorted_rows_for_mirror_map(cuda):
    """The deferred check of an asynchronous fill raises what the synchronous
    fill raises: a mirrored-edge map over unsorted rows."""
    import torch
    from att_gb300 import graphs, ops, _lib
    rowptr, col = graphs.random_csr(64, 64, 8, seed=9, sort_rows=False)
    p = ops.block_convert_async(torch.from_numpy(rowptr), torch.from_numpy(col), None, window=8,
                                wide=8, part=32, want_map=True, want_trans=True)
    p.event.synchronize()
    f = ops.block_convert_finish(p, check_later=True)
    torch.cuda.synchronize()
    with pytest.raises(_lib.AttError):
        ops.block_fill_check(f)


def test_async_convert_rejects_bad_column(cuda):
    import torch
    from att_gb300 import ops, _lib
    col = COL.copy()
    col[5] = 40
    p = ops.block_convert_async(torch.from_numpy(ROW), torch.from_numpy(col),
                                torch.ones(32, dtype=torch.float16), window=8, wide=8, part=32)
    p.event.synchronize()
    with pytest.raises(_lib.AttError):
        ops.block_convert_finish(p)
