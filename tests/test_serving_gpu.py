"""Serving loop on the GPU: work groups, the batched multi-graph SpMM and the
continuous-batching loop.

Tolerances: the batched SpMM against FP64 1e-2 normwise (fp16 features and
values, fp32 accumulation); against the single-graph kernel 1e-5 (fp32
summation order of split windows only); alone vs in a mix and CUDA-graph
replay vs direct launch 0 (bit-identical: no atomics); a served request alone
vs in the mix 0 for the aggregation and 1e-6 relative end to end."""
import numpy as np
import pytest
import torch

from oracle import oracle

pytestmark = pytest.mark.gpu


def groups_np(win, G=4, n_windows=0):
    """Restatement of att_spmm_groups: runs of <= G parts of one window, and
    the windows below n_windows that own no part."""
    win = np.asarray(win)
    P = len(win)
    gp, gs, rf = [], [], []
    slot, p = 0, 0
    while p < P:
        q = p
        while q < P and win[q] == win[p]:
            q += 1
        multi = q - p > G
        if multi:
            rf.append(len(gp))
        for s in range(p, q, G):
            gp.append(s)
            gs.append(slot if multi else -1)
            slot += multi
        p = q
    gp.append(P)
    rf.append(len(gp) - 1)
    empty = np.setdiff1d(np.arange(n_windows), win)
    return np.array(gp), np.array(gs), np.array(rf), slot, empty


def _graph(kind, seed):
    from att_gb300 import graphs
    if kind == "hubs":   # hub rows -> windows of up to 16 parts (several groups)
        rp, col = graphs.random_csr(4000, 4000, 40, seed, hub_rows=6, hub_len=3500)
        return torch.from_numpy(rp), torch.from_numpy(col)
    if kind == "empty":  # empty windows and rows past the last edge
        rp, col = graphs.random_csr(1203, 1203, 12, seed, empty_frac=0.6)
        return torch.from_numpy(rp), torch.from_numpy(col)
    n, deg = {"small": (1000, 5.0), "mid": (20000, 30.0), "dense": (6000, 50.0)}[kind]
    return graphs.chung_lu(n, deg, 2.1, seed=seed, device="cpu")


def _prepared(kind, seed, F=128):
    from att_gb300 import graphs, ops, serving
    rp, col = _graph(kind, seed)
    n = rp.shape[0] - 1
    rp8 = graphs.pad_rows(rp.cuda(), 8)
    deg = graphs.gcn_degree(rp8, torch.float16)
    deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg))  # rows without edges
    fmt = ops.block_convert(rp8, col.cuda(), deg, window=8, wide=8, part=32)
    g = serving.spmm_groups(fmt, m_out=n)
    part = torch.empty(max(g.n_slots, 1) * 8 * F, dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    X = (torch.rand(n, F, generator=gen, device="cuda") * 2 - 1).half()
    return dict(rp=rp, col=col, n=n, fmt=fmt, groups=g, partial=part, X=X, deg=deg)


def _job(d, Y=None):
    from att_gb300 import serving
    if Y is None:
        Y = torch.full((d["n"], d["X"].shape[1]), float("nan"), device="cuda")
    return serving.Job(d["fmt"], d["groups"], d["partial"], d["X"], Y, d["n"])


KINDS = [("hubs", 1), ("empty", 2), ("small", 3), ("mid", 4), ("dense", 5)]


def test_groups_match_restatement(cuda):
    for kind, seed in KINDS:
        d = _prepared(kind, seed)
        g = d["groups"]
        gp, gs, rf, ns, em = groups_np(d["fmt"].window_of_part.cpu().numpy(), 4, (d["n"] + 7) // 8)
        assert (g.n_groups, g.n_red, g.n_slots, g.n_empty) == (len(gp) - 1, len(rf) - 1, ns,
                                                                len(em)), kind
        assert np.array_equal(g.empty_win.cpu().numpy()[: len(em)], em), kind
        assert np.array_equal(g.group_part.cpu().numpy()[: len(gp)], gp), kind
        assert np.array_equal(g.group_slot.cpu().numpy()[: len(gs)], gs), kind
        assert np.array_equal(g.red_first.cpu().numpy()[: len(rf)], rf), kind
    # the hub case really has multi-group windows, the sparse one empty windows
    assert _prepared("hubs", 1)["groups"].n_red > 0
    assert _prepared("empty", 2)["groups"].n_empty > 0


def test_group_sizes(cuda):
    """Groups of 1, 2, 4 and 8 parts: structure as the restatement, results
    equal to FP64 within 1e-2 and to each other within 1e-5."""
    from att_gb300 import serving
    d = _prepared("hubs", 1)
    ys = []
    for G in (1, 2, 4, 8):
        g = serving.spmm_groups(d["fmt"], G, m_out=d["n"])
        gp, gs, rf, ns, _ = groups_np(d["fmt"].window_of_part.cpu().numpy(), G)
        assert (g.n_groups, g.n_red, g.n_slots) == (len(gp) - 1, len(rf) - 1, ns), G
        assert np.array_equal(g.group_part.cpu().numpy()[: len(gp)], gp), G
        assert np.array_equal(g.group_slot.cpu().numpy()[: len(gs)], gs), G
        part = torch.empty(max(g.n_slots, 1) * 8 * 128, dtype=torch.float32, device="cuda")
        j = serving.Job(d["fmt"], g, part, d["X"], torch.empty(d["n"], 128, device="cuda"), d["n"])
        serving.spmm_batched([j]).check()
        ys.append(j.Y.cpu().numpy())
    for y in ys[1:]:
        assert oracle.rel_err(y, ys[0]) <= 1e-5


def test_groups_empty_format(cuda):
    from att_gb300 import ops, serving
    fmt = ops.block_convert(torch.zeros(17, dtype=torch.int32), torch.zeros(0, dtype=torch.int32),
                            torch.ones(16, dtype=torch.float16), window=8, wide=8, part=32)
    g = serving.spmm_groups(fmt)
    assert (g.n_groups, g.n_red, g.n_slots, g.n_empty) == (0, 0, 0, 2)
    j = serving.Job(fmt, g, None, torch.ones(16, 64, dtype=torch.float16, device="cuda"),
                    torch.full((16, 64), float("nan"), device="cuda"), 16)
    serving.spmm_batched([j]).check()
    assert torch.equal(j.Y, torch.zeros_like(j.Y))
    assert int(g.group_part[0]) == 0 and int(g.red_first[0]) == 0


def test_batched_single_job_vs_single_graph_and_fp64(cuda):
    from att_gb300 import ops, serving
    for kind, seed in KINDS:
        d = _prepared(kind, seed)
        job = _job(d)
        b = serving.spmm_batched([job])
        torch.cuda.synchronize()
        b.check()
        Y = job.Y
        assert torch.isfinite(Y).all(), kind   # every row written, including empty windows
        Ys = ops.spmm_format(d["fmt"], d["X"], d["n"])
        assert oracle.rel_err(Y.cpu().numpy(), Ys.cpu().numpy()) <= 1e-5, kind
        rp, col = d["rp"].numpy(), d["col"].numpy()
        n8 = rp.shape[0] - 1
        deg = d["deg"].cpu().numpy()[: n8]
        vals = oracle.gcn_values(rp, col, deg)
        ref = oracle.spmm_csr_fp64(rp, col, vals, d["X"].cpu().numpy().astype(np.float64), None)
        assert oracle.rel_err(Y.cpu().numpy(), ref[: d["n"]]) <= 1e-2, kind


def test_alone_equals_mixed_bit_exact(cuda):
    """Each job's Y is bit-identical alone and inside a mixed batch (any order,
    any neighbours), through a direct launch and a CUDA-graph replay."""
    from att_gb300 import serving
    preps = [_prepared(k, s) for k, s in KINDS]
    alone = []
    for d in preps:
        j = _job(d)
        serving.spmm_batched([j]).check()
        alone.append(j.Y.clone())
    rng = np.random.default_rng(0)
    b = serving.BatchedSpmm(16, use_graph=True)
    for trial in range(3):
        order = rng.permutation(len(preps))
        reps = [int(i) for i in order] + [int(i) for i in order[:2]]  # duplicates in the mix
        jobs = [_job(preps[i]) for i in reps]
        # several jobs may share one partial buffer only if they are the same
        # graph run back to back; give the duplicates their own
        for j, i in zip(jobs[len(order):], reps[len(order):]):
            j.partial = torch.empty_like(preps[i]["partial"])
        b.run(jobs)
        torch.cuda.synchronize()
        b.check()
        for j, i in zip(jobs, reps):
            assert torch.equal(j.Y, alone[i]), (trial, KINDS[i])


def test_graph_replay_equals_direct_launch(cuda):
    from att_gb300 import serving
    preps = [_prepared(k, s, F=64) for k, s in KINDS[:3]]
    direct = serving.BatchedSpmm(4, use_graph=False)
    graphed = serving.BatchedSpmm(4, use_graph=True)
    for subset in ([0, 1, 2], [2], [1, 0]):
        j1 = [_job(preps[i]) for i in subset]
        direct.run(j1)
        j2 = [_job(preps[i]) for i in subset]
        graphed.run(j2)
        torch.cuda.synchronize()
        for a, c in zip(j1, j2):
            assert torch.equal(a.Y, c.Y)
    assert graphed.launches == 3


def test_batched_flags_bad_column(cuda):
    """A column id past n_x is flagged (error bit 1) and the gather skipped."""
    from att_gb300 import serving, _lib
    d = _prepared("small", 7, F=64)
    X = d["X"][: d["n"] // 2]       # too few feature rows for the graph
    j = serving.Job(d["fmt"], d["groups"], d["partial"], X, torch.empty(d["n"], 64, device="cuda"), d["n"])
    b = serving.spmm_batched([j])
    torch.cuda.synchronize()
    with pytest.raises(_lib.AttError):
        b.check()


def _pool(specs, F=128):
    out = []
    for kind, seed in specs:
        rp, col = _graph(kind, seed)
        n = rp.shape[0] - 1
        gen = torch.Generator()
        gen.manual_seed(seed)
        X = (torch.rand(n, F, generator=gen) * 2 - 1).half()
        out.append((rp.pin_memory(), col.pin_memory(), X.pin_memory(), n, int(col.numel())))
    return out


def _clone(reqs):
    from att_gb300 import serving
    return [serving.Request(r.rid, r.arrival, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs]


def test_serving_alone_vs_mix_and_vs_one_by_one(cuda):
    from att_gb300 import serving
    model = serving.GCN2(seed=4)
    pool = _pool(KINDS)
    reqs = serving.make_requests(pool, rate=400.0, count=16, seed=11)
    # alone: each request served by itself
    alone = {}
    srv = serving.Server(model, max_active=16, workers=4)
    for r in _clone(reqs):
        srv.run([r], realtime=False)
        assert r.error is None
        alone[r.rid] = r.out.clone()
    # in the mix: all at once, with Poisson arrivals in real time, and with
    # results written straight into pinned host memory by the batched kernel
    # instead of copied back from device memory
    direct_srv = serving.Server(model, max_active=16, workers=4, direct_output=True, checksum=True)
    for realtime, server in ((False, srv), (True, srv), (True, direct_srv)):
        mixed = _clone(reqs)
        server.run(mixed, realtime=realtime)
        for r in mixed:
            assert r.error is None and r.out is not None
            ref = alone[r.rid]
            diff = (r.out - ref).abs().max().item()
            assert diff <= 1e-6 * max(ref.abs().max().item(), 1e-30), (realtime, r.rid, diff)
            if server is direct_srv:   # checksum of the result in host memory
                assert abs(r.checksum - ref.double().sum().item()) <= 1e-6 * ref.abs().sum().item()
    assert max(srv.jobs_per_tick) > 1    # ticks really held several graphs
    # the one-graph-per-call path (att_spmm, split windows by atomics) agrees
    seq = serving.serve_one_by_one(_clone(reqs), model, realtime=False)
    for r in seq:
        assert oracle.rel_err(r.out.numpy(), alone[r.rid].numpy()) <= 1e-4
    st = serving.latency_stats(mixed)
    assert st["requests"] == len(reqs) and st["p99_ms"] >= st["p50_ms"] > 0


def test_serving_matches_fp64_two_layer_gcn(cuda):
    from att_gb300 import serving
    model = serving.GCN2(seed=4)
    pool = _pool([("mid", 21)])
    r = serving.make_requests(pool, rate=100.0, count=1, seed=3)
    serving.serve(r, model, realtime=False, workers=1)
    r = r[0]
    rp, col = r.rowptr.numpy(), r.col.numpy()
    n8 = rp.shape[0] - 1
    rp8 = np.concatenate([rp, np.full(8 - n8 % 8, rp[-1], np.int32)])
    with np.errstate(divide="ignore"):
        deg = (1.0 / np.sqrt(np.diff(rp8).astype(np.float32))).astype(np.float16)
    deg[~np.isfinite(deg)] = 0
    vals = oracle.gcn_values(rp, col, deg[:n8]).astype(np.float64)
    W1 = model.W1.double().cpu().numpy()
    W2 = model.W2.double().cpu().numpy()
    X = r.X.double().numpy()
    H = np.maximum(oracle.spmm_csr_fp64(rp, col, vals, X @ W1, None), 0)
    ref = oracle.spmm_csr_fp64(rp, col, vals, H @ W2, None)
    assert oracle.rel_err(r.out.numpy(), ref) <= 1e-2


def test_serving_rejects_bad_requests_and_keeps_serving(cuda):
    """Host-side fault injection: a request over the whole budget and one with
    a malformed CSR (column past the node count) fail alone; the rest complete
    and the budget returns to zero."""
    from att_gb300 import serving
    model = serving.GCN2(seed=4)
    pool = _pool([("small", 31), ("mid", 32)])
    reqs = serving.make_requests(pool, rate=1000.0, count=6, seed=5)
    bad_col = reqs[2].col.clone()
    bad_col[len(bad_col) // 2] = reqs[2].n + 1000
    reqs[2] = serving.Request(reqs[2].rid, reqs[2].arrival, reqs[2].rowptr, bad_col.pin_memory(),
                              reqs[2].X, reqs[2].n, reqs[2].nnz)
    huge = serving.Request(99, 0.0, reqs[0].rowptr, reqs[0].col, reqs[0].X, 10**9, 10**10)
    srv = serving.Server(model, budget=50e9, max_active=4, workers=2)
    srv.run(reqs + [huge], realtime=False)
    assert huge.error is not None and "budget" in huge.error
    assert reqs[2].error is not None
    for i, r in enumerate(reqs):
        if i != 2:
            assert r.error is None and r.out is not None
    assert srv.adm.used == 0 and srv.adm.active == 0


def test_host_output_equals_device_output(cuda):
    """A Y in pinned host memory (written over the CPU-GPU link) equals the
    device Y bit for bit; pageable memory is refused."""
    from att_gb300 import serving, _lib
    d = _prepared("hubs", 1)
    dev = _job(d)
    serving.spmm_batched([dev]).check()
    host = torch.full((d["n"], 128), float("nan"), pin_memory=True)
    j = serving.Job(d["fmt"], d["groups"], d["partial"], d["X"], host, d["n"],
                    serving.host_device_pointer(host))
    serving.spmm_batched([j]).check()
    torch.cuda.synchronize()
    assert torch.equal(host, dev.Y.cpu())
    with pytest.raises(_lib.AttError):
        serving.host_device_pointer(torch.zeros(16))


def test_autotune_group_parts(cuda):
    """tune_group_parts times the batched launch for each group size on
    prepared requests and returns the fastest; the batched result with that
    size equals the default size's within fp32 summation order (1e-5)."""
    from att_gb300 import autotune, serving
    model = serving.GCN2(seed=4)
    s = torch.cuda.current_stream()
    reqs = []
    for i, (kind, seed) in enumerate(KINDS):
        rp, col = _graph(kind, seed)
        n = rp.shape[0] - 1
        gen = torch.Generator().manual_seed(seed)
        X = (torch.rand(n, 128, generator=gen) * 2 - 1).half()
        r = serving.Request(i, 0.0, rp.to(torch.int32), col.to(torch.int32), X, n, int(col.shape[0]))
        serving.prepare(r, model, s, with_groups=False)
        reqs.append(r)
    torch.cuda.synchronize()
    G, table = autotune.tune_group_parts(reqs, candidates=(1, 2, 4, 8),
                                         tuner=autotune.Tuner(warmup=1, reps=3))
    assert set(table) == {1, 2, 4, 8} and G == min(table, key=table.get)
    outs = {}
    for g_parts in (G, 4):
        jobs = []
        for r in reqs:
            g = serving.spmm_groups(r.dev["fmt"], g_parts, m_out=r.n)
            part = torch.empty(max(g.n_slots, 1) * 8 * 128, dtype=torch.float32, device="cuda")
            jobs.append(serving.Job(r.dev["fmt"], g, part, r.dev["X"],
                                    torch.empty(r.n, 128, device="cuda"), r.n))
        serving.spmm_batched(jobs).check()
        outs[g_parts] = [j.Y.cpu().numpy() for j in jobs]
    for a, b in zip(outs[G], outs[4]):
        assert oracle.rel_err(a, b) <= 1e-5
