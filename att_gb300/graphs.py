"""Seeded synthetic power-law graphs (Chung-Lu) standing in for the
reddit / ogbn-arxiv / ogbn-products shapes the reference evaluates
(end2end_ori/gcn_final/eva_gcn_100.py:76-85), whose dataset files are not
available.

``chung_lu`` samples undirected endpoint pairs with probability proportional
to power-law node weights w_i = (i + i0)^(-1/(gamma-1)) (node ids randomly
permuted), symmetrises, removes duplicates and self-pairs, and keeps sampling
until the number of distinct directed edges reaches ``n * mean_deg``; then it
trims at random to that count, adds a self-loop per node (when asked) and
returns a canonical CSR (rows sorted by column).  ``i0`` is chosen so that the
largest expected degree stays below ``max_deg_frac * n``, otherwise a heavy
tail (gamma < 2) would lose most samples to de-duplication.
"""
import math

import numpy as np
import torch


def _offset_for_cap(n, target, alpha, max_deg_frac):
    """Smallest i0 with expected max degree target*w_0/sum(w) <= max_deg_frac*n."""
    idx = np.arange(n, dtype=np.float64)

    def maxdeg(i0):
        w = (idx + i0) ** (-alpha)
        return target * w[0] / w.sum()

    lo, hi = 1.0, 1.0
    while maxdeg(hi) > max_deg_frac * n and hi < 1e9:
        hi *= 2.0
    if hi == 1.0:
        return 1.0
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if maxdeg(mid) > max_deg_frac * n:
            lo = mid
        else:
            hi = mid
    return hi


def chung_lu(n, mean_deg, gamma, seed, self_loops=True, device="cpu", max_deg_frac=0.5,
             batch=1 << 24):
    """Return (rowptr int32 [n+1], col int32 [nnz]) on ``device``."""
    target = int(round(n * mean_deg))
    alpha = 1.0 / (gamma - 1.0)
    i0 = _offset_for_cap(n, target, alpha, max_deg_frac)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    w = (torch.arange(n, dtype=torch.float64, device=device) + i0) ** (-alpha)
    perm = torch.randperm(n, generator=g, device=device)
    cdf = torch.cumsum(w, 0)
    cdf = cdf / cdf[-1]
    keys = torch.empty(0, dtype=torch.int64, device=device)
    need_pairs = target // 2
    rounds = 0
    while keys.numel() < need_pairs and rounds < 64:
        m = int(min(max(need_pairs - keys.numel(), 1024) * 1.3, batch))
        u = torch.searchsorted(cdf, torch.rand(m, generator=g, device=device, dtype=torch.float64))
        v = torch.searchsorted(cdf, torch.rand(m, generator=g, device=device, dtype=torch.float64))
        u = perm[u.clamp_(max=n - 1)]
        v = perm[v.clamp_(max=n - 1)]
        keep = u != v
        u, v = u[keep], v[keep]
        lo_, hi_ = torch.minimum(u, v), torch.maximum(u, v)
        keys = torch.unique(torch.cat([keys, lo_ * n + hi_]))
        rounds += 1
    if keys.numel() > need_pairs:
        sel = torch.randperm(keys.numel(), generator=g, device=device)[:need_pairs]
        keys = torch.sort(keys[sel]).values
    a, b = keys // n, keys % n
    rows = torch.cat([a, b])
    cols = torch.cat([b, a])
    if self_loops:
        ar = torch.arange(n, dtype=torch.int64, device=device)
        rows = torch.cat([rows, ar])
        cols = torch.cat([cols, ar])
    order = torch.argsort(rows * n + cols)
    rows, cols = rows[order], cols[order]
    counts = torch.bincount(rows, minlength=n)
    rowptr = torch.zeros(n + 1, dtype=torch.int64, device=device)
    rowptr[1:] = torch.cumsum(counts, 0)
    return rowptr.to(torch.int32), cols.to(torch.int32)


def gcn_degree(rowptr, dtype=torch.float16):
    """deg = rsqrt(row length) in fp32, then cast (mdataset_fp16.py:54-56)."""
    d = (rowptr[1:] - rowptr[:-1]).to(torch.float32)
    d = torch.rsqrt(d)
    return d.to(dtype)


def pad_rows(rowptr, multiple=8):
    """Pad the CSR with empty rows to n + multiple - n % multiple rows, as the
    reference's loaders do (mdataset_fp16.py:44)."""
    n = rowptr.shape[0] - 1
    n_pad = n + multiple - (n % multiple)
    extra = rowptr[-1:].expand(n_pad - n)
    return torch.cat([rowptr, extra])


def random_csr(n_rows, n_cols, max_len, seed, hub_rows=0, hub_len=0, empty_frac=0.0,
               sort_rows=True, dup=False):
    """Small irregular CSR for tests (numpy, CPU)."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, max_len + 1, size=n_rows)
    if empty_frac > 0:
        lens[rng.random(n_rows) < empty_frac] = 0
    if hub_rows:
        lens[rng.integers(0, n_rows, size=hub_rows)] = hub_len
    cols = []
    for L in lens:
        if dup:
            c = rng.integers(0, n_cols, size=L)
        else:
            c = rng.choice(n_cols, size=min(L, n_cols), replace=False)
        cols.append(np.sort(c) if sort_rows else c)
    lens = np.array([len(c) for c in cols])
    rowptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    col = (np.concatenate(cols) if cols else np.zeros(0)).astype(np.int32)
    return rowptr, col
