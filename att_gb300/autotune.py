"""Launch-shape autotuner for the SpMM kernels.

Two shapes are tuned by measurement, not by a model:

* ``att_spmm`` (one graph per call): features per work item and cp.async ring
  depth of the 16-bit kernel (``spmm_fc`` x ``spmm_stages``) or of the fp32
  (3xTF32) kernel (``spmm_tf32``), or the FP8 dequantization kernel
  (``spmm_fp8``).  The best pair depends on how many
  warps stay resident against how deep each warp's prefetch is, which moves
  with F, the dtype and the graph's part lengths.
* ``att_spmm_batched`` (the serving loop): parts per work group.  Larger
  groups mean fewer partial slots to reduce, smaller ones a finer work queue.

``Tuner`` times every candidate with CUDA events on the current stream (the
median of ``reps`` runs after ``warmup`` runs) and keeps the fastest per key,
so each (kernel, dtype, F, format shape) is tuned once per process.  The
timer is injectable, which is how the selection logic is tested without a
GPU.
"""
import math

import torch

from . import _lib, ops


def cuda_timer(run, warmup, reps):
    """Median milliseconds of `run()` on the current stream (CUDA events)."""
    for _ in range(warmup):
        run()
    s = torch.cuda.current_stream()
    times = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(s)
        run()
        b.record(s)
        b.synchronize()
        times.append(a.elapsed_time(b))
    times.sort()
    return times[len(times) // 2]


class Tuner:
    """Pick the fastest candidate per key and remember it."""

    def __init__(self, warmup=2, reps=5, timer=cuda_timer):
        self.warmup, self.reps, self.timer = warmup, reps, timer
        self.cache = {}   # key -> (choice, {candidate: ms})

    def best(self, key, candidates, setup, run):
        """For each candidate: ``setup(c)`` then time ``run()``; returns
        (fastest candidate, {candidate: ms}).  A cached key is not re-timed;
        ``setup`` is applied to its stored choice."""
        if key in self.cache:
            choice, table = self.cache[key]
            setup(choice)
            return choice, table
        if not candidates:
            raise ValueError("no candidates to tune")
        table = {}
        for c in candidates:
            setup(c)
            table[c] = float(self.timer(run, self.warmup, self.reps))
        choice = min(table, key=lambda c: (table[c], candidates.index(c)))
        setup(choice)
        self.cache[key] = (choice, table)
        return choice, table


_default = Tuner()


SHAPE_KNOBS = ("spmm_fc", "spmm_stages", "spmm_fp8", "spmm_tf32")


def clear_shape():
    """Return the calling thread to the process-wide launch-shape defaults."""
    ops.set_launch_shape(None)


def spmm_candidates(x_dtype, F):
    """Launch shapes worth timing for att_spmm with these features."""
    if x_dtype in (torch.float16, torch.bfloat16):
        fcs = (64, 128) if F > 64 else (64,)
        return [("spmm", fc, st) for fc in fcs for st in (2, 3, 4)]
    if x_dtype == torch.float8_e4m3fn:
        return [("fp8", 1), ("fp8", 0)]
    if x_dtype == torch.float32:
        return [("tf32", k) for k in (0, 1, 2, 3)] if F > 32 else []
    return []


def apply_shape(c):
    """Set the calling thread's att_spmm launch shape to candidate `c`."""
    ops.set_launch_shape(c)


def tune_spmm(fmt, X, m_out, x_scale=None, out=None, val=None, tuner=None):
    """Time att_spmm's launch shapes on this format and features (block
    values `val`, default the format's own) and return (choice, {choice:
    ms}).  Candidates are applied to the calling thread only and the thread
    is returned to the defaults afterwards: pass the choice to
    ``ops.spmm(..., shape=choice)`` for the calls it was tuned for.  Shapes
    with nothing to tune (fp32 features with F <= 32) return (None, {})."""
    tuner = tuner or _default
    F = int(X.shape[1])
    cands = spmm_candidates(X.dtype, F)
    if not cands:
        return None, {}
    Y = out if out is not None else torch.empty(m_out, F, dtype=torch.float32, device=X.device)
    parts_bucket = int(math.log2(max(fmt.n_parts, 1)))
    key = ("att_spmm", str(X.dtype), F, fmt.window, fmt.wide, parts_bucket)

    vals = fmt.val if val is None else val

    cur = [None]

    def setup(c):
        cur[0] = c

    def run():
        ops.spmm(fmt.rowptr, fmt.col, vals, fmt.window_of_part, fmt.atomic, X, m_out,
                 window=fmt.window, wide=fmt.wide, out=Y, x_scale=x_scale, shape=cur[0])
    try:
        return tuner.best(key, cands, setup, run)
    finally:
        clear_shape()


def tune_group_parts(requests, candidates=(1, 2, 4, 8), tuner=None):
    """Time the batched SpMM over the prepared `requests` (serving.Request
    with a resident format and features) for each group size; returns
    (fastest group size, {group size: ms})."""
    from . import serving
    tuner = tuner or _default
    reqs = [r for r in requests if r.dev is not None and "fmt" in r.dev]
    if not reqs:
        raise ValueError("no prepared requests to tune on")
    F = int(reqs[0].dev["X"].shape[1])
    built = {}

    def setup(G):
        if G not in built:
            jobs = []
            for r in reqs:
                g = serving.spmm_groups(r.dev["fmt"], G, m_out=r.n)
                part = torch.empty(max(g.n_slots, 1) * 8 * F, dtype=torch.float32,
                                   device="cuda")
                jobs.append(serving.Job(r.dev["fmt"], g, part, r.dev["X"], r.dev["Y"], r.n))
            built[G] = (jobs, serving.BatchedSpmm(len(jobs), use_graph=False))
        setup.cur = built[G]

    def run():
        jobs, b = setup.cur
        b.run(jobs)
    key = ("att_spmm_batched", F, len(reqs), sum(r.n for r in reqs))
    return tuner.best(key, list(candidates), setup, run)
