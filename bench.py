"""Benchmark of the ATT sparse hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl {ours,reference}]
                    [--workload NAME]

Workloads (synthetic seeded Chung-Lu graphs standing in for the reference's
datasets, which are not available):

  spmm_products_fp16   blocked SpMM Y = A_hat X, N = 2,449,029 nodes (ogbn-products
                       shape), gamma 2.2, mean degree 25 (~62M edges) + self-loops,
                       GCN-normalised fp16 values, X [N, 128] fp16 U[-1,1] with 100
                       real dims and 28 zero dims, reference block format
                       (8-row windows, 8-wide blocks, partSize 32), fp32 output.

One step = one pass of the hot path over the whole graph.  ``value`` is
algorithmic GB/s (bytes defined in the roofline note below) with inputs
resident in HBM; every input (format 1.2 GB, X 0.6 GB) is larger than L2, so
no flush is needed between steps.  ``e2e`` times the same step through the
reference-facing drop-in (``SpMM_sr_bcrs.forward_fp16_gnn``) with X copied
from pinned host memory and Y copied back every step, pipelined over two
buffer sets so that step i's copy in, step i-1's kernel and step i-2's copy
out overlap.

Multi-GPU: the path runs as independent replicas (one whole graph per GPU,
weak scaling; no collective on the data path).

``--impl reference`` times the reference's CPU path for this op, restated in
the oracle (torch.sparse CSR SpMM in fp32 on all host cores), on a bounded
sample of rows of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes per launch of the dominant kernel, from one ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum, --clock-control none, GB300)
# of the named kernel at the named launch shape on the full-size workload:
# a profiler counter cannot be read inside the timed run, so the figure is
# carried here with its source (kernel, shape, the commit it was captured
# at).  roofline() uses an entry only when the run timed the same launch
# shape; otherwise it reports traffic null and an algorithmic fraction.
MEASURED_TRAFFIC = {
    ("spmm_products_fp16", 1.0): {
        "bytes": 9881965568 + 1404438784, "shape": ("spmm", 64, 3),
        "kernel": "k_spmm16<__half, 8, 64, 8, 3, int, 1>", "ncu_ms": 2.128, "commit": "6b938d9",
        "profile": "profiles/spmm16_products_fp16_full_dram.md",
        "note": "read 9.88 GB + write 1.40 GB; X rows of hub columns hit L2 (37.0 % of sectors)"},
    ("spmm_products_fp8", 1.0): {
        "bytes": 5512719360 + 1383769344, "shape": ("fp8", 1),
        "kernel": "k_spmm_fp8r<8, 128, 8, int, 1>", "ncu_ms": 1.805, "commit": "6b938d9",
        "profile": "profiles/spmm_fp8r_products_fp8_full_dram.md",
        "note": "read 5.51 GB + write 1.38 GB; L2 hit rate 48.7 % of sectors"},
}
METRIC = "SpMM/SDDMM HBM GB/s (% roofline); GAT step ms; serve p50/p99 vs plain"


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ---------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def distinct_window_columns(rowptr, col, window=8):
    """Number of distinct (row // window, column) pairs of a host CSR: the X
    rows a blocked kernel gathers."""
    import torch
    rowptr = torch.as_tensor(rowptr).long()
    n = rowptr.numel() - 1
    rows = torch.repeat_interleave(torch.arange(n), rowptr[1:] - rowptr[:-1])
    key = (rows // window) * (int(col.max()) + 1 if col.numel() else 1) + torch.as_tensor(col).long()
    return int(torch.unique(key).numel())


class PipelinedE2E:
    """End-to-end steps pipelined over two buffer sets and three streams, as a
    serving caller would run them: step i's input copy (pinned host -> device,
    copy-in stream) overlaps step i-1's kernels (compute stream) and step
    i-2's result copy (device -> pinned host, copy-out stream).  Every step
    still moves its whole input in and its whole result out inside the timed
    region; `e2e_begin` orders the first copy after the region's start event
    and `e2e_finish` joins the copy-out stream back before the stop event.
    The result tensor of step i is held until its copy-out has completed and
    released on the compute stream after waiting for that copy, so step i+2
    reuses its memory: no allocation outlives its use (a `record_stream`
    here let the caching allocator grow by one result per step and
    periodically free them all, stalling a step by about 100 ms)."""

    def _pipe_setup(self, host_in, host_out_shape):
        torch = self.torch
        self._cin = torch.cuda.Stream()
        self._cout = torch.cuda.Stream()
        self._din = [[torch.empty(h.shape, dtype=h.dtype, device="cuda") for h in host_in]
                     for _ in range(2)]
        self._hin = host_in
        self._hout = [torch.empty(host_out_shape, dtype=torch.float32).pin_memory()
                      for _ in range(2)]
        self._done = [None, None]  # compute event of the last step that read buffer set b
        self._held = [None, None]  # (result tensor, its copy-out event) of buffer set b
        self._it = 0

    def e2e_begin(self):
        self._cin.wait_stream(self.torch.cuda.current_stream())

    def e2e_finish(self):
        self.torch.cuda.current_stream().wait_stream(self._cout)

    def _pipe_step(self, compute):
        torch = self.torch
        cur = torch.cuda.current_stream()
        b = self._it & 1
        self._it += 1
        if self._done[b] is not None:
            self._cin.wait_event(self._done[b])
        with torch.cuda.stream(self._cin):
            for d, h in zip(self._din[b], self._hin):
                d.copy_(h, non_blocking=True)
        cur.wait_stream(self._cin)
        if self._held[b] is not None:  # free step i-2's result once its copy is done
            cur.wait_event(self._held[b][1])
            self._held[b] = None
        out = compute(*self._din[b])
        ev = torch.cuda.Event()
        ev.record(cur)
        self._done[b] = ev
        self._cout.wait_event(ev)
        with torch.cuda.stream(self._cout):
            self._hout[b].copy_(out, non_blocking=True)
            copied = torch.cuda.Event()
            copied.record(self._cout)
        self._held[b] = (out, copied)


class SpmmProducts(PipelinedE2E):
    """Blocked FP16 SpMM on the 2.45M-node power-law graph."""
    name = "spmm_products_fp16"
    unit = "GB/s"
    N, MEAN_DEG, GAMMA, SEED, F, F_REAL = 2_449_029, 25, 2.2, 2, 128, 100

    e2e_api = "SpMM_sr_bcrs.forward_fp16_gnn"
    x_kind = "fp16"

    def __init__(self, device, scale=1.0, light=False):
        import torch
        from att_gb300 import graphs
        self.torch = torch
        n = int(self.N * scale)
        self.n = n
        rp, col = graphs.chung_lu(n, self.MEAN_DEG, self.GAMMA, self.SEED, device=device)
        rp = graphs.pad_rows(rp, 8)
        self.rowptr, self.colidx = rp, col
        deg = graphs.gcn_degree(rp, torch.float16)
        deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg))
        self.deg = deg
        g = torch.Generator(device=device)
        g.manual_seed(self.SEED)
        X = torch.rand(n, self.F, generator=g, device=device, dtype=torch.float32) * 2 - 1
        X[:, self.F_REAL:] = 0
        self.X = X.half()
        self.nnz = int(col.shape[0])
        if light:  # CSR and features only: no kernel of this package runs
            self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz,
                           "features": self.F, "real_features": self.F_REAL}
            return
        from att_gb300 import ops
        self.fmt = ops.block_convert(rp, col, deg, window=8, wide=8, part=32)
        self.Y = torch.empty(n, self.F, device=device, dtype=torch.float32)
        f = self.fmt
        real = (f.rowptr[1::2] - f.rowptr[0:-1:2]).sum().item()
        self.U = int(real)  # distinct (8-row window, column) pairs = gathered X rows
        F = self.F
        self.val = f.val
        self.x_scale = None
        self.Xk = self.X
        sx = 2
        self.Xf64 = X.double()  # unquantized features (for the error report)
        if self.x_kind == "bf16":
            self.val = f.val.to(torch.bfloat16)
            self.Xk = X.to(torch.bfloat16)
        elif self.x_kind == "fp8":
            amax = X.abs().amax(1).clamp_min(1e-12)
            self.x_scale = (amax / 448.0).float().contiguous()
            self.Xk = (X / self.x_scale[:, None]).to(torch.float8_e4m3fn)
            sx = 1
        self.bytes_alg = (4 * (n + 1) + self.nnz * (4 + 2) + self.U * F * sx + n * F * 4
                          + (self.U * 4 if self.x_kind == "fp8" else 0))
        # the same pass with fp16 features: the yardstick for comparing forms
        self.bytes_fp16 = 4 * (n + 1) + self.nnz * (4 + 2) + self.U * F * 2 + n * F * 4
        # compulsory: the resident format once, every X row once, Y once (a
        # lower bound on the DRAM traffic of any schedule)
        s_v = 2
        self.bytes_format = (4 * (2 * f.n_parts + 1) + 4 * f.n_condensed
                             + s_v * f.n_condensed * 8 + 8 * f.n_parts)
        self.bytes_compulsory = (self.bytes_format + n * F * sx + n * F * 4
                                 + (n * 4 if self.x_kind == "fp8" else 0))
        self.flops = 2 * self.nnz * F
        self.launches_per_step = 2  # k_zero_uncovered + k_spmm16
        self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz,
                       "features": F, "real_features": self.F_REAL, "gamma": self.GAMMA,
                       "mean_degree": self.MEAN_DEG, "seed": self.SEED,
                       "format": "window 8, wide 8, partSize 32",
                       "parts": f.n_parts, "condensed_cols": f.n_condensed,
                       "gathered_rows_U8": self.U, "x_dtype": self.x_kind, "y_dtype": "fp32",
                       "l2": "inputs larger than L2 (no flush)"}

    shape = None  # att_spmm launch shape of every call (None: the library defaults)

    def step(self):
        from att_gb300 import ops
        f = self.fmt
        ops.spmm(f.rowptr, f.col, self.val, f.window_of_part, f.atomic, self.Xk, self.n,
                 out=self.Y, x_scale=self.x_scale, shape=self.shape)

    def autotune(self, pinned=None):
        """Launch shape of att_spmm picked by the autotuner on this graph (or
        `pinned`, untimed), used by every later call of this workload."""
        from att_gb300 import autotune
        if pinned is not None:
            self.shape = tuple(pinned)
            return {"choice": list(self.shape), "ms_by_shape": None, "pinned": True}
        choice, table = autotune.tune_spmm(self.fmt, self.Xk, self.n, x_scale=self.x_scale,
                                           out=self.Y, val=self.val)
        self.shape = choice
        return {"choice": list(choice) if choice else None,
                "ms_by_shape": {"/".join(str(v) for v in k): ms for k, ms in table.items()}}

    # end to end through the reference-facing drop-in, host buffers
    def e2e_setup(self):
        Xh = self.Xk.cpu().pin_memory()
        from att_gb300.compat import SpMM_sr_bcrs
        self._mod = SpMM_sr_bcrs
        self._pipe_setup([Xh], (self.n, self.F))
        self.h2d = Xh.numel() * Xh.element_size()
        self.d2h = self.n * self.F * 4

    def _e2e_compute(self, Xd):
        f = self.fmt
        if self.x_kind == "fp16":
            return self._mod.forward_fp16_gnn(f.rowptr, f.col, f.val, f.window_of_part, f.atomic,
                                              Xd, self.rowptr.shape[0] - 1, self.F, self.n)[0]
        from att_gb300 import ops
        return ops.spmm(f.rowptr, f.col, self.val, f.window_of_part, f.atomic, Xd, self.n,
                        x_scale=self.x_scale)

    def e2e_step(self):
        self._pipe_step(self._e2e_compute)

    # the plain FP16 drop-in: the reference's own kernel on the fp16 data
    def plain_available(self):
        from oracle import ref_spmm
        return ref_spmm.available() and self.F % 16 == 0

    plain_kind = ("the reference's forward_fp16_gnn kernel (gcn/SpMM/src/spmmKernel.cu:158-265, "
                  "fp16 accumulation) built for sm_103a, on the fp16 form of the same data")

    def plain_step(self):
        from oracle import ref_spmm
        f = self.fmt
        return ref_spmm.forward_fp16_gnn(f.rowptr, f.col, f.val, f.window_of_part, f.atomic,
                                         self.X, self.rowptr.shape[0] - 1, self.F, self.n)[0]

    def check(self):
        """Size-independent property at full size: A_hat applied to a constant
        column equals the per-row sum of the block values (checksum of checksums)."""
        torch = self.torch
        from att_gb300 import ops
        ones = torch.zeros(self.n, 8, device=self.X.device, dtype=torch.float16)
        ones[:, 0] = 1
        f = self.fmt
        Y1 = ops.spmm(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, ones, self.n)[:, 0]
        rows = torch.repeat_interleave(torch.arange(self.rowptr.shape[0] - 1, device=self.X.device),
                                       (self.rowptr[1:] - self.rowptr[:-1]).long())
        ev = (self.deg[rows].float() * self.deg[self.colidx.long()].float()).half().float()
        rs = torch.zeros(self.rowptr.shape[0] - 1, device=self.X.device).index_add_(0, rows, ev)
        err = ((Y1 - rs[: self.n]).abs().max() / rs.abs().max().clamp_min(1e-30)).item()
        from att_gb300 import ops
        Y = ops.spmm(f.rowptr, f.col, self.val, f.window_of_part, f.atomic, self.Xk, self.n,
                     x_scale=self.x_scale, shape=self.shape)
        self.err_vs_fp64 = self.sample_error(Y)
        if self.x_kind == "fp8":
            # the kernel's arithmetic alone: FP64 of the dequantized features
            self.err_vs_fp64_own_inputs = self.sample_error(
                Y, X64=(self.Xk.float() * self.x_scale[:, None]).double())
        if self.plain_available():
            self.plain_err_vs_fp64 = self.sample_error(self.plain_step(), X64=self.X.double())
        return err

    def sample_error(self, Y, rows=20000, X64=None):
        """Error of an output Y against the FP64 product for the first `rows`
        rows of the full graph (normwise max and Frobenius relative).  X64
        defaults to the features before this form's rounding (fp16 for the
        fp16 form, the unquantized fp32 values for bf16 / fp8)."""
        torch = self.torch
        rows = min(rows, self.n)
        rp = self.rowptr[: rows + 1].long()
        col = self.colidx[: int(rp[-1])].long()
        ridx = torch.repeat_interleave(torch.arange(rows, device=rp.device), rp[1:] - rp[:-1])
        vals = (self.deg[ridx].float() * self.deg[col].float()).half().double()
        if X64 is None:
            X64 = self.X.double() if self.x_kind == "fp16" else self.Xf64
        ref = torch.zeros(rows, self.F, dtype=torch.float64, device=rp.device)
        ref.index_add_(0, ridx, vals[:, None] * X64[col])
        got = Y[:rows].double()
        d = (got - ref)
        return {"rows": rows, "max_rel": float(d.abs().max() / ref.abs().max()),
                "fro_rel": float(d.norm() / ref.norm())}

    # CPU baseline: the oracle's restatement of the reference's CPU path
    def cpu_sample(self, max_rows):
        """CSR fp32 of the first `max_rows` rows (host), and the algorithmic bytes."""
        torch = self.torch
        rows = min(max_rows, self.n)
        rp = self.rowptr[: rows + 1].cpu().long()
        col = self.colidx[: int(rp[-1])].cpu().long()
        ridx = torch.repeat_interleave(torch.arange(rows), rp[1:] - rp[:-1])
        d = self.deg.cpu().float()
        vals = (d[ridx] * d[col]).half().float()
        X = self.X.float().cpu()
        U = distinct_window_columns(rp, col)
        nnz = int(col.shape[0])
        b = 4 * (rows + 1) + nnz * (4 + 2) + U * self.F * 2 + rows * self.F * 4
        return rp, col, vals, X, rows, b


class GatReddit(PipelinedE2E):
    """One GAT layer forward on the 232,965-node graph: X' = X W (cuBLAS), then
    the fused SDDMM -> LeakyReLU -> edge softmax -> SpMM kernel."""
    name = "gat_reddit_fp16"
    unit = "GB/s"
    N, MEAN_DEG, GAMMA, SEED, F = 232_965, 490, 1.9, 1, 64

    e2e_api = "att_gb300.gat.GATGraph.attention (C ABI att_gat_forward) after torch.mm"

    def __init__(self, device, scale=1.0, light=False):
        import torch
        from att_gb300 import graphs
        self.torch = torch
        n = max(int(self.N * scale), 64)
        self.n = n
        rp, col = graphs.chung_lu(n, self.MEAN_DEG * min(1.0, scale ** 0.5), self.GAMMA,
                                  self.SEED, device=device)
        self.rowptr, self.colidx = rp, col
        g = torch.Generator(device=device)
        g.manual_seed(self.SEED)
        F = self.F
        self.X = (torch.rand(n, F, generator=g, device=device) * 2 - 1).half()
        a = (6.0 / (F + F)) ** 0.5  # Glorot-uniform bound
        self.W = ((torch.rand(F, F, generator=g, device=device) * 2 - 1) * a).half()
        self.nnz = int(col.shape[0])
        if light:  # CSR and features only: no kernel of this package runs
            self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz, "features": F}
            return
        from att_gb300 import gat
        self.G = gat.GATGraph(rp, col)
        self.out = torch.empty(n, F, device=device, dtype=torch.float32)
        f = self.G.fmt
        self.U = int((f.rowptr[1::2] - f.rowptr[0:-1:2]).sum().item())
        # fused kernel: CSR-granular structure + query rows + gathered rows + output
        self.bytes_fused = 4 * (n + 1) + 4 * self.nnz + n * F * 2 + self.U * F * 2 + n * F * 4
        self.bytes_alg = self.bytes_fused + 2 * n * F * 2  # + the projection's X read, X' write
        # compulsory for the fused kernel: the resident structure (rowptr pairs,
        # columns, slot bitmap, window ids) once, X' once, the output once
        self.bytes_structure = (4 * (2 * f.n_parts + 1) + 4 * f.n_condensed + f.n_condensed
                                + 4 * f.n_parts)
        self.bytes_compulsory = self.bytes_structure + n * F * 2 + n * F * 4
        self.flops = 2 * n * F * F + 4 * self.nnz * F
        self.launches_per_step = 2 + (1 if self.G.n_multi else 0)
        self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz, "features": F,
                       "heads": 1, "gamma": self.GAMMA, "mean_degree": self.MEAN_DEG,
                       "seed": self.SEED, "format": "window 8, wide 8, partSize 32",
                       "parts": f.n_parts, "condensed_cols": f.n_condensed,
                       "gathered_rows_U8": self.U, "chunks": self.G.n_chunks,
                       "split_windows": self.G.n_multi, "x_dtype": "fp16", "out_dtype": "fp32",
                       "attention": "dot-product logits (X W)(X W)^T on the edges, "
                                    "LeakyReLU 0.2, row softmax with fp32 max/sum",
                       "l2": "X' (30 MB) is L2-resident; structure arrays are larger than L2"}

    kernel_name = "att_gat_forward (k_gat_zero_rows + k_gat_fused + k_gat_combine)"

    def step(self):
        Xp = self.torch.mm(self.X, self.W)
        self.G.attention(Xp, out=self.out, stats=False)

    def kernel_step(self):
        """the dominant kernel launch alone (for the roofline timing)"""
        self.G.attention(self.Xp, out=self.out, stats=False)

    def prepare_kernel(self):
        self.Xp = self.torch.mm(self.X, self.W)

    def e2e_setup(self):
        Xh = self.X.cpu().pin_memory()
        Wh = self.W.cpu().pin_memory()
        self._pipe_setup([Xh, Wh], (self.n, self.F))
        self.h2d = Xh.numel() * 2 + Wh.numel() * 2
        self.d2h = self.n * self.F * 4

    def _e2e_compute(self, X, W):
        out, _, _ = self.G.attention(self.torch.mm(X, W), stats=False)
        return out

    def e2e_step(self):
        self._pipe_step(self._e2e_compute)

    def plain_step(self):
        """The reference's chain of separate ops for the same layer (SDDMM,
        LeakyReLU, row softmax, SpMM of the edge values), same dtype."""
        if getattr(self, "chain", None) is None:
            from att_gb300 import gat
            self.chain = gat.DotAttentionChain(self.rowptr, self.colidx)
        return self.chain(self.torch.mm(self.X, self.W))

    def sample_error(self, out, Xp, rows=2000):
        """Error of the layer's output against the FP64 layer on the same X'
        for the first `rows` rows (normwise max and Frobenius relative)."""
        torch = self.torch
        rows = min(rows, self.n)
        rp = self.rowptr[: rows + 1].long()
        col = self.colidx[: int(rp[-1])].long()
        lengths = rp[1:] - rp[:-1]
        ridx = torch.repeat_interleave(torch.arange(rows, device=rp.device), lengths)
        Xd = Xp.double()
        e = torch.nn.functional.leaky_relu((Xd[ridx] * Xd[col]).sum(1), 0.2)
        m = torch.segment_reduce(e, "max", lengths=lengths, unsafe=True)
        pe = torch.exp(e - m[ridx])
        pe = pe / torch.segment_reduce(pe, "sum", lengths=lengths, unsafe=True)[ridx]
        ref = torch.zeros(rows, Xp.shape[1], dtype=torch.float64, device=rp.device)
        ref.index_add_(0, ridx, pe[:, None] * Xd[col])
        d = out[:rows].double() - ref
        return {"rows": rows, "max_rel": float(d.abs().max() / ref.abs().max()),
                "fro_rel": float(d.norm() / ref.norm())}

    def check(self):
        """Size-independent property at full size: every output row is a convex
        combination of its neighbours' X' rows, so it lies within their
        per-feature min/max (checked on a sample of rows against the CSR).
        Also the error against the FP64 layer on a row sample."""
        torch = self.torch
        Xp = torch.mm(self.X, self.W).float()
        out, rmax, rsum = self.G.attention(Xp.half())
        self.err_vs_fp64 = self.sample_error(out, Xp.half())
        rp = self.rowptr.long()
        worst = 0.0
        for r in torch.linspace(0, self.n - 1, 64).long().tolist():
            nb = self.colidx[rp[r]:rp[r + 1]].long()
            if nb.numel() == 0:
                continue
            lo = Xp[nb].min(0).values
            hi = Xp[nb].max(0).values
            span = (hi - lo).abs().max().clamp_min(1e-6)
            over = torch.clamp(out[r] - hi, min=0).max() + torch.clamp(lo - out[r], min=0).max()
            worst = max(worst, float(over / span))
        return worst

    def cpu_sample(self, max_rows):
        torch = self.torch
        rows = min(max_rows, self.n)
        rp = self.rowptr[: rows + 1].cpu().long()
        col = self.colidx[: int(rp[-1])].cpu().long()
        Xp = torch.mm(self.X.float().cpu(), self.W.float().cpu())
        U = distinct_window_columns(rp, col)
        nnz = int(col.shape[0])
        b = 4 * (rows + 1) + 4 * nnz + rows * self.F * 2 + U * self.F * 2 + rows * self.F * 4
        return rp, col, Xp, rows, b


class GatArxivTrain:
    """2-layer GAT training step: forward, fused backward and Adam on the
    169,343-node graph (4 heads x 64 hidden, 40 classes, BF16 features,
    cross-entropy on uniform random labels)."""
    name = "gat_arxiv_train_bf16"
    unit = "ms"
    higher_is_better = False
    N, MEAN_DEG, GAMMA, SEED, F_IN, HID, HEADS, CLASSES = 169_343, 14, 2.1, 3, 128, 64, 4, 40
    e2e_api = "att_gb300.layers.GATNet (fused GATAttention forward/backward) + torch.optim.Adam"
    kernel_name = "att_gat_forward, layer 1 (4 heads x 64)"

    def __init__(self, device, scale=1.0, light=False):
        import torch
        from att_gb300 import graphs
        self.torch = torch
        n = max(int(self.N * scale), 64)
        self.n = n
        rp, col = graphs.chung_lu(n, self.MEAN_DEG, self.GAMMA, self.SEED, device=device)
        self.rowptr, self.colidx = rp, col
        self.nnz = int(col.shape[0])
        g = torch.Generator(device=device)
        g.manual_seed(self.SEED)
        self.X = torch.rand(n, self.F_IN, generator=g, device=device).bfloat16()
        self.y = torch.randint(0, self.CLASSES, (n,), generator=g, device=device)
        self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz,
                       "features": self.F_IN, "hidden": self.HID, "heads": self.HEADS,
                       "classes": self.CLASSES, "gamma": self.GAMMA,
                       "mean_degree": self.MEAN_DEG, "seed": self.SEED, "dtype": "bf16",
                       "optimizer": "Adam lr 1e-2 wd 5e-4",
                       "loss": "mean negative log-likelihood of log_softmax (gather + mean)"}
        if light:
            return
        from att_gb300 import layers
        rows = torch.repeat_interleave(torch.arange(n, device=device), (rp[1:] - rp[:-1]).long())
        self.info = layers.GATInput(rows.cpu(), col.long().cpu(), n)
        self.info.fused_graph()
        torch.manual_seed(0)
        self.net = layers.GATNet(self.F_IN, self.HID, self.CLASSES, heads=self.HEADS,
                                 impl="fused").cuda()
        self.opt = torch.optim.Adam(self.net.parameters(), lr=1e-2, weight_decay=5e-4)
        torch.manual_seed(0)
        self.plain = layers.GATNet(self.F_IN, self.HID, self.CLASSES, heads=self.HEADS,
                                   impl="dropin").cuda()
        self.opt_plain = torch.optim.Adam(self.plain.parameters(), lr=1e-2, weight_decay=5e-4)
        G = self.info.fused_graph()
        f = G.fmt
        self.U = int((f.rowptr[1::2] - f.rowptr[0:-1:2]).sum().item())
        F = self.HEADS * self.HID
        self.bytes_fused = 4 * (n + 1) + 4 * self.nnz + n * F * 2 + self.U * F * 2 + n * F * 4
        self.bytes_alg = self.bytes_fused
        self.flops = 0
        self.launches_per_step = 12  # node scores x2, fused fwd (3) x2 layers, bwd x2, ...
        self.config.update({"parts": f.n_parts, "condensed_cols": f.n_condensed,
                            "gathered_rows_U8": self.U})

    @staticmethod
    def nll(logp, y):
        """Mean negative log-likelihood of the labels (nll_loss's value), as a
        gather and a mean: torch's nll_loss kernel reduces in one CTA."""
        return -logp.gather(1, y[:, None]).mean()

    def _train(self, net, opt, X, y):
        # backward on the calling thread (no hop to autograd's device thread)
        with self.torch.autograd.set_multithreading_enabled(False):
            loss = self.nll(net(X, self.info), y)
            opt.zero_grad(set_to_none=True)
            loss.backward()
        opt.step()
        return loss

    def step(self):
        self.last_loss = self._train(self.net, self.opt, self.X, self.y)

    def plain_step(self):
        self._train(self.plain, self.opt_plain, self.X.half(), self.y)

    def prepare_kernel(self):
        torch = self.torch
        from att_gb300 import gat_ops
        layer = self.net.layers[0]
        G = self.info.fused_graph()
        self.Xp = torch.mm(self.X, layer.W.detach().to(torch.bfloat16)).contiguous()
        X3 = self.Xp.view(self.n, self.HEADS, self.HID).permute(1, 0, 2)
        self.s0 = gat_ops.node_scores(X3, layer.a0.detach().float())
        self.s1 = gat_ops.node_scores(X3, layer.a1.detach().float())

    def kernel_step(self):
        from att_gb300 import gat
        self.info.fused_graph().attention(self.Xp, n_heads=self.HEADS, mode=gat.MODE_ADD,
                                          s0=self.s0, s1=self.s1, stats=False)

    def e2e_setup(self):
        self.Xh = self.X.cpu().pin_memory()
        self.yh = self.y.cpu().pin_memory()
        self.h2d = self.Xh.numel() * 2 + self.yh.numel() * 8
        self.d2h = 4

    def e2e_step(self):
        X = self.Xh.to("cuda", non_blocking=True)
        y = self.yh.to("cuda", non_blocking=True)
        loss = self._train(self.net, self.opt, X, y)
        loss.to("cpu", non_blocking=True)

    def check(self):
        """Gradient sanity at full size: the fused layer-1 gradient of a random
        projection agrees with the plain drop-in chain's (normwise relative
        difference; both fp16-class)."""
        torch = self.torch
        from att_gb300 import layers
        G = self.info.fused_graph()
        torch.manual_seed(1)
        plain = layers.GATConv_multi(self.F_IN, self.HID, 0.0, 0.2, self.HEADS).cuda()
        fused = layers.FusedGATConv(self.F_IN, self.HID, self.HEADS, 0.2,
                                    dtype=torch.float16).cuda()
        with torch.no_grad():
            fused.W.copy_(plain.fc.weight.t())
            fused.a0.copy_(plain.a0[:, 0, :])
            fused.a1.copy_(plain.a1[:, 0, :])
        X = self.X.half()
        R = torch.randn(self.n, self.HEADS, self.HID, device=X.device)
        (plain(X, self.info)[: self.n].float() * R).sum().backward()
        (fused(X, G).float() * R).sum().backward()
        a, b = fused.W.grad.float(), plain.fc.weight.grad.t().float()
        return float((a - b).abs().max() / b.abs().max())

    def cpu_sample(self, max_rows):
        raise NotImplementedError


class GatRedditTF32(GatReddit):
    """The same GAT layer in fp32: X' = X W in fp32, then the fused kernel on
    TF32 tensor cores (3xTF32 logits and aggregation); the plain comparison
    is the chain of separate ops on the TF32 kernels (att_sddmm, row softmax,
    att_spmm)."""
    name = "gat_reddit_tf32"
    e2e_api = "att_gb300.gat.GATGraph.attention (C ABI att_gat_forward, fp32 / 3xTF32) after torch.mm"
    kernel_name = "att_gat_forward fp32 (k_gat_zero_rows + k_gat_fused<float> + k_gat_combine)"

    def __init__(self, device, scale=1.0, light=False):
        super().__init__(device, scale=scale, light=light)
        self.X = self.X.float()
        self.W = self.W.float()
        F, n = self.F, self.n
        self.config["workload"] = self.name
        if light:
            return
        from att_gb300 import gat
        self.chain = gat.DotAttentionChain(self.rowptr, self.colidx)
        # the layer's algorithmic bytes with fp32 operands (as the fused count)
        self.bytes_fused = 4 * (n + 1) + 4 * self.nnz + n * F * 4 + self.U * F * 4 + n * F * 4
        self.bytes_alg = self.bytes_fused + 2 * n * F * 4
        self.bytes_compulsory = self.bytes_structure + n * F * 4 + n * F * 4
        self.config.update({"x_dtype": "fp32 (TF32 tensor cores, 3xTF32 split)",
                            "path": "fused kernel; plain = chain of separate ops"})

    def step(self):
        self.G.attention(self.torch.mm(self.X, self.W), out=self.out, stats=False)

    def plain_step(self):
        return self.chain(self.torch.mm(self.X, self.W))

    def prepare_kernel(self):
        self.Xp = self.torch.mm(self.X, self.W)

    def kernel_step(self):
        self.G.attention(self.Xp, out=self.out, stats=False)

    def _e2e_compute(self, X, W):
        out, _, _ = self.G.attention(self.torch.mm(X, W), stats=False)
        return out

    def e2e_setup(self):
        super().e2e_setup()
        self.h2d = self.n * self.F * 4 + self.F * self.F * 4

    def check(self):
        Xp = self.torch.mm(self.X, self.W)
        out, _, _ = self.G.attention(Xp)
        self.err_vs_fp64 = self.sample_error(out, Xp)
        chain = self.chain(Xp)
        self.chain_err_vs_fp64 = self.sample_error(chain, Xp)
        return self.err_vs_fp64["max_rel"]


class SpmmProductsBF16(SpmmProducts):
    """The same SpMM with BF16 features and BF16 block values."""
    name = "spmm_products_bf16"
    e2e_api = "att_gb300.ops.spmm (C ABI att_spmm), bf16"
    x_kind = "bf16"


class SpmmProductsFP8(SpmmProducts):
    """The same SpMM with FP8 E4M3 features and per-row fp32 scales (fp16 values)."""
    name = "spmm_products_fp8"
    e2e_api = "att_gb300.ops.spmm (C ABI att_spmm), fp8 e4m3 + row scales"
    x_kind = "fp8"
    kernel_name = "att_spmm (k_zero_uncovered + k_spmm_fp8r)"


class ConvertProducts:
    """CSR -> row-window block format (8-row windows, 8-wide blocks,
    partSize 32, fp16 GCN values) of the 2.45M-node graph on the GPU: the
    reference's blockProcess_fp16_balance (gcn/Block_gcn/example.cpp:48-200)."""
    name = "convert_products_fp16"
    unit = "GB/s"
    e2e_api = "Block_sr_bcrs.blockProcess_fp16_balance (host CSR in, host format out)"
    kernel_name = ("att_block_plan + att_block_fill (k_unique_warp, k_chunk_rows, k_merge_rank, "
                   "scans, k_merge_emit, k_window_counts, k_fill_cols, k_fill_parts, "
                   "k_fill_edges)")

    def __init__(self, device, scale=1.0, light=False):
        import torch
        from att_gb300 import graphs
        self.torch = torch
        c = SpmmProducts
        n = int(c.N * scale)
        self.n = n
        rp, col = graphs.chung_lu(n, c.MEAN_DEG, c.GAMMA, c.SEED, device=device)
        rp = graphs.pad_rows(rp, 8)
        deg = graphs.gcn_degree(rp, torch.float16)
        self.rowptr, self.colidx = rp, col
        self.deg = torch.where(torch.isfinite(deg), deg, torch.zeros_like(deg))
        self.nnz = int(col.shape[0])
        self.config = {"workload": self.name, "nodes": n, "nnz": self.nnz, "gamma": c.GAMMA,
                       "mean_degree": c.MEAN_DEG, "seed": c.SEED,
                       "format": "window 8, wide 8, partSize 32, fp16 values"}
        if light:
            return
        self.step()
        f = self.fmt
        self.bytes_out = (4 * (2 * f.n_parts + 1) + 4 * f.n_condensed + 2 * f.n_condensed * 8
                          + 8 * f.n_parts)
        self.bytes_alg = 4 * (rp.shape[0]) + 4 * self.nnz + 2 * rp.shape[0] + self.bytes_out
        self.bytes_compulsory = self.bytes_alg
        self.flops = 0
        self.launches_per_step = 24  # plan 20 (its int32 scan 5 here) + fill 4
        self.config.update({"parts": f.n_parts, "condensed_cols": f.n_condensed,
                            "l2": "inputs and outputs larger than L2 (no flush)"})

    def step(self):
        from att_gb300 import ops
        self.fmt = ops.block_convert(self.rowptr, self.colidx, self.deg, window=8, wide=8, part=32)

    def check(self):
        """Structure of the whole format: rowptr pairs non-decreasing and
        within the column array, real columns of each part sorted and valid
        (the full bit-exact comparison with the oracle is a GPU test)."""
        torch = self.torch
        f = self.fmt
        rp = f.rowptr.long()
        ok = bool((rp[1:] >= rp[:-1]).all()) and int(rp[-1]) == f.n_condensed
        col = f.col.long()
        ok = ok and bool(((col >= -1) & (col < self.n)).all())
        return 0.0 if ok else 1.0

    def e2e_setup(self):
        torch = self.torch
        from att_gb300.compat import Block_sr_bcrs
        self._mod = Block_sr_bcrs
        self._h = [self.rowptr.cpu().pin_memory(), self.colidx.cpu().pin_memory(),
                   self.deg.cpu().pin_memory()]
        self.h2d = sum(t.numel() * t.element_size() for t in self._h)
        self.d2h = self.bytes_out

    def e2e_step(self):
        rp, col, deg = self._h
        self._mod.blockProcess_fp16_balance(rp, col, deg, 8, 8, 32)

    def cpu_port(self):
        """The oracle's C restatement of the reference's conversion, one host
        core, the whole graph: (seconds, oracle output)."""
        from oracle import oracle as orc
        rp = self.rowptr.cpu().numpy()
        col = self.colidx.cpu().numpy()
        deg = self.deg.cpu().numpy()
        t0 = time.perf_counter()
        o = orc.block_convert(rp, col, deg, 8, 8, 32)
        return time.perf_counter() - t0, o


def _convert_form(torch, stream, steps, warmup):
    wl = ConvertProducts("cuda")
    wl.check()
    rec = measure(wl, torch, stream, steps, warmup, e2e=False, plain=False)
    peak, peak_kind = peaks()
    gbs = wl.bytes_alg / (rec["ms_per_step"] * 1e-3) / 1e9
    sec, _ = wl.cpu_port()
    out = {"ms": rec["ms_per_step"], "gbs": gbs, "frac_of_hbm_peak": gbs / peak,
           "peak_kind": peak_kind, "bytes": wl.bytes_alg,
           "cpu_baseline": {"value_ms": sec * 1e3, "cores": 1, "kind": "port",
                            "sample": "the whole graph through oracle/block_oracle.c (the C "
                                      "restatement of example.cpp:48-200), one host core"},
           "speedup_vs_cpu": sec * 1e3 / rec["ms_per_step"]}
    del wl
    _free(torch)
    return out


class SpmmGcn16k(SpmmProducts):
    """GCN aggregation SpMM on the 16,384-node power-law graph (gamma 2.1,
    mean degree 10, seed 0), X [N, 64] fp16 U[-1,1]: the correctness case of
    the reference's own forward_fp16_gnn.  Its inputs (2 MB of features, a few
    MB of format) fit in L2, so L2 is flushed between timed steps, outside the
    timed events; the call is launch-latency bound."""
    name = "spmm_gcn16k_fp16"
    N, MEAN_DEG, GAMMA, SEED, F, F_REAL = 16_384, 10, 2.1, 0, 64, 64
    l2_flush = True

    def __init__(self, device, scale=1.0, light=False):
        super().__init__(device, scale=scale, light=light)
        self.config["l2"] = "L2 flushed between timed steps (256 MiB write outside the events)"
        if not light:
            self.config["format"] = "window 8, wide 8, partSize 32"


WORKLOADS = {SpmmProducts.name: SpmmProducts, GatReddit.name: GatReddit,
             GatRedditTF32.name: GatRedditTF32,
             GatArxivTrain.name: GatArxivTrain, SpmmProductsBF16.name: SpmmProductsBF16,
             SpmmProductsFP8.name: SpmmProductsFP8, SpmmGcn16k.name: SpmmGcn16k,
             ConvertProducts.name: ConvertProducts}
DEFAULT_WORKLOAD = SpmmProducts.name


# ---------------------------------------------------------------------------
def _env_rank():
    from att_gb300 import replicas
    return replicas.env_rank()


def cpu_baseline(wl, budget_s=12.0):
    """Time the oracle (torch.sparse CSR SpMM, fp32, all host threads) on a
    bounded row sample; returns the cpu_baseline dict."""
    import torch
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    rows = wl.n if wl.n <= 100_000 else max(8, wl.n // 64)
    if isinstance(wl, GatArxivTrain):
        return cpu_baseline_train(wl, threads, budget_s)
    if isinstance(wl, ConvertProducts):
        sec, _ = wl.cpu_port()
        return {"value": wl.bytes_alg / sec / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                "sample": "the whole graph through oracle/block_oracle.c (the C restatement of "
                          "gcn/Block_gcn/example.cpp:48-200), one host core, one run",
                "ms_per_sample": sec * 1e3}
    if isinstance(wl, GatReddit):
        rp, col, Xp, rows, b = wl.cpu_sample(rows)
        run = lambda: orc.gat_dot_layer_cpu_fp32(rp, col, Xp)  # noqa: E731
        what = "GAT layer (dot logits, LeakyReLU, softmax, aggregation) in torch fp32"
        F = Xp.shape[1]
    else:
        rp, col, vals, X, rows, b = wl.cpu_sample(rows)
        A = orc.csr_fp32(rp, col, vals, X.shape[0])
        run = lambda: orc.spmm_cpu_fp32(A, X)  # noqa: E731
        what = "torch.sparse CSR fp32 SpMM"
        F = X.shape[1]
    t0 = time.perf_counter()
    run()
    one = time.perf_counter() - t0
    reps = max(3, min(50, int(budget_s / max(one, 1e-3))))
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        run()
        ts.append(time.perf_counter() - t0)
    ts.sort()
    med = ts[len(ts) // 2]
    return {"value": b / med / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": "first %d rows of the same graph (%d edges), %s, F=%d, median of %d runs"
                      % (rows, int(col.shape[0]), what, F, reps),
            "ms_per_sample": med * 1e3}


def cpu_baseline_train(wl, threads, budget_s):
    """2-layer GAT training step in torch fp32 on the host cores (the oracle's
    differentiable restatement of the layer) on the whole graph; one or two
    steps (tens of seconds on a many-core host)."""
    import torch
    from oracle import oracle as orc
    k = wl.n
    srp = wl.rowptr.cpu().long()
    c = wl.colidx.cpu().long()
    X = wl.X.float().cpu()
    y = wl.y.cpu()
    H, Fh, C = wl.HEADS, wl.HID, wl.CLASSES
    g = torch.Generator().manual_seed(0)
    W1 = (torch.randn(wl.F_IN, H * Fh, generator=g) * 0.1).requires_grad_(True)
    a01 = (torch.randn(H, Fh, generator=g) * 0.1).requires_grad_(True)
    a11 = (torch.randn(H, Fh, generator=g) * 0.1).requires_grad_(True)
    W2 = (torch.randn(H * Fh, C, generator=g) * 0.1).requires_grad_(True)
    a02 = (torch.randn(1, C, generator=g) * 0.1).requires_grad_(True)
    a12 = (torch.randn(1, C, generator=g) * 0.1).requires_grad_(True)
    params = [W1, a01, a11, W2, a02, a12]
    opt = torch.optim.Adam(params, lr=1e-2, weight_decay=5e-4)

    def step():
        h = orc.gat_add_layer_torch(srp, c, X @ W1, a01, a11)
        h = torch.nn.functional.elu(h)
        o = orc.gat_add_layer_torch(srp, c, h @ W2, a02, a12)
        loss = torch.nn.functional.nll_loss(torch.log_softmax(o, 1), y)
        opt.zero_grad()
        loss.backward()
        opt.step()

    t0 = time.perf_counter()
    step()
    one = time.perf_counter() - t0
    ts = [one]
    if one * 2 < budget_s:
        t0 = time.perf_counter()
        step()
        ts.append(time.perf_counter() - t0)
    med = min(ts)
    return {"value": med * 1e3, "unit": "ms", "cores": threads, "kind": "port",
            "sample": "2-layer GAT train step (torch fp32, oracle restatement) on the whole "
                      "graph (%d nodes, %d edges); best of %d" % (k, int(c.numel()), len(ts)),
            "ms_per_sample": med * 1e3}


def run_reference(args):
    rank, local, world = _env_rank()
    if rank != 0:
        return 0
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t_setup = time.time()
    wl = WORKLOADS[args.workload](dev, scale=args.scale, light=True)
    base = cpu_baseline(wl, budget_s=max(3.0, 20.0 / max(1, args.steps + args.warmup)))
    line = {"metric": METRIC, "impl": "reference", "value": base["value"], "unit": wl.unit,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": base["ms_per_sample"],
            "higher_is_better": getattr(wl, "higher_is_better", True), "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(wl.config, note="reference CPU path restated by the oracle "
                                           "(no CPU SpMM ships in the reference)"),
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": base["value"], "unit": wl.unit, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "setup_s": time.time() - t_setup}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# serving workload (continuous batching vs one graph per call)
# ---------------------------------------------------------------------------
SERVE = "serve_gcn_fp16"
SERVE_RATE, SERVE_SEED, SERVE_POOL = 200.0, 4, 32


def _serve_pool_and_model(scale):
    from att_gb300 import serving
    pool = serving.make_graph_pool(SERVE_POOL, SERVE_SEED, n_min=max(8, int(1000 * scale)),
                                   n_max=max(16, int(500_000 * scale)))
    return pool, serving.GCN2(seed=SERVE_SEED)


def _tune_serving_groups(pool, model):
    """Parts per work group of the batched SpMM, picked by the autotuner on
    the pool's graphs (formats resident, layer-1 features)."""
    import torch
    from att_gb300 import autotune, serving
    s = torch.cuda.current_stream()
    reqs = [serving.Request(i, 0.0, rp, col, X, n, nnz) for i, (rp, col, X, n, nnz) in enumerate(pool)]
    for r in reqs:
        serving.prepare(r, model, s, with_groups=False)
    torch.cuda.synchronize()
    G, table = autotune.tune_group_parts(reqs)
    for r in reqs:
        r.dev = {}
    torch.cuda.synchronize()
    return G, table


def _batched_roofline(pool, model, steps, group_parts):
    """Kernel-only timing of one batched launch over every pool graph (their
    formats resident), against the same graphs as one att_spmm call each."""
    import torch
    from att_gb300 import ops, serving
    s = torch.cuda.current_stream()
    reqs = [serving.Request(i, 0.0, rp, col, X, n, nnz) for i, (rp, col, X, n, nnz) in enumerate(pool)]
    for r in reqs:
        serving.prepare(r, model, s, group_parts=group_parts)
    torch.cuda.synchronize()
    jobs = [serving.Job(r.dev["fmt"], r.dev["groups"], r.dev["partial"], r.dev["X"], r.dev["Y"], r.n)
            for r in reqs]
    b_alg = 0
    for r in reqs:
        f = r.dev["fmt"]
        U = int((f.rowptr[1::2] - f.rowptr[0:-1:2]).sum().item())
        F = model.hidden
        b_alg += 4 * (r.n + 1) + r.nnz * (4 + 2) + U * F * 2 + r.n * F * 4
    b = serving.BatchedSpmm(len(jobs), use_graph=True)
    for _ in range(3):
        b.run(jobs)
    torch.cuda.synchronize()
    b.check()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(s)
        b.run(jobs)
        ev[k][1].record(s)
    torch.cuda.synchronize()
    batched_ms = sum(a.elapsed_time(c) for a, c in ev) / steps
    for _ in range(3):
        for r in reqs:
            ops.spmm_format(r.dev["fmt"], r.dev["X"], r.n, out=r.dev["Y"])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(steps):
        for r in reqs:
            ops.spmm_format(r.dev["fmt"], r.dev["X"], r.n, out=r.dev["Y"])
    e1.record(s)
    torch.cuda.synchronize()
    per_graph_ms = e0.elapsed_time(e1) / steps
    nodes = sum(r.n for r in reqs)
    edges = sum(r.nnz for r in reqs)
    for r in reqs:
        r.dev = {}
    return {"batched_ms": batched_ms, "per_graph_calls_ms": per_graph_ms, "bytes": b_alg,
            "graphs": len(reqs), "nodes": nodes, "edges": edges}


def _cpu_serve_baseline(pool, model, budget_s=12.0):
    """2-layer GCN per request in torch fp32 on all host cores (torch.sparse
    CSR, the oracle's restatement of the reference's CPU path), over pool
    graphs in order until the time budget is spent; mean ms per request."""
    import torch
    import numpy as np
    from oracle import oracle as orc
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    W1, W2 = model.W1.float().cpu(), model.W2.float().cpu()
    ts, nodes, edges = [], 0, 0
    t_all = time.perf_counter()
    for rp, col, X, n, nnz in pool:
        if time.perf_counter() - t_all > budget_s:
            break
        t0 = time.perf_counter()
        rpl = rp.long()
        d = (rpl[1:] - rpl[:-1]).float().rsqrt()
        ridx = torch.repeat_interleave(torch.arange(n), rpl[1:] - rpl[:-1])
        vals = (d[ridx] * d[col.long()]).half().float()
        A = orc.csr_fp32(rp.numpy(), col.numpy(), vals.numpy(), n)
        H = torch.relu(orc.spmm_cpu_fp32(A, X.float() @ W1))
        orc.spmm_cpu_fp32(A, H @ W2)
        ts.append(time.perf_counter() - t0)
        nodes += n
        edges += nnz
    ms = 1e3 * sum(ts) / len(ts)
    return {"value": ms, "unit": "ms", "cores": threads, "kind": "port",
            "sample": "%d pool graphs (%d nodes, %d edges) served one by one: 2-layer GCN "
                      "(hidden 128) with torch.sparse CSR fp32; mean ms per request"
                      % (len(ts), nodes, edges)}


def run_serving(args):
    import numpy as np
    import torch
    from att_gb300 import builder, serving, _lib
    rank, local, world = _env_rank()
    torch.cuda.set_device(local)
    if rank == 0:
        builder.build()
    _lib.load()
    t_setup = time.time()
    pool, model = _serve_pool_and_model(args.scale)
    count = max(args.steps, 20)
    group_parts, group_ms = _tune_serving_groups(pool, model)
    reqs = serving.make_requests(pool, SERVE_RATE, count, SERVE_SEED)
    srv = serving.Server(model, budget=120e9, max_active=64, workers=2, keep_outputs=False,
                         group_parts=group_parts)
    # warm-up to the steady state of a running server: a real-time trace of
    # another seed through both paths (the caching device and pinned-host
    # allocators then hold blocks for the concurrency the rate brings)
    n_warm = max(100, min(count, 400))
    for _ in range(max(1, args.warmup // 3)):
        srv.run(serving.make_requests(pool, SERVE_RATE, n_warm, SERVE_SEED + 100), realtime=True)
        serving.serve_one_by_one(serving.make_requests(pool, SERVE_RATE, n_warm // 2,
                                                       SERVE_SEED + 101),
                                 model, realtime=True, keep_outputs=False)
    torch.cuda.synchronize()
    ticks0 = len(srv.jobs_per_tick)

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    srv.run(reqs, realtime=True)
    wall = time.perf_counter() - t0
    clocks = sampler.stop()
    st = serving.latency_stats(reqs)
    tick_jobs = srv.jobs_per_tick[ticks0:]
    plain = [serving.Request(r.rid, r.arrival, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs]
    serving.serve_one_by_one(plain, model, realtime=True, keep_outputs=False)
    pst = serving.latency_stats(plain)
    # saturation throughput: the same trace with every request arrived at t = 0
    cap = {}
    for name, fn in (("continuous_batching", lambda q: srv.run(q, realtime=False)),
                     ("one_graph_per_call",
                      lambda q: serving.serve_one_by_one(q, model, realtime=False, keep_outputs=False))):
        q = [serving.Request(r.rid, 0.0, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs[:300]]
        c0 = time.perf_counter()
        fn(q)
        cap[name] = len(q) / (time.perf_counter() - c0)
    # results agree between the two paths: full outputs of 48 requests
    # (untimed; the batched path is deterministic, the one-by-one path adds
    # split windows with atomics, so they differ by fp32 rounding only)
    vr = [serving.Request(r.rid, 0.0, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs[:48]]
    vp = [serving.Request(r.rid, 0.0, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs[:48]]
    serving.Server(model, budget=120e9, max_active=64, workers=2,
                   group_parts=group_parts).run(vr, realtime=False)
    serving.serve_one_by_one(vp, model, realtime=False)
    agree = max(float((a.out - b.out).abs().max() / b.out.abs().max().clamp_min(1e-30))
                for a, b in zip(vr, vp))
    del vr, vp
    roof_raw = _batched_roofline(pool, model, max(5, min(args.steps, 20)), group_parts)
    peak, peak_kind = peaks()
    achieved = roof_raw["bytes"] / (roof_raw["batched_ms"] * 1e-3) / 1e9
    base = None if args.no_cpu_baseline else _cpu_serve_baseline(pool, model)
    h2d = float(np.mean([r.rowptr.numel() * 4 + r.col.numel() * 4 + r.X.numel() * 2 for r in reqs]))
    d2h = float(np.mean([r.n * model.F_out * 4 for r in reqs]))
    n_ticks = len(tick_jobs)
    line = {"metric": METRIC, "value": st["p99_ms"], "unit": "ms", "n_gpus": world,
            "steps": count, "warmup": args.warmup, "ms_per_step": st["mean_ms"],
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f16",
            "data": "synthetic",
            "config": {"workload": SERVE, "requests": count, "rate_per_s": SERVE_RATE,
                       "seed": SERVE_SEED, "graph_pool": len(pool),
                       "nodes": "log-uniform [%d, %d]" % (min(p[3] for p in pool), max(p[3] for p in pool)),
                       "mean_degree": "uniform [5, 50]", "model": "2-layer GCN, hidden 128, fp16",
                       "hbm_budget_bytes": 120e9, "max_active": 64, "workers": 2,
                       "step": "one request (arrival -> result in pinned host memory)",
                       "l2": "graphs and features change every request; no flush"},
            "serve": {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
                      "graphs_per_s": st["graphs_per_s"], "wall_s": wall, "ticks": n_ticks,
                      "jobs_per_tick_mean": float(np.mean(tick_jobs)) if tick_jobs else 0.0,
                      "jobs_per_tick_max": int(max(tick_jobs)) if tick_jobs else 0,
                      "rejected": st["rejected"]},
            "plain_one_graph_per_call": {"p50_ms": pst["p50_ms"], "p99_ms": pst["p99_ms"],
                                         "mean_ms": pst["mean_ms"],
                                         "graphs_per_s": pst["graphs_per_s"]},
            "saturation_graphs_per_s": cap,
            "autotune": {"group_parts": group_parts,
                         "batched_launch_ms_by_group_parts": {str(k): v for k, v in group_ms.items()}},
            "max_rel_diff_vs_plain_48_requests": agree,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_kind": peak_kind,
                         "kernel": "att_spmm_batched over %d resident graphs (%d nodes, %d edges)"
                                   % (roof_raw["graphs"], roof_raw["nodes"], roof_raw["edges"]),
                         "bytes_per_launch": roof_raw["bytes"],
                         "launch_ms": roof_raw["batched_ms"],
                         "same_graphs_one_att_spmm_call_each_ms": roof_raw["per_graph_calls_ms"]},
            "cpu_baseline": base and {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": st["p99_ms"], "unit": "ms", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "att_gb300.serving.Server.run",
                    "note": "every latency is end to end: pinned host CSR + features in, "
                            "fp32 result in pinned host memory out"},
            "gpu_launches": serving.PREPARE_LAUNCHES * count + serving.TICK_LAUNCHES * n_ticks,
            "clocks": clocks, "setup_s": time.time() - t_setup - wall}
    print(json.dumps(line))
    return 0


def run_reference_serving(args):
    rank, local, world = _env_rank()
    if rank != 0:
        return 0
    import torch
    from att_gb300 import serving

    class _M:  # the same weights as the GPU model, generated on the host
        pass
    g = torch.Generator().manual_seed(SERVE_SEED)
    m = _M()
    import math
    m.W1 = ((torch.rand(128, 128, generator=g) * 2 - 1) * math.sqrt(6.0 / 256)).half()
    m.W2 = ((torch.rand(128, 128, generator=g) * 2 - 1) * math.sqrt(6.0 / 256)).half()
    sizes = serving.graph_sizes(SERVE_POOL, SERVE_SEED, n_min=max(8, int(1000 * args.scale)),
                                n_max=max(16, int(500_000 * args.scale)))
    from att_gb300 import graphs
    pool = []
    for i, (n, deg) in enumerate(sizes[:8]):
        rp, col = graphs.chung_lu(n, deg, 2.1, seed=SERVE_SEED * 1000 + i, device="cpu")
        X = (torch.rand(n, 128, generator=g) * 2 - 1).half()
        pool.append((rp, col, X, n, int(col.numel())))
    base = _cpu_serve_baseline(pool, m, budget_s=max(3.0, 20.0 / max(1, args.warmup)))
    line = {"metric": METRIC, "impl": "reference", "value": base["value"], "unit": "ms",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": base["value"], "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": SERVE, "note": "reference CPU path (torch.sparse CSR "
                       "2-layer GCN, one graph per call) restated by the oracle"},
            "cpu_baseline": {k: base[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": base["value"], "unit": "ms", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def _git_head():
    try:
        return subprocess.run(["git", "rev-parse", "--short=12", "HEAD"], cwd=ROOT,
                              stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                              text=True).stdout.strip() or None
    except Exception:
        return None


def _events(torch, stream, n):
    return [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(n)]


def _time_each(torch, fn, steps, stream, flush=None):
    """Per-call device milliseconds of `fn` (CUDA events on `stream`); with
    `flush`, that buffer is rewritten (L2 flushed) before every call, outside
    the events."""
    ev = _events(torch, stream, steps)
    for a, b in ev:
        if flush is not None:
            flush.zero_()
        a.record(stream)
        fn()
        b.record(stream)
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def roofline(wl, avg_launch_ms, shape):
    """The dominant kernel's roofline object.

    `frac` is DRAM-based when an ncu capture of the same kernel and launch
    shape on the same workload exists (MEASURED_TRAFFIC): measured DRAM bytes
    per launch / the CUDA-event launch time / the measured copy peak.
    Otherwise it falls back to the algorithmic bytes and says so (those can
    exceed the peak: they count gathers of hub rows that L2 serves).  Both
    the algorithmic fraction and the compulsory fraction (format + each X row
    once + output, a lower bound on DRAM traffic) are always given."""
    peak, peak_kind = peaks()
    t = avg_launch_ms * 1e-3
    kbytes = getattr(wl, "bytes_fused", wl.bytes_alg)
    alg = kbytes / t / 1e9
    mt = MEASURED_TRAFFIC.get((wl.name, 1.0 if getattr(wl, "scale", 1.0) == 1.0 else wl.scale))
    if mt is not None and mt.get("shape") is not None and shape is not None \
            and tuple(mt["shape"]) != tuple(shape):
        mt = None  # captured on another launch shape: its bytes are not this kernel's
    comp = getattr(wl, "bytes_compulsory", None)
    roof = {"bound": "hbm", "peak": peak, "unit": "GB/s", "peak_kind": peak_kind,
            "kernel": getattr(wl, "kernel_name", "att_spmm (k_zero_uncovered + k_spmm16)"),
            "launch_ms": avg_launch_ms, "launch_shape": list(shape) if shape else None,
            "alg_bytes": kbytes, "alg_achieved": alg, "alg_frac": alg / peak,
            "compulsory_bytes": comp,
            "compulsory_frac": (comp / t / 1e9 / peak) if comp else None}
    if mt is not None:
        dram = mt["bytes"] / t / 1e9
        roof.update({"achieved": dram, "frac": dram / peak, "traffic": mt["bytes"],
                     "basis": "DRAM bytes of one launch of this kernel and shape (ncu) / "
                              "CUDA-event launch time",
                     "traffic_source": dict(mt, method="ncu dram__bytes_read.sum + "
                                                       "dram__bytes_write.sum, one launch")})
    else:
        roof.update({"achieved": alg, "frac": alg / peak, "traffic": None,
                     "basis": "algorithmic bytes / CUDA-event launch time (no DRAM capture "
                              "of this kernel and shape; can exceed 1 where L2 serves re-reads)"})
    return roof


def measure(wl, torch, stream, steps, warmup, world=1, dist=None, clocks=False, e2e=True,
            plain=True):
    """Warm up, time `steps` steps (bracketed by barrier + synchronize), time
    the dominant kernel per launch, the plain comparison path and the end to
    end call; returns a dict of the numbers."""
    from att_gb300 import replicas
    for _ in range(warmup):
        wl.step()
    torch.cuda.synchronize()
    # workloads whose inputs fit in L2 flush it before every timed step,
    # outside that step's events (a write of a buffer larger than L2)
    flush = (torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
             if getattr(wl, "l2_flush", False) else None)
    sampler = None
    if clocks:
        sampler = ClockSampler(torch.cuda.current_device())
        sampler.start()
        time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    t_all0 = torch.cuda.Event(enable_timing=True)
    t_all1 = torch.cuda.Event(enable_timing=True)
    t_all0.record(stream)
    # each timed step sits in an NVTX range "bench_step", so a profiler can
    # capture exactly these launches (--nvtx --nvtx-include "bench_step/")
    def step():
        torch.cuda.nvtx.range_push("bench_step")
        wl.step()
        torch.cuda.nvtx.range_pop()
    if flush is not None:
        per_step = _time_each(torch, step, steps, stream, flush)
    else:
        for _ in range(steps):
            step()
    t_all1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    total_ms = sum(per_step) if flush is not None else t_all0.elapsed_time(t_all1)
    # dominant kernel alone, per launch, for the roofline
    kernel_step = getattr(wl, "kernel_step", wl.step)
    if hasattr(wl, "prepare_kernel"):
        wl.prepare_kernel()
    torch.cuda.synchronize()
    per_launch = sorted(_time_each(torch, kernel_step, steps, stream, flush))
    clk = sampler.stop() if sampler else None
    total_ms = replicas.max_over_ranks([total_ms], device="cuda")[0] if world > 1 else total_ms
    rec = {"ms_per_step": total_ms / steps, "per_launch": per_launch,
           "avg_launch_ms": sum(per_launch) / len(per_launch), "clocks": clk}
    # the plain comparison path on the same data
    rec["plain_ms"] = None
    if plain and getattr(wl, "plain_step", None) and getattr(wl, "plain_available", lambda: True)():
        for _ in range(2):
            wl.plain_step()
        torch.cuda.synchronize()
        n_plain = max(3, min(steps, 10))
        pt = _time_each(torch, wl.plain_step, n_plain, stream, flush)
        rec["plain_ms"] = sum(pt) / len(pt)
    # end to end through the reference-facing call with host buffers
    if e2e:
        wl.e2e_setup()
        for _ in range(10):
            wl.e2e_step()
        torch.cuda.synchronize()
        # Timed in 5 blocks of up to 10 steps.  On the GB300 machine the
        # device-to-host link stalls every half second or so of sustained
        # traffic: three consecutive 1.25 GB result copies then take 40-55 ms
        # instead of 6.9 ms, while the kernels and the host's enqueueing keep
        # their pace.  The median block is the steady state; the mean over all
        # blocks, stalls included, is reported beside it.
        per_block = max(1, min(steps, 10))
        blocks = []
        for _ in range(5):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if hasattr(wl, "e2e_begin"):
                wl.e2e_begin()
            for _ in range(per_block):
                wl.e2e_step()
            if hasattr(wl, "e2e_finish"):
                wl.e2e_finish()
            e1.record(stream)
            torch.cuda.synchronize()
            blocks.append(e0.elapsed_time(e1) / per_block)
        e2e_ms = sorted(blocks)[len(blocks) // 2]
        mean_ms = sum(blocks) / len(blocks)
        if world > 1:
            e2e_ms, mean_ms = replicas.max_over_ranks([e2e_ms, mean_ms], device="cuda")
        rec["e2e_ms"] = e2e_ms
        rec["e2e_mean_ms"] = mean_ms
        rec["e2e_blocks_ms"] = blocks
        rec["e2e_steps"] = 5 * per_block
    return rec


def _free(torch):
    import gc
    gc.collect()
    torch.cuda.empty_cache()


def _spmm_form(cls, torch, stream, steps, warmup):
    wl = cls("cuda")
    tuned = wl.autotune()
    wl.check()
    rec = measure(wl, torch, stream, steps, warmup, e2e=False)
    out = {"ms": rec["ms_per_step"], "kernel_launch_ms": rec["avg_launch_ms"],
           "gbs_own_bytes": wl.bytes_alg / (rec["ms_per_step"] * 1e-3) / 1e9,
           "gbs_fp16_equivalent": wl.bytes_fp16 / (rec["ms_per_step"] * 1e-3) / 1e9,
           "err_vs_fp64": wl.err_vs_fp64,
           "plain_fp16_dropin_ms": rec["plain_ms"],
           "plain": wl.plain_kind if rec["plain_ms"] is not None else None,
           "speedup_vs_plain": (rec["plain_ms"] / rec["ms_per_step"]) if rec["plain_ms"] else None,
           "launch_shape": tuned["choice"] if tuned else None}
    if hasattr(wl, "err_vs_fp64_own_inputs"):
        out["err_vs_fp64_of_dequantized_inputs"] = wl.err_vs_fp64_own_inputs
    del wl
    _free(torch)
    return out


def _gat_form(cls, torch, stream, steps, warmup):
    wl = cls("cuda")
    wl.check()
    rec = measure(wl, torch, stream, steps, warmup, e2e=False)
    out = {"ms": rec["ms_per_step"], "fused_launch_ms": rec["avg_launch_ms"],
           "alg_gbs": wl.bytes_alg / (rec["ms_per_step"] * 1e-3) / 1e9,
           "err_vs_fp64": wl.err_vs_fp64,
           "plain_chain_ms": rec["plain_ms"],
           "plain": "the reference's chain of separate ops (SDDMM, edge softmax, SpMM of edge "
                    "values; end2end_ori/gat_final/mgat_csr/mgat_conv.py:173-198) on this "
                    "package's drop-in kernels (the reference's GAT kernels ship no source)",
           "speedup_vs_plain": (rec["plain_ms"] / rec["ms_per_step"]) if rec["plain_ms"] else None}
    if hasattr(wl, "chain_err_vs_fp64"):
        out["plain_chain_err_vs_fp64"] = wl.chain_err_vs_fp64
    del wl
    _free(torch)
    return out


def _train_form(torch, stream, steps, warmup):
    wl = GatArxivTrain("cuda")
    grad_diff = wl.check()
    rec = measure(wl, torch, stream, steps, warmup, e2e=False)
    out = {"ms": rec["ms_per_step"], "plain_chain_ms": rec["plain_ms"],
           "plain": "the same 2-layer GAT on the reference's chain of separate ops (fp16 "
                    "drop-ins, torch autograd glue), same GPU",
           "speedup_vs_plain": (rec["plain_ms"] / rec["ms_per_step"]) if rec["plain_ms"] else None,
           "layer1_weight_grad_rel_diff_fused_vs_chain": grad_diff}
    del wl
    _free(torch)
    return out


def _serve_form(torch, requests=600, seeds=(4, 5, 6)):
    """p50 / p99 of the continuous-batching server and of one graph per call
    on Poisson traces of `requests` requests per seed (200 req/s)."""
    from att_gb300 import serving
    pool, model = _serve_pool_and_model(1.0)
    srv = serving.Server(model, budget=120e9, max_active=64, workers=2, keep_outputs=False)
    srv.run(serving.make_requests(pool, SERVE_RATE, 100, SERVE_SEED + 100), realtime=True)
    serving.serve_one_by_one(serving.make_requests(pool, SERVE_RATE, 50, SERVE_SEED + 101),
                             model, realtime=True, keep_outputs=False)
    out = {"requests_per_seed": requests, "rate_per_s": SERVE_RATE, "seeds": list(seeds),
           "p50_ms": [], "p99_ms": [], "plain_p50_ms": [], "plain_p99_ms": []}
    for sd in seeds:
        reqs = serving.make_requests(pool, SERVE_RATE, requests, sd)
        srv.run(reqs, realtime=True)
        st = serving.latency_stats(reqs)
        plain = [serving.Request(r.rid, r.arrival, r.rowptr, r.col, r.X, r.n, r.nnz) for r in reqs]
        serving.serve_one_by_one(plain, model, realtime=True, keep_outputs=False)
        pst = serving.latency_stats(plain)
        out["p50_ms"].append(st["p50_ms"])
        out["p99_ms"].append(st["p99_ms"])
        out["plain_p50_ms"].append(pst["p50_ms"])
        out["plain_p99_ms"].append(pst["p99_ms"])
    del pool, srv
    _free(torch)
    return out


def run_forms(torch, stream, steps, warmup, skip=()):
    """The chosen forms (bf16 / fp8 SpMM, fused GAT layers, the train step,
    the serving loop) beside their plain paths, each measured
    on its own workload after the headline one (a few seconds each)."""
    forms = {}
    jobs = [("spmm_products_bf16", lambda: _spmm_form(SpmmProductsBF16, torch, stream, steps, warmup)),
            ("spmm_products_fp8", lambda: _spmm_form(SpmmProductsFP8, torch, stream, steps, warmup)),
            ("gat_reddit_fp16", lambda: _gat_form(GatReddit, torch, stream, steps, warmup)),
            ("gat_reddit_tf32", lambda: _gat_form(GatRedditTF32, torch, stream, steps, warmup)),
            ("gat_arxiv_train_bf16", lambda: _train_form(torch, stream, steps, warmup)),
            ("convert_products_fp16", lambda: _convert_form(torch, stream, steps, warmup)),
            ("spmm_gcn16k_fp16", lambda: _spmm_form(SpmmGcn16k, torch, stream, steps, warmup)),
            ("serve_gcn_fp16", lambda: _serve_form(torch))]
    for name, fn in jobs:
        if name in skip:
            continue
        t0 = time.time()
        try:
            forms[name] = fn()
        except Exception as exc:  # one form failing must not hide the others
            forms[name] = {"error": "%s: %s" % (type(exc).__name__, exc)}
        forms[name]["wall_s"] = time.time() - t0
    return forms


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS) + [SERVE])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the other forms (measured after the headline workload)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="node-count scale of the workload (1.0 = the named config)")
    ap.add_argument("--shape", default=None,
                    help="pin the SpMM launch shape instead of autotuning it, e.g. spmm,64,3 "
                         "(for profiler captures of a known kernel)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload == SERVE:
        return run_reference_serving(args) if args.impl == "reference" else run_serving(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist
    rank, local, world = _env_rank()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from att_gb300 import builder
    if rank == 0:
        builder.build()
    if world > 1:
        dist.barrier()
    from att_gb300 import _lib
    _lib.load()

    wl = WORKLOADS[args.workload]("cuda", scale=args.scale)
    wl.scale = args.scale
    pinned = None
    if args.shape:
        pinned = tuple(int(v) if v.isdigit() else v for v in args.shape.split(","))
    tuned = wl.autotune(pinned) if hasattr(wl, "autotune") else None
    check_err = wl.check()
    stream = torch.cuda.current_stream()
    rec = measure(wl, torch, stream, args.steps, args.warmup, world=world, dist=dist,
                  clocks=True)
    ms_per_step = rec["ms_per_step"]
    is_time = wl.unit == "ms"
    from att_gb300 import replicas
    value = (ms_per_step if is_time
             else replicas.aggregate_rate(wl.bytes_alg, ms_per_step, world) / 1e9)
    e2e_ms = rec["e2e_ms"]
    shape = tuple(tuned["choice"]) if tuned and tuned.get("choice") else None
    line = None
    if rank == 0:
        base = None
        if not args.no_cpu_baseline:
            base = cpu_baseline(wl)
        per_launch = rec["per_launch"]
        line = {"metric": METRIC, "value": value, "unit": wl.unit, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "higher_is_better": not is_time, "scaling": "weak", "vs_baseline": None,
                "dtype": ("bf16" if "bf16" in wl.name else "e4m3" if "fp8" in wl.name
                          else "tf32" if "tf32" in wl.name else "f16"),
                "data": "synthetic",
                "config": dict(wl.config),
                "workload_ms_per_step": ms_per_step,
                "roofline": roofline(wl, rec["avg_launch_ms"], shape),
                "cpu_baseline": ({k: base[k] for k in ("value", "unit", "cores", "kind", "sample")}
                                 if base else None),
                "e2e": {"value": e2e_ms if is_time else world * wl.bytes_alg / (e2e_ms * 1e-3) / 1e9,
                        "unit": wl.unit,
                        "h2d_bytes_per_step": wl.h2d, "d2h_bytes_per_step": wl.d2h,
                        "ms_per_step": e2e_ms, "api": wl.e2e_api,
                        "timing": "median of 5 blocks of %d steps (CUDA events)" % (rec["e2e_steps"] // 5),
                        "mean_ms_per_step_all_blocks": rec["e2e_mean_ms"],
                        "blocks_ms_per_step": rec["e2e_blocks_ms"]},
                "gpu_launches": wl.launches_per_step * args.steps,
                "clocks": rec["clocks"],
                "gflops": world * wl.flops / (ms_per_step * 1e-3) / 1e9,
                "plain_dropin_ms_per_step": rec["plain_ms"],
                "plain_dropin": getattr(wl, "plain_kind", None) if rec["plain_ms"] else None,
                "speedup_vs_plain_dropin": (rec["plain_ms"] / ms_per_step) if rec["plain_ms"] else None,
                "autotune": tuned,
                "fp16_equivalent_gbs": (world * wl.bytes_fp16 / (ms_per_step * 1e-3) / 1e9
                                        if hasattr(wl, "bytes_fp16") else None),
                "check_rel_err": check_err,
                "err_vs_fp64": getattr(wl, "err_vs_fp64", None),
                "plain_dropin_err_vs_fp64": getattr(wl, "plain_err_vs_fp64", None),
                "launch_ms_p50": per_launch[len(per_launch) // 2],
                "commit": _git_head()}
        if hasattr(wl, "err_vs_fp64_own_inputs"):
            line["err_vs_fp64_of_dequantized_inputs"] = wl.err_vs_fp64_own_inputs
    if rank == 0 and world == 1 and not args.no_forms:
        del wl
        _free(torch)
        line["forms"] = run_forms(torch, stream, min(args.steps, 10), 3, skip=(args.workload,))
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
