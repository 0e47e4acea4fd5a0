"""Torch-level entry points over the C ABI.

Tensors live on the current CUDA device; every kernel launches on
``torch.cuda.current_stream()``.  Outputs and workspaces are allocated with
torch (the caching allocator) and handed to the C ABI as raw pointers.
"""
import threading
from dataclasses import dataclass, field
from typing import Optional

import torch

from . import _lib

_DT = {torch.float32: _lib.F32, torch.float16: _lib.F16, torch.bfloat16: _lib.BF16,
       torch.int32: _lib.I32}
if hasattr(torch, "float8_e4m3fn"):
    _DT[torch.float8_e4m3fn] = _lib.F8E4M3


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("att_gb300 runs only on a CUDA device (sm_103a); there is no CPU path")
    _lib.load()


def _p(t):
    return None if t is None else t.data_ptr()


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _dev(t, dtype=None):
    """Contiguous CUDA copy (no copy if already so)."""
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if dtype is not None and t.dtype != dtype:
        t = t.to(dtype)
    if t.device.type != "cuda":
        t = t.to("cuda", non_blocking=False)
    return t.contiguous()


@dataclass
class BlockFormat:
    """Row-window block-condensed format resident on the GPU."""
    rowptr: torch.Tensor            # int32 [2*parts+1]
    col: torch.Tensor               # int32 [n_condensed]
    window_of_part: torch.Tensor    # int32 [parts]
    atomic: torch.Tensor            # int32 [parts]
    window: int
    wide: int
    part: int
    n_rows: int
    n_cols: int
    nnz: int
    val: Optional[torch.Tensor] = None       # [n_condensed*window]
    map: Optional[torch.Tensor] = None       # int32 slot -> CSR edge id
    map_t: Optional[torch.Tensor] = None     # int32 slot -> mirrored edge id
    edge_slot: Optional[torch.Tensor] = None # int32 CSR edge -> slot
    extra: dict = field(default_factory=dict)

    @property
    def n_parts(self):
        return int(self.window_of_part.shape[0])

    @property
    def n_condensed(self):
        return int(self.col.shape[0])

    def cpu_tuple(self):
        return (self.rowptr.cpu(), self.col.cpu(), self.val.cpu(), self.window_of_part.cpu(),
                self.atomic.cpu())


def block_workspace_bytes(n_rows, nnz, n_cols, window):
    return int(_lib.lib().att_block_workspace_bytes(n_rows, nnz, n_cols, window))


def _conv_args(rowptr, col, deg, window, wide, part, emit_empty, val_dtype, want_val, n_cols):
    require_cuda()
    rowptr = _dev(rowptr, torch.int32)
    col = _dev(col, torch.int32)
    n_rows = int(rowptr.shape[0]) - 1
    nnz = int(col.shape[0])
    if n_rows < 0:
        raise ValueError("rowptr must have at least one entry")
    deg_t, deg_kind = None, _lib.NONE
    if deg is not None and want_val:
        deg_t = _dev(deg)
        if deg_t.dtype not in (torch.float16, torch.float32):
            raise TypeError("degree must be float16 or float32, got %s" % deg_t.dtype)
        if deg_t.shape[0] < n_rows:
            raise ValueError("degree has %d entries for %d rows" % (deg_t.shape[0], n_rows))
        deg_kind = _DT[deg_t.dtype]
        if val_dtype is None:
            val_dtype = deg_t.dtype
    if n_cols is None:
        n_cols = int(deg_t.shape[0]) if deg_t is not None else n_rows
    return dict(rowptr=rowptr, col=col, n_rows=n_rows, nnz=nnz, n_cols=n_cols, window=window,
                wide=wide, part=part, emit_empty=int(bool(emit_empty)), deg=deg_t,
                deg_kind=deg_kind, val_dtype=val_dtype)


def _conv_fill(a, ws, ws_bytes, P, NC, want_map, want_trans, want_edge_slot, flags=None):
    """att_block_fill, or with ``flags`` (pinned int32 [4]) att_block_fill_async:
    no host synchronisation, the device-side checks copied to ``flags``."""
    dev = a["rowptr"].device
    W = a["window"]
    out_rowptr = torch.empty(2 * P + 1, dtype=torch.int32, device=dev)
    out_col = torch.empty(NC, dtype=torch.int32, device=dev)
    out_win = torch.empty(P, dtype=torch.int32, device=dev)
    out_atomic = torch.empty(P, dtype=torch.int32, device=dev)
    val = None
    if a["deg"] is not None:
        val = torch.empty(NC * W, dtype=a["val_dtype"], device=dev)
    mp = torch.empty(NC * W, dtype=torch.int32, device=dev) if want_map else None
    mpt = torch.empty(NC * W, dtype=torch.int32, device=dev) if want_trans else None
    es = torch.empty(a["nnz"], dtype=torch.int32, device=dev) if want_edge_slot else None
    vdt = _DT[a["val_dtype"]] if val is not None else _lib.NONE
    if flags is None:
        _lib.call("att_block_fill", _p(a["rowptr"]), _p(a["col"]), a["n_rows"], a["nnz"],
                  a["n_cols"], W, a["wide"], a["part"], a["emit_empty"], _p(a["deg"]),
                  a["deg_kind"], _p(ws), ws_bytes, _p(out_rowptr), _p(out_col), _p(val), vdt,
                  _p(mp), _p(mpt), _p(es), _p(out_win), _p(out_atomic), _stream())
    else:
        _lib.call("att_block_fill_async", _p(a["rowptr"]), _p(a["col"]), a["n_rows"], a["nnz"],
                  a["n_cols"], W, a["wide"], a["part"], a["emit_empty"], _p(a["deg"]),
                  a["deg_kind"], _p(ws), ws_bytes, P, NC, _p(out_rowptr), _p(out_col), _p(val),
                  vdt, _p(mp), _p(mpt), _p(es), _p(out_win), _p(out_atomic), _p(flags),
                  _stream())
    return BlockFormat(rowptr=out_rowptr, col=out_col, window_of_part=out_win, atomic=out_atomic,
                       window=W, wide=a["wide"], part=a["part"], n_rows=a["n_rows"],
                       n_cols=a["n_cols"], nnz=a["nnz"], val=val, map=mp, map_t=mpt,
                       edge_slot=es)


def block_convert(rowptr, col, deg=None, window=8, wide=8, part=32, emit_empty=False,
                  val_dtype=None, want_val=True, want_map=False, want_trans=False,
                  want_edge_slot=False, n_cols=None):
    """CSR -> block format on the GPU (bit-identical to the reference CPU
    conversion, gcn/Block_gcn/example.cpp:48-348).

    ``deg``: per-node degree factor (fp16 -> fp16 values as
    ``blockProcess_fp16_balance``; fp32 -> fp32 values as ``_tf32_balance``);
    None for a structure/map-only format (the GAT form).  Synchronises the
    current stream once (the plan's sizes).
    """
    a = _conv_args(rowptr, col, deg, window, wide, part, emit_empty, val_dtype, want_val, n_cols)
    ws_bytes = block_workspace_bytes(a["n_rows"], a["nnz"], a["n_cols"], window)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
    n_parts = _lib.ctypes.c_int64(0)
    n_cond = _lib.ctypes.c_int64(0)
    _lib.call("att_block_plan", _p(a["rowptr"]), _p(a["col"]), a["n_rows"], a["nnz"],
              a["n_cols"], window, wide, part, a["emit_empty"], _p(ws), ws_bytes,
              _lib.ctypes.byref(n_parts), _lib.ctypes.byref(n_cond), _stream())
    return _conv_fill(a, ws, ws_bytes, n_parts.value, n_cond.value, want_map, want_trans,
                      want_edge_slot)


@dataclass
class PendingConvert:
    """A conversion whose plan is enqueued (block_convert_async); `event`
    completes when the plan's summary has reached the host."""
    args: dict
    ws: torch.Tensor
    ws_bytes: int
    summary: torch.Tensor   # pinned int64 [3]
    event: torch.cuda.Event
    options: tuple

    def ready(self):
        return self.event.query()


def block_convert_async(rowptr, col, deg=None, window=8, wide=8, part=32, emit_empty=False,
                        val_dtype=None, want_val=True, want_map=False, want_trans=False,
                        want_edge_slot=False, n_cols=None):
    """Phase 1 of block_convert enqueued on the current stream without a
    host synchronisation (att_block_plan_async); finish with
    block_convert_finish once ``pending.ready()``."""
    a = _conv_args(rowptr, col, deg, window, wide, part, emit_empty, val_dtype, want_val, n_cols)
    ws_bytes = block_workspace_bytes(a["n_rows"], a["nnz"], a["n_cols"], window)
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device="cuda")
    summary = torch.zeros(3, dtype=torch.int64, pin_memory=True)
    _lib.call("att_block_plan_async", _p(a["rowptr"]), _p(a["col"]), a["n_rows"], a["nnz"],
              a["n_cols"], window, wide, part, a["emit_empty"], _p(ws), ws_bytes, _p(summary),
              _stream())
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream())
    return PendingConvert(a, ws, ws_bytes, summary, ev, (want_map, want_trans, want_edge_slot))


def block_convert_finish(pending, check_later=False):
    """Phase 2: validate the plan's summary (raises AttError for a malformed
    CSR) and enqueue the fill on the current stream (the plan's stream, or one
    ordered after it).  The fill's device-side checks are read back with a
    host synchronisation -- or, with ``check_later``, copied to pinned memory
    without one: the format then carries them (``fmt.extra["fill_flags"]``,
    with the workspace the fill reads) and ``block_fill_check(fmt)`` raises
    their error once the stream has passed the fill."""
    if not pending.event.query():
        raise RuntimeError("the plan has not completed: wait for pending.ready()")
    n_parts = _lib.ctypes.c_int64(0)
    n_cond = _lib.ctypes.c_int64(0)
    a = pending.args
    _lib.call("att_block_plan_result", _p(pending.summary), a["n_cols"], a["window"],
              _lib.ctypes.byref(n_parts), _lib.ctypes.byref(n_cond))
    flags = torch.zeros(4, dtype=torch.int32).pin_memory() if check_later else None
    fmt = _conv_fill(a, pending.ws, pending.ws_bytes, n_parts.value, n_cond.value,
                     *pending.options, flags=flags)
    if flags is not None:
        fmt.extra["fill_flags"] = flags
        fmt.extra["fill_workspace"] = pending.ws  # read by the fill until the stream passes it
    return fmt


def block_fill_check(fmt):
    """Raise the error of a fill enqueued with ``check_later`` (call once the
    stream has passed it)."""
    flags = fmt.extra.pop("fill_flags", None)
    if flags is not None:
        fmt.extra.pop("fill_workspace", None)
        _lib.call("att_block_fill_result", _p(flags), 1 if fmt.map_t is not None else 0)


_SHAPE_KNOBS = {"spmm": ("spmm_fc", "spmm_stages"), "fp8": ("spmm_fp8",),
                "tf32": ("spmm_tf32",)}
_ALL_KNOBS = ("spmm_fc", "spmm_stages", "spmm_fp8", "spmm_tf32")
_tls = threading.local()


def set_launch_shape(shape):
    """Make the calling thread's att_spmm launch shape `shape` (an autotuner
    candidate such as ("spmm", 64, 3); None = the process-wide defaults).  The
    thread's current shape is remembered, so repeating it costs no call into
    the library."""
    cur = getattr(_tls, "shape", None)
    if cur == shape:
        return
    for k in _ALL_KNOBS:
        _lib.call("att_set_thread_option", k.encode(), -1)
    if shape is not None:
        for k, v in zip(_SHAPE_KNOBS[shape[0]], shape[1:]):
            _lib.call("att_set_thread_option", k.encode(), int(v))
    _tls.shape = None if shape is None else tuple(shape)


def spmm(rowptr, col, val, window_of_part, atomic, X, m_out, window=8, wide=8, out=None,
         x_scale=None, err_flag=None, shape=None):
    """Y[m_out, F] (fp32) = A_blocks X on tensor cores.

    X: [n_x, F] fp16 / bf16 (with matching ``val``), fp32 (3xTF32), or
    float8_e4m3fn with ``x_scale`` fp32 [n_x] (values fp16).  F must be a
    multiple of 8 (16-bit) or 4 (fp32); callers pad otherwise.  ``shape``: a
    launch shape returned by ``autotune.tune_spmm`` (the process-wide
    defaults when None).
    """
    set_launch_shape(shape)
    require_cuda()
    if X.dim() != 2:
        raise ValueError("X must be 2-D [nodes, features]")
    if X.stride(1) != 1:
        X = X.contiguous()
    n_x, F = int(X.shape[0]), int(X.shape[1])
    ldx = int(X.stride(0)) if n_x > 1 else F
    if out is None:
        out = torch.empty((m_out, F), dtype=torch.float32, device=X.device)
    if out.dtype != torch.float32 or out.stride(1) != 1:
        raise ValueError("out must be fp32 with unit feature stride")
    ldy = int(out.stride(0)) if m_out > 1 else F
    n_parts = int(window_of_part.shape[0])
    _lib.call("att_spmm", _p(rowptr), _p(col), _p(val), _DT[val.dtype], _p(window_of_part),
              _p(atomic), n_parts, _p(X), _DT[X.dtype], _p(x_scale), n_x, F, ldx, _p(out),
              m_out, ldy, window, wide, _p(err_flag), _stream())
    return out


def spmm_format(fmt: BlockFormat, X, m_out, out=None, x_scale=None):
    return spmm(fmt.rowptr, fmt.col, fmt.val, fmt.window_of_part, fmt.atomic, X, m_out,
                window=fmt.window, wide=fmt.wide, out=out, x_scale=x_scale)
