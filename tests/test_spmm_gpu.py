"""Blocked SpMM on the GPU vs the FP64 oracle.

Tolerances (normwise relative, max|err| / max|ref|): fp16 and bf16 features
1e-2, fp32 (3xTF32) 1e-4; integer-valued inputs must match exactly, as the
reference's own test_balance.py demands."""
import numpy as np
import pytest
import torch

from oracle import oracle
from tests._fixture import ROW, COL

pytestmark = pytest.mark.gpu

TOL = {torch.float16: 1e-2, torch.bfloat16: 1e-2, torch.float32: 1e-4}


def _format(rowptr, col, deg, W, w, P, emit=False):
    from att_gb300 import ops
    return ops.block_convert(torch.from_numpy(rowptr), torch.from_numpy(col),
                             torch.from_numpy(deg), window=W, wide=w, part=P, emit_empty=emit)


def _ref(rowptr, col, vals, X, m_out, W):
    n_used = (rowptr.shape[0] - 1) // W * W
    rp = rowptr[: n_used + 1]
    Y = oracle.spmm_csr_fp64(rp, col[: rp[-1]], vals[: rp[-1]], X, None)
    out = np.zeros((m_out, X.shape[1]))
    k = min(m_out, Y.shape[0])
    out[:k] = Y[:k]
    return out


def test_reference_balance_test_exact(cuda):
    """gcn/SpMM/test/mgcn/test_balance.py:20-62: fixture, deg = 1, integer
    features -> exact."""
    from att_gb300.compat import Block_sr_bcrs, SpMM_sr_bcrs
    for dimN in (64, 128, 66, 125):
        fmt = Block_sr_bcrs.blockProcess_fp16_balance(torch.from_numpy(ROW), torch.from_numpy(COL),
                                                      torch.ones(32, dtype=torch.float16), 8, 8, 32)
        rhs = torch.randint(1, 3, (30, dimN)).half()
        fmt = [t.cuda() for t in fmt]
        Y = SpMM_sr_bcrs.forward_fp16_gnn(fmt[0], fmt[1], fmt[2], fmt[3], fmt[4], rhs.cuda(), 32,
                                          dimN, 30)[0]
        ref = _ref(ROW, COL, np.ones(COL.shape[0]), rhs.double().numpy(), 30, 8)
        assert Y.shape == (30, dimN) and Y.dtype == torch.float32
        assert np.array_equal(Y.cpu().double().numpy(), ref)


def test_reference_balance_test_exact_tf32(cuda):
    from att_gb300.compat import Block_sr_bcrs, SpMM_sr_bcrs
    fmt = Block_sr_bcrs.blockProcess_tf32_balance(torch.from_numpy(ROW), torch.from_numpy(COL),
                                                  torch.ones(32, dtype=torch.float32), 8, 4, 2)
    rhs = torch.randint(1, 3, (30, 64)).float()
    fmt = [t.cuda() for t in fmt]
    Y = SpMM_sr_bcrs.forward_tf32_gnn(fmt[0], fmt[1], fmt[2], fmt[3], fmt[4], rhs.cuda(), 32, 64,
                                      30)[0]
    ref = _ref(ROW, COL, np.ones(COL.shape[0]), rhs.double().numpy(), 30, 8)
    assert np.array_equal(Y.cpu().double().numpy(), ref)


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16, torch.float32])
@pytest.mark.parametrize("W,w,P", [(8, 8, 32), (16, 8, 32), (8, 8, 2), (16, 16, 3), (8, 4, 32),
                                   (16, 4, 5)])
@pytest.mark.parametrize("F", [32, 64, 128, 256, 96])
def test_random_power_law_vs_fp64(cuda, dtype, W, w, P, F):
    from att_gb300 import graphs, ops
    if (dtype == torch.float32) != (w == 4):
        if not (dtype == torch.float32 and w == 8):
            pytest.skip("wide 4 is the fp32 layout")
    rp_t, col_t = graphs.chung_lu(3000, 12, 2.1, seed=11)
    rowptr = graphs.pad_rows(rp_t, 8).numpy()
    col = col_t.numpy()
    n = 3000
    deg32 = graphs.gcn_degree(torch.from_numpy(rowptr), torch.float32).numpy()
    deg32[~np.isfinite(deg32)] = 0
    deg = deg32.astype(np.float16) if dtype != torch.float32 else deg32
    f = _format(rowptr, col, deg, W, w, P, emit=(dtype == torch.float32))
    val = f.val if dtype != torch.bfloat16 else f.val.to(torch.bfloat16)
    rng = np.random.default_rng(F)
    X = torch.from_numpy(rng.uniform(-1, 1, size=(n, F)).astype(np.float32)).to(dtype)
    Y = ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, X.cuda(), n, window=W, wide=w)
    vals = val.float().cpu().numpy()
    # reference values: the block format's own (rounded) values, per CSR edge
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    if dtype == torch.bfloat16:
        ev = torch.from_numpy(ev).to(torch.bfloat16).double().numpy()
    ref = _ref(rowptr, col, ev, X.double().numpy(), n, W)
    err = oracle.rel_err(Y.cpu().numpy(), ref)
    assert err <= TOL[dtype], (dtype, W, w, P, F, err)
    # error against the unrounded FP64 problem stays within the same bound
    ev64 = oracle.gcn_values(rowptr, col, deg32).astype(np.float64)
    ref64 = _ref(rowptr, col, ev64, X.float().double().numpy(), n, W)
    assert oracle.rel_err(Y.cpu().numpy(), ref64) <= max(TOL[dtype], 1e-2 if dtype != torch.float32 else 1e-4)


def test_hub_window_split_and_uncovered_rows(cuda):
    from att_gb300 import graphs, ops
    rowptr, col = graphs.random_csr(203, 4000, 9, seed=3, hub_rows=2, hub_len=3500,
                                    empty_frac=0.3)
    deg = np.full(4000, 0.5, np.float16)
    f = _format(rowptr, col, deg, 8, 8, 4)
    assert int(f.atomic.sum()) > 0
    X = torch.randn(4000, 64).half().cuda()
    m_out = 210  # rows past the last window must come back zero
    Y = torch.full((m_out, 64), float("nan"), device="cuda")
    ops.spmm(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, X, m_out, window=8, wide=8, out=Y)
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    ref = _ref(rowptr, col, ev, X.double().cpu().numpy(), m_out, 8)
    assert oracle.rel_err(Y.cpu().numpy(), ref) <= 1e-2
    assert torch.all(Y[200:] == 0)


def test_bad_column_sets_error_flag(cuda):
    from att_gb300 import ops
    f = _format(ROW, COL, np.ones(32, np.float16), 8, 8, 32)
    col = f.col.clone()
    col[3] = 1000
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    X = torch.ones(30, 64, dtype=torch.float16, device="cuda")
    ops.spmm(f.rowptr, col, f.val, f.window_of_part, f.atomic, X, 30, err_flag=err)
    torch.cuda.synchronize()
    assert int(err.item()) != 0


def _quant_e4m3(X):
    """Per-row fp32 scales and e4m3 codes (scale = max|x| / 448)."""
    amax = X.abs().amax(1).clamp_min(1e-12)
    scale = (amax / 448.0).float()
    Xq = (X / scale[:, None]).to(torch.float8_e4m3fn)
    return Xq, scale


@pytest.mark.parametrize("W,w", [(8, 8), (16, 8), (8, 16)])
@pytest.mark.parametrize("F", [64, 128, 256])
def test_fp8_features_vs_fp64(cuda, W, w, F):
    """FP8 E4M3 features with per-row fp32 scales.  The kernel: within 1e-2 of
    the FP64 product on the dequantized features.  The format: against the
    FP64 product on the unquantized features, Frobenius-relative error within
    the stated FP8 tolerance 3e-2; E4M3 keeps 3 mantissa bits (rounding error
    up to 3.1 % per element), so the max-elementwise normwise error is bounded
    at 5e-2."""
    from att_gb300 import graphs, ops
    rp_t, col_t = graphs.chung_lu(3000, 12, 2.1, seed=13)
    rowptr = graphs.pad_rows(rp_t, 8).numpy()
    col = col_t.numpy()
    n = 3000
    deg = graphs.gcn_degree(torch.from_numpy(rowptr), torch.float32).numpy()
    deg[~np.isfinite(deg)] = 0
    deg = deg.astype(np.float16)
    f = _format(rowptr, col, deg, W, w, 32)
    g = torch.Generator().manual_seed(F)
    X = torch.rand(n, F, generator=g) * 2 - 1
    Xq, scale = _quant_e4m3(X)
    Y = ops.spmm(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, Xq.cuda(), n, window=W,
                 wide=w, x_scale=scale.cuda())
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    Xdq = (Xq.float() * scale[:, None]).double().numpy()
    ref_q = _ref(rowptr, col, ev, Xdq, n, W)
    assert oracle.rel_err(Y.cpu().numpy(), ref_q) <= 1e-2
    ref = _ref(rowptr, col, ev, X.double().numpy(), n, W)
    assert oracle.rel_err_fro(Y.cpu().numpy(), ref) <= 3e-2
    assert oracle.rel_err(Y.cpu().numpy(), ref) <= 5e-2


@pytest.fixture
def gather_mode():
    """Set att_set_option("spmm_gather", mode) for a test and restore it."""
    from att_gb300 import _lib
    import ctypes
    old = ctypes.c_int(0)
    _lib.call("att_get_option", b"spmm_gather", ctypes.byref(old))
    yield lambda m: _lib.call("att_set_option", b"spmm_gather", m)
    _lib.call("att_set_option", b"spmm_gather", old.value)


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16])
@pytest.mark.parametrize("P", [32, 2])
@pytest.mark.parametrize("F", [64, 72, 128, 96])
def test_bulk_row_copies_match(cuda, gather_mode, dtype, P, F):
    """spmm_gather = 2 (one cp.async.bulk per gathered row) gives the default
    producer's result (same arithmetic; split windows add atomically, so
    within fp32 rounding) and stays within 1e-2 of FP64, including partial
    feature chunks (F = 72, 96), split windows and rows past the last window."""
    from att_gb300 import graphs, ops
    rowptr, col = graphs.random_csr(3003, 3003, 30, seed=P + F, hub_rows=5, hub_len=2500,
                                    empty_frac=0.2)
    deg = np.full(3003, 0.25, np.float16)
    f = _format(rowptr, col, deg, 8, 8, P)
    val = f.val if dtype == torch.float16 else f.val.to(torch.bfloat16)
    X = torch.from_numpy(np.random.default_rng(F).uniform(-1, 1, (3003, F)).astype(np.float32))
    X = X.to(dtype).cuda()
    m_out = 3010
    outs = []
    for mode in (0, 2):
        gather_mode(mode)
        Y = torch.full((m_out, F), float("nan"), device="cuda")
        ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, X, m_out, window=8, wide=8,
                 out=Y)
        outs.append(Y.cpu().numpy())
    assert oracle.rel_err(outs[1], outs[0]) <= 1e-6
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    if dtype == torch.bfloat16:
        ev = torch.from_numpy(ev).to(torch.bfloat16).double().numpy()
    ref = _ref(rowptr, col, ev, X.double().cpu().numpy(), m_out, 8)
    assert oracle.rel_err(outs[1], ref) <= 1e-2
    assert np.all(outs[1][3000:] == 0)


def test_bulk_row_copies_flag_bad_column(cuda, gather_mode):
    from att_gb300 import ops
    gather_mode(2)
    f = _format(ROW, COL, np.ones(32, np.float16), 8, 8, 32)
    col = f.col.clone()
    col[3] = 1000
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    X = torch.ones(30, 64, dtype=torch.float16, device="cuda")
    Y = ops.spmm(f.rowptr, col, f.val, f.window_of_part, f.atomic, X, 30, err_flag=err)
    torch.cuda.synchronize()
    assert int(err.item()) & 1 and bool(torch.isfinite(Y).all())


@pytest.fixture
def fp8_mode():
    """Set att_set_option("spmm_fp8", mode) for a test and restore it."""
    from att_gb300 import _lib
    import ctypes
    old = ctypes.c_int(1)
    _lib.call("att_get_option", b"spmm_fp8", ctypes.byref(old))
    yield lambda m: _lib.call("att_set_option", b"spmm_fp8", m)
    _lib.call("att_set_option", b"spmm_fp8", old.value)


@pytest.mark.parametrize("W,w", [(8, 8), (16, 8), (8, 16), (16, 16)])
@pytest.mark.parametrize("F,pad", [(128, 0), (80, 0), (64, 0), (144, 0), (128, 1)])
def test_fp8_register_dequant_matches_tile(cuda, fp8_mode, W, w, F, pad):
    """The register-dequant FP8 kernel (spmm_fp8 = 1, the default) rounds
    fp16(value * scale) where the tile kernel rounds fp16(code * scale): one
    fp16 rounding (2^-11 relative) per product in each, in a different place,
    so the two agree within 2e-3 max-normwise.  Covers 128-feature
    items with a partial last chunk (F = 80, 144), 64-feature items (F = 64),
    an odd output stride (scalar stores instead of float2), split windows and
    rows past the last window; and stays within 1e-2 of FP64 on the
    dequantized features."""
    from att_gb300 import graphs, ops
    n = 2403
    rowptr, col = graphs.random_csr(n, n, 20, seed=F + W + w, hub_rows=4, hub_len=1800,
                                    empty_frac=0.2)
    deg = np.full(n, 0.3, np.float16)
    f = _format(rowptr, col, deg, W, w, 8)
    assert int(f.atomic.sum()) > 0
    X = torch.from_numpy(np.random.default_rng(F).uniform(-2, 2, (n, F)).astype(np.float32))
    X[5] = 0  # an all-zero row: scale clamps, codes are zero
    Xq, scale = _quant_e4m3(X)
    m_out = n + 9
    outs = []
    for mode in (0, 1):
        fp8_mode(mode)
        Yb = torch.full((m_out, F + pad), float("nan"), device="cuda")
        Y = Yb[:, :F]
        ops.spmm(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, Xq.cuda(), m_out, window=W,
                 wide=w, x_scale=scale.cuda(), out=Y)
        outs.append(Y.cpu().numpy())
        if pad:
            assert torch.isnan(Yb[:, F:]).all()
    assert np.all(np.isfinite(outs[1]))
    assert oracle.rel_err(outs[1], outs[0]) <= 2e-3
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    Xdq = (Xq.float() * scale[:, None]).double().numpy()
    ref_q = _ref(rowptr, col, ev, Xdq, m_out, W)
    assert oracle.rel_err(outs[1], ref_q) <= 1e-2
    assert np.all(outs[1][n:] == 0)


@pytest.mark.parametrize("W,w", [(8, 8), (16, 16)])
def test_fp8_scale_fallback_steps(cuda, fp8_mode, W, w):
    """Row scales spanning about 5e-10 .. 36 (dequantized features up to
    16000, inside fp16's range as every FP8 path needs): the register kernel
    folds each step's scales into the block values as fp16(value * scale *
    2^15) and, on a step where one of those leaves fp16's normal range (value
    0.3 times a scale above 6.6 overflows it), scales the e4m3 codes instead
    for that step.  Steps of both kinds inside one work item; the result stays
    within 1e-2 of FP64 on the dequantized features and within 2e-3 of the
    tile kernel."""
    from att_gb300 import graphs, ops
    n = 4099
    rowptr, col = graphs.random_csr(n, n, 24, seed=W + 5, hub_rows=3, hub_len=2000,
                                    empty_frac=0.1)
    deg = np.full(n, 0.3, np.float16)
    f = _format(rowptr, col, deg, W, w, 32)
    rng = np.random.default_rng(W)
    X = rng.uniform(-2, 2, (n, 128)).astype(np.float32)
    X *= (10.0 ** rng.uniform(-2, 1, n)).astype(np.float32)[:, None]
    X[::97] = rng.uniform(-2, 2, (len(X[::97]), 128)) * 8000.0  # scale about 36: steps fall back
    X[3::89] *= 1e-5       # scales down to about 5e-10
    X = torch.from_numpy(X)
    Xq, scale = _quant_e4m3(X)
    outs = []
    for mode in (0, 1):
        fp8_mode(mode)
        Y = ops.spmm(f.rowptr, f.col, f.val, f.window_of_part, f.atomic, Xq.cuda(), n, window=W,
                     wide=w, x_scale=scale.cuda())
        outs.append(Y.cpu().numpy())
    assert np.all(np.isfinite(outs[1]))
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    Xdq = (Xq.float() * scale[:, None]).double().numpy()
    ref_q = _ref(rowptr, col, ev, Xdq, n, W)
    assert oracle.rel_err(outs[1], ref_q) <= 1e-2
    assert oracle.rel_err(outs[1], outs[0]) <= 2e-3


def test_fp8_register_dequant_flags_bad_column(cuda, fp8_mode):
    from att_gb300 import ops
    fp8_mode(1)
    f = _format(ROW, COL, np.ones(32, np.float16), 8, 8, 32)
    col = f.col.clone()
    col[3] = 1000
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    Xq, scale = _quant_e4m3(torch.ones(30, 128))
    Y = ops.spmm(f.rowptr, col, f.val, f.window_of_part, f.atomic, Xq.cuda(), 30,
                 x_scale=scale.cuda(), err_flag=err)
    torch.cuda.synchronize()
    assert int(err.item()) & 1 and bool(torch.isfinite(Y).all())


@pytest.fixture
def restore_spmm_options():
    from att_gb300 import _lib
    import ctypes
    keys = (b"spmm_fc", b"spmm_stages", b"spmm_fp8", b"spmm_gather", b"spmm_tf32")
    old = {}
    for k in keys:
        v = ctypes.c_int(0)
        _lib.call("att_get_option", k, ctypes.byref(v))
        old[k] = v.value
    yield
    for k, v in old.items():
        _lib.call("att_set_option", k, v)


@pytest.mark.parametrize("dtype", [torch.float16, torch.bfloat16, torch.float8_e4m3fn,
                                   torch.float32])
def test_autotune_spmm_picks_a_measured_shape(cuda, restore_spmm_options, dtype):
    """tune_spmm times every candidate shape and returns the fastest without
    changing the options in effect afterwards (read back through
    att_get_option); the chosen shape, passed per call, gives the default
    shape's result (same arithmetic; atomics may reorder fp32 adds -- except
    FP8, whose two kernels round the scaled products in different places and
    agree within 2e-3), and the next call without a shape is back at the
    defaults."""
    from att_gb300 import _lib, autotune, graphs, ops
    import ctypes
    rowptr, col = graphs.random_csr(2000, 2000, 25, seed=9, hub_rows=3, hub_len=1500)
    deg = np.full(2000, 0.2, np.float16)
    f = _format(rowptr, col, deg, 8, 8, 32)
    X = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, (2000, 128)).astype(np.float32))
    scale = None
    val = f.val
    if dtype == torch.float8_e4m3fn:
        Xk, scale = _quant_e4m3(X)
        Xk, scale = Xk.cuda(), scale.cuda()
    else:
        Xk = X.to(dtype).cuda()
        val = f.val.to(dtype)

    def options():
        got = {}
        for k in (b"spmm_fc", b"spmm_stages", b"spmm_fp8", b"spmm_tf32"):
            v = ctypes.c_int(0)
            _lib.call("att_get_option", k, ctypes.byref(v))
            got[k] = v.value
        return got
    before = options()
    Y0 = ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, Xk, 2000, x_scale=scale)
    tuner = autotune.Tuner(warmup=1, reps=3)
    choice, table = autotune.tune_spmm(f, Xk, 2000, x_scale=scale, val=val, tuner=tuner)
    assert set(table) == set(autotune.spmm_candidates(dtype, 128))
    assert choice == min(table, key=table.get)
    assert options() == before
    Y1 = ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, Xk, 2000, x_scale=scale,
                  shape=choice)
    same = 2e-3 if dtype == torch.float8_e4m3fn else 1e-6
    assert oracle.rel_err(Y1.cpu().numpy(), Y0.cpu().numpy()) <= same
    # a call without a shape runs (and leaves the thread) at the defaults
    Y2 = ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, Xk, 2000, x_scale=scale)
    assert options() == before
    assert oracle.rel_err(Y2.cpu().numpy(), Y0.cpu().numpy()) <= 1e-6


@pytest.mark.parametrize("F", [64, 72, 128, 36])
def test_tf32_shapes_vs_fp64(cuda, restore_spmm_options, F):
    """Every fp32-feature kernel shape (spmm_tf32 0..3: 64 x 4, 32 x 3,
    32 x 4, 64 x 2 features per item x ring depth) within 1e-4 of FP64,
    including partial feature chunks, split windows and rows past the last
    window."""
    from att_gb300 import _lib, graphs, ops
    rowptr, col = graphs.random_csr(2003, 2003, 25, seed=F, hub_rows=4, hub_len=1700,
                                    empty_frac=0.2)
    deg = np.full(2003, 0.3, np.float16)
    f = _format(rowptr, col, deg, 8, 4, 8)
    val = f.val.float()
    X = torch.from_numpy(np.random.default_rng(F).uniform(-1, 1, (2003, F)).astype(np.float32))
    ev = oracle.gcn_values(rowptr, col, deg).astype(np.float64)
    ref = _ref(rowptr, col, ev, X.double().numpy(), 2010, 8)
    for shape in range(4):
        _lib.call("att_set_option", b"spmm_tf32", shape)
        Y = torch.full((2010, F), float("nan"), device="cuda")
        ops.spmm(f.rowptr, f.col, val, f.window_of_part, f.atomic, X.cuda(), 2010, window=8,
                 wide=4, out=Y)
        assert oracle.rel_err(Y.cpu().numpy(), ref) <= 1e-4, shape
