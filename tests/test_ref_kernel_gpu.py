"""The reference's own GCN SpMM kernel (built from the reference tree into
oracle/_ref/ref_spmm.fatbin) beside this repository's kernel on the same
inputs, both against FP64.

The reference kernel accumulates in fp16 (m16n8k8 f16.f16.f16.f16,
gcn/SpMM/spmm_utils/compute_utils.h:324-332); this repository's accumulates
in fp32.  On the reference's own integer test both are exact; on the
16,384-node graph each error is reported, ours held to 1e-2 normwise and the
reference's only to 5e-2 (a check that the launch reproduces the reference's
call, not a claim about its accuracy).  Skipped where the fatbin was not
built (it needs the reference tree at build time)."""
import numpy as np
import pytest
import torch

from oracle import oracle, ref_spmm
from tests._fixture import ROW, COL

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_spmm.available(), reason="reference fatbin not built")]


def test_reference_kernel_on_its_own_integer_test(cuda):
    """gcn/SpMM/test/mgcn/test_balance.py:20-62: the fixture, deg = 1,
    integer features -> both kernels exact."""
    from att_gb300.compat import Block_sr_bcrs, SpMM_sr_bcrs
    fmt = Block_sr_bcrs.blockProcess_fp16_balance(torch.from_numpy(ROW), torch.from_numpy(COL),
                                                  torch.ones(32, dtype=torch.float16), 8, 8, 32)
    fmt = [t.cuda() for t in fmt]
    for dimN in (64, 128):
        rhs = torch.randint(1, 3, (30, dimN), generator=torch.Generator().manual_seed(dimN)).half()
        ref = oracle.spmm_csr_fp64(ROW, COL, np.ones(COL.shape[0]), rhs.double().numpy(), 30)
        theirs = ref_spmm.forward_fp16_gnn(*fmt, rhs.cuda(), 32, dimN, 30)[0]
        ours = SpMM_sr_bcrs.forward_fp16_gnn(*fmt, rhs.cuda(), 32, dimN, 30)[0]
        assert np.array_equal(theirs.cpu().double().numpy(), ref)
        assert np.array_equal(ours.cpu().double().numpy(), ref)


def test_reference_tf32_kernel_on_its_own_integer_test(cuda):
    from att_gb300.compat import Block_sr_bcrs, SpMM_sr_bcrs
    fmt = Block_sr_bcrs.blockProcess_tf32_balance(torch.from_numpy(ROW), torch.from_numpy(COL),
                                                  torch.ones(32, dtype=torch.float32), 8, 4, 32)
    fmt = [t.cuda() for t in fmt]
    rhs = torch.randint(1, 3, (30, 64), generator=torch.Generator().manual_seed(1)).float()
    ref = oracle.spmm_csr_fp64(ROW, COL, np.ones(COL.shape[0]), rhs.double().numpy(), 30)
    theirs = ref_spmm.forward_tf32_gnn(*fmt, rhs.cuda(), 32, 64, 30)[0]
    ours = SpMM_sr_bcrs.forward_tf32_gnn(*fmt, rhs.cuda(), 32, 64, 30)[0]
    assert np.array_equal(theirs.cpu().double().numpy(), ref)
    assert np.array_equal(ours.cpu().double().numpy(), ref)


def test_both_kernels_vs_fp64_on_gcn16k(cuda):
    """The 16,384-node GCN graph (gamma 2.1, mean degree 10, seed 0), F = 64."""
    import bench
    from att_gb300.compat import SpMM_sr_bcrs
    wl = bench.SpmmGcn16k("cuda")
    f = wl.fmt
    rp = wl.rowptr.cpu().numpy()
    col = wl.colidx.cpu().numpy()
    vals = oracle.gcn_values(rp, col, wl.deg.cpu().numpy()).astype(np.float64)
    ref = oracle.spmm_csr_fp64(rp, col, vals, wl.X.double().cpu().numpy(), wl.n)
    args = (f.rowptr, f.col, f.val, f.window_of_part, f.atomic, wl.X, rp.shape[0] - 1, wl.F, wl.n)
    theirs = ref_spmm.forward_fp16_gnn(*args)[0]
    ours = SpMM_sr_bcrs.forward_fp16_gnn(*args)[0]
    e_theirs = oracle.rel_err(theirs.cpu().numpy(), ref)
    e_ours = oracle.rel_err(ours.cpu().numpy(), ref)
    print("rel err vs FP64: reference kernel %.3g, ours %.3g" % (e_theirs, e_ours))
    assert e_ours <= 1e-2
    assert e_theirs <= 5e-2
    assert e_ours <= e_theirs
