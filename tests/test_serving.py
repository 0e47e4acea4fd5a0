"""Host logic of the serving loop (no GPU): admission by HBM budget, arrival
process, request sizes, the job-table prefixes and the C layout of
att_spmm_job as the ctypes mirror sees it."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest
import torch

from att_gb300 import _lib, ops, serving

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_admission_budget_and_slots():
    adm = serving.Admission(budget=100, max_active=3)
    assert adm.try_admit(40) and adm.try_admit(40)
    assert not adm.try_admit(30)          # 110 > 100: waits
    assert adm.try_admit(20)              # 100 fits exactly
    assert not adm.try_admit(0)           # no free slot
    adm.release(40)
    assert adm.used == 60 and adm.active == 2
    assert adm.try_admit(30)
    assert adm.fits_ever(100) and not adm.fits_ever(101)
    with pytest.raises(RuntimeError):
        serving.Admission(10, 1).release(5)   # release without admission


def test_admission_injected_failures_keep_accounting():
    """Requests that fail after admission (a malformed graph, an allocation
    failure) release exactly what they took; the budget returns to zero."""
    adm = serving.Admission(budget=1000, max_active=8)
    taken = []
    rng = np.random.default_rng(0)
    for i in range(200):
        est = int(rng.integers(1, 300))
        if adm.try_admit(est):
            taken.append(est)
        if taken and rng.random() < 0.5:   # a completion or an injected failure
            adm.release(taken.pop(int(rng.integers(0, len(taken)))))
        assert 0 <= adm.used <= adm.budget and adm.active == len(taken) <= adm.max_active
    for est in taken:
        adm.release(est)
    assert adm.used == 0 and adm.active == 0


def test_memory_estimate_monotone():
    a = serving.memory_estimate(1000, 10_000)
    assert serving.memory_estimate(2000, 10_000) > a
    assert serving.memory_estimate(1000, 20_000) > a
    # the largest request of the workload (500K nodes, mean degree 50) fits ~80x in 120 GB
    big = serving.memory_estimate(500_000, 25_000_000)
    assert 0.5e9 < big < 2e9


def test_poisson_arrivals_rate():
    t = serving.poisson_arrivals(200.0, 20_000, seed=4)
    assert np.all(np.diff(t) > 0)
    rate = len(t) / t[-1]
    assert abs(rate - 200.0) / 200.0 < 0.03
    assert np.array_equal(t, serving.poisson_arrivals(200.0, 20_000, seed=4))


def test_graph_sizes_distribution():
    s = serving.graph_sizes(4000, seed=4)
    n = np.array([a for a, _ in s], dtype=np.float64)
    d = np.array([b for _, b in s])
    assert n.min() >= 1000 and n.max() <= 500_000
    assert d.min() >= 5 and d.max() <= 50
    # log-uniform: log n roughly uniform over [log 1e3, log 5e5]
    u = (np.log(n) - np.log(1e3)) / (np.log(5e5) - np.log(1e3))
    assert abs(u.mean() - 0.5) < 0.02 and abs(d.mean() - 27.5) < 1.0


def _fake_job(n, F, n_parts, n_groups, n_red):
    i32 = lambda k: torch.zeros(max(k, 1), dtype=torch.int32)
    fmt = ops.BlockFormat(rowptr=i32(2 * n_parts + 1), col=i32(8), window_of_part=i32(n_parts),
                          atomic=i32(n_parts), window=8, wide=8, part=32, n_rows=n, n_cols=n,
                          nnz=0, val=torch.zeros(64, dtype=torch.float16))
    g = serving.Groups(i32(n_groups + 1), i32(n_groups), i32(n_red + 1), i32(3), n_groups, n_red,
                       2 * n_red, 1, n)
    part = torch.zeros(2 * n_red * 8 * F, dtype=torch.float32) if n_red else None
    X = torch.zeros(n, F, dtype=torch.float16)
    Y = torch.zeros(n, F, dtype=torch.float32)
    return serving.Job(fmt, g, part, X, Y, n, y_ptr=Y.data_ptr())  # host Y: address given


def test_job_table_prefixes():
    jobs = [_fake_job(100, 128, 20, 15, 2), _fake_job(7, 64, 1, 1, 0), _fake_job(33, 192, 9, 9, 1)]
    table, header = serving.build_job_table(jobs)
    assert header == (3, 15 * 2 + 1 * 1 + 9 * 3, 3, 3, 0)
    assert [table[k].item_begin for k in range(3)] == [0, 30, 31]
    assert [table[k].empty_begin for k in range(3)] == [0, 1, 2]
    assert [table[k].red_begin for k in range(3)] == [0, 2, 2]
    assert table[1].partial is None and table[0].partial == jobs[0].partial.data_ptr()
    assert table[2].ldx == 192 and table[2].ldy == 192 and table[2].m_out == 33
    assert table[0].n_slots == 4 and table[1].n_empty == 1


def test_job_table_rejects_bad_jobs():
    j = _fake_job(16, 64, 2, 2, 1)
    j.partial = None
    with pytest.raises(ValueError):
        serving.build_job_table([j])
    j = _fake_job(16, 64, 2, 2, 0)
    j.X = torch.zeros(16, 64, dtype=torch.float32)
    with pytest.raises(ValueError):
        serving.build_job_table([j])
    j = _fake_job(16, 64, 2, 2, 0)
    j.y_ptr = None  # a host Y without its device address
    with pytest.raises(ValueError):
        serving.build_job_table([j])
    j = _fake_job(16, 64, 2, 2, 0)
    j.m_out = 15   # groups built for another row count
    j.Y = torch.zeros(15, 64)
    with pytest.raises(ValueError):
        serving.build_job_table([j])


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_job_struct_layout_matches_header(tmp_path):
    """Offsets and size of att_spmm_job from the C header equal the ctypes mirror."""
    fields = [f for f, _ in _lib.SpmmJob._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "att_gb300.h"\n'
                   'int main(void) {\n  printf("%zu", sizeof(att_spmm_job));\n'
                   + "".join('  printf(" %%zu", offsetof(att_spmm_job, %s));\n' % f for f in fields)
                   + '  printf("\\n");\n  return 0;\n}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    want = [ctypes.sizeof(_lib.SpmmJob)] + [getattr(_lib.SpmmJob, f).offset for f in fields]
    assert got == want
