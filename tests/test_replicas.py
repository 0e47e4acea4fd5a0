"""Multi-GPU runs as independent replicas (att_gb300.replicas), exercised on
CPU with the gloo backend and two ranks: the step time is the maximum over
ranks, the job's throughput counts every rank's units, only rank 0 reports,
and the replicas compute identical results (each rank converts and
aggregates its own copy of the same seeded graph with the oracle)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      LOCAL_RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from att_gb300 import graphs, replicas
        from oracle import oracle
        r, lr, w = replicas.env_rank()
        assert (r, lr, w) == (rank, rank, world)
        # rank-dependent local times: the job's time is the slowest rank's
        mx = replicas.max_over_ranks([1.0 + rank, 5.0 - rank])
        rate = replicas.aggregate_rate(1000.0, mx[0], world)
        # each replica: the whole seeded graph, converted and aggregated
        rp, col = graphs.random_csr(400, 400, 12, seed=7, hub_rows=2, hub_len=300)
        deg = np.full(400, 0.5, np.float16)
        fmt = oracle.block_convert(rp, col, deg, 8, 8, 4)
        X = np.random.default_rng(3).uniform(-1, 1, (400, 16))
        Y = oracle.spmm_blocks_fp64(fmt, X, 400)
        sums = torch.tensor([float(Y.sum()), float(np.abs(Y).sum())], dtype=torch.float64)
        gathered = [torch.zeros_like(sums) for _ in range(world)]
        dist.all_gather(gathered, sums)
        np.save(os.path.join(out_dir, "r%d.npy" % rank),
                np.array([mx[0], mx[1], rate, float(replicas.reports(rank))]
                         + [float(v) for g in gathered for v in g]))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_gloo(tmp_path):
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    res = [np.load(tmp_path / ("r%d.npy" % r)) for r in range(world)]
    for r, v in enumerate(res):
        assert v[0] == 2.0 and v[1] == 5.0            # max over ranks, element-wise
        assert v[2] == pytest.approx(2 * 1000.0 / 2e-3)  # world x units / slowest time
        assert v[3] == (1.0 if r == 0 else 0.0)         # rank 0 alone reports
        sums = v[4:].reshape(world, 2)
        assert np.array_equal(sums[0], sums[1])         # replicas agree bit-for-bit


def test_single_process_passthrough():
    from att_gb300 import replicas
    assert replicas.max_over_ranks([3.5, 1.25]) == [3.5, 1.25]
    assert replicas.aggregate_rate(10.0, 1.0, 1) == pytest.approx(1e4)
