"""Sharded (multi-rank) basis build on CPU: world_size 2 over gloo.

Each rank builds its work-balanced cell range with the FP64 oracle (the GPU
library is not needed to test the rank logic), the Galerkin blocks are
all-gathered, and every rank must hold exactly the single-process result.
Also checks the partition (coverage, order, balance), the max-over-ranks
timing reduction and the weak-scaling throughput of the benchmark's
multi-GPU mode (every rank builds a whole batch).
"""
import os
import socket
import tempfile

import numpy as np
import pytest

import sharding
import workloads


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 7])
def test_partition_covers_in_order_and_balances(world):
    cells = workloads.q1_uneven(m=4, seed=3)[0]
    w = sharding.cell_work(cells, "q1")
    ranges = [sharding.partition(w, world, r) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == len(cells)
    for (a, b), (c, d) in zip(ranges, ranges[1:]):
        assert b == c and a <= b
    share = np.array([w[a:b].sum() for a, b in ranges])
    assert share.sum() == w.sum()
    # every range ends within one cell of its quantile
    assert share.max() <= w.sum() / world + w.max()


def test_cell_work_matches_the_workload_measures():
    """Per-cell work of every pairing sums to the workload generators' totals."""
    cells = workloads.coarse_grid(2, [1, 2, 3, 2, 1, 3, 2, 1])
    assert sharding.cell_work(cells, "q1").sum() == workloads.work_dof_rhs(cells)
    assert sharding.cell_work(cells, "nedrt").sum() == workloads.nedrt_work_dof_rhs(cells)
    assert sharding.cell_work(cells, "qned").sum() == workloads.qned_work_dof_rhs(cells)
    assert sharding.cell_work(cells, "rtdq").sum() == workloads.rtdq_work_dof_rhs(cells)
    with pytest.raises(ValueError):
        sharding.cell_work(cells, "p2")


def test_partition_more_ranks_than_cells():
    w = np.array([5, 1, 1])
    ranges = [sharding.partition(w, 5, r) for r in range(5)]
    assert sum(b - a for a, b in ranges) == 3 and ranges[-1][1] == 3


def _oracle_build(cells, arrays):
    from oracle import oracle
    (a,) = arrays
    if len(cells) == 0:
        return np.zeros((0, 8, 8)), np.zeros((0, 8))
    r = oracle.q1_build(cells["origin"], cells["size"], cells["depth"], a,
                        load_kind=oracle.LOAD_SIN_PRODUCT, load_params=(1, 1, 0, 0), want_phi=False)
    return r["KH"], r["FH"]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cells, a, _, _ = workloads.q1_lognormal(m=2, depth=2, seed=11, reaction=False)
        KH, FH = sharding.build_sharded(_oracle_build, cells, [a], "q1", world, rank, dist)
        t = sharding.max_over_ranks(1.0 + rank, dist)
        # weak scaling (the benchmark's multi-GPU mode): every rank builds the whole batch
        KHw, FHw = _oracle_build(cells, [a])
        work = float(workloads.work_dof_rhs(cells))
        v = sharding.weak_scaling_value(work, 1.0 + rank, dist)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), KH=KH, FH=FH, t=t, KHw=KHw, v=v, work=work)
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_match_single_process(oracle_lib):
    import torch.multiprocessing as mp
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(world, _free_port(), d), nprocs=world, start_method="spawn")
        cells, a, _, _ = workloads.q1_lognormal(m=2, depth=2, seed=11, reaction=False)
        KH_ref, FH_ref = _oracle_build(cells, [a])
        for r in range(world):
            g = np.load(os.path.join(d, f"rank{r}.npz"))
            assert np.array_equal(g["KH"], KH_ref) and np.array_equal(g["FH"], FH_ref)
            assert float(g["t"]) == 2.0
            assert np.array_equal(g["KHw"], KH_ref)
            assert float(g["v"]) == world * float(g["work"]) / 2.0  # all ranks' work / slowest rank


class _FakeDist:
    """Stand-in for torch.distributed that reports a backend name."""

    def __init__(self, backend):
        self.backend = backend

    def get_backend(self, group=None):
        return self.backend


def test_exchange_device_follows_the_backend(monkeypatch):
    """NCCL collectives take CUDA tensors only: the helpers put their tensors
    on the current CUDA device for NCCL and on the host for gloo."""
    import torch
    assert sharding.exchange_device(_FakeDist("gloo")) == torch.device("cpu")
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 3)
    assert sharding.exchange_device(_FakeDist("nccl")) == torch.device("cuda", 3)
