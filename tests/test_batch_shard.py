"""Batched domains across ranks: whole domains dealt out by cell count
(longest processing time first), and the one quantity that crosses between
ranks, the FP64 conservation sums, gathered identically on every rank (two
gloo ranks on CPU)."""
import os
import socket

import numpy as np
import pytest

from lbm_gb300.batch import batched_workload, partition, sharded_totals


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_deals_every_domain_once_and_balances(world):
    nx, ny, _, _, _ = batched_workload(64, 3)
    parts = partition(nx, ny, world)
    assert len(parts) == world
    got = np.sort(np.concatenate(parts))
    np.testing.assert_array_equal(got, np.arange(64))
    cells = nx.astype(np.int64) * ny
    loads = np.array([cells[p].sum() for p in parts])
    assert loads.max() <= cells.sum() / world + cells.max()  # the LPT bound
    assert all(np.all(np.diff(p) > 0) for p in parts)
    assert [list(p) for p in partition(nx, ny, world)] == [list(p) for p in parts]  # deterministic


def test_partition_examples():
    # cells 8, 7, 6, 5, 4 (rank loads before each deal in brackets): 8 -> rank 0 (0, 0: tie to
    # the lower rank); 7 -> rank 1 (8, 0); 6 -> rank 1 (8, 7); 5 -> rank 0 (8, 13); 4 -> rank 0 (13, 13)
    nx = np.array([8, 7, 6, 5, 4])
    ny = np.ones(5, np.int64)
    p = partition(nx, ny, 2)
    assert [list(a) for a in p] == [[0, 3, 4], [1, 2]]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(100 + rank)
        local = rng.standard_normal((5 + rank, 3)) * 1e3
        np.save(os.path.join(out_dir, "local%d.npy" % rank), local)
        np.save(os.path.join(out_dir, "total%d.npy" % rank), sharded_totals(local, dist))
    finally:
        dist.destroy_process_group()


def test_sharded_totals_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    want = np.zeros(3)
    for r in range(2):
        want = want + np.load(tmp_path / ("local%d.npy" % r)).sum(axis=0)  # rank order
    for r in range(2):
        np.testing.assert_array_equal(np.load(tmp_path / ("total%d.npy" % r)), want)
    np.testing.assert_array_equal(sharded_totals(np.load(tmp_path / "local0.npy")),
                                  np.load(tmp_path / "local0.npy").sum(axis=0))
