"""Replicas across ranks on the CPU (gloo, world size 2): every system is owned by exactly one rank,
the load is balanced, and per-system results gathered from the ranks come back in system order."""
import os
import socket

import numpy as np
import pytest

from openmm_rigidbody_plugin_gb300 import partition


def test_assignment_covers_and_balances():
    rng = np.random.default_rng(6)
    work = np.exp(rng.uniform(np.log(64), np.log(4096), size=4096))
    for world in (1, 2, 4, 8):
        owner, load = partition.assign_systems(work, world)
        assert set(np.unique(owner)) == set(range(world))
        assert np.isclose(load.sum(), work.sum())
        assert load.max() - load.min() <= work.max()  # LPT bound
        parts = [partition.local_systems(work, world, r) for r in range(world)]
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(len(work)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, work, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = partition.local_systems(work, world, rank)
        # stand-in per-system result: (system index, work, rank) as floats
        vals = np.stack([mine, work[mine], np.full(len(mine), rank)], axis=1)
        rows = partition.gather_by_system(vals, mine, len(work))
        if rank == 0:
            np.save(result_path, rows)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_gloo_two_ranks_gather_in_system_order(tmp_path):
    import torch.multiprocessing as mp
    work = np.arange(1, 41, dtype=np.float64)[::-1] * 3.0
    out = str(tmp_path / "rows.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), work, out), nprocs=2, join=True, start_method="spawn")
    rows = np.load(out)
    assert np.array_equal(rows[:, 0], np.arange(len(work)))
    assert np.array_equal(rows[:, 1], work)
    owner, _ = partition.assign_systems(work, 2)
    assert np.array_equal(rows[:, 2], owner)
