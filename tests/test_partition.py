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


def _oracle_energies(systems, nsteps=4, dt=0.002):
    """[U, KE_t, KE_r] of each system after nsteps full steps of the FP64 oracle (robust integrator
    and all-pairs cutoff LJ + reaction-field forces), one thread."""
    import oracle
    from openmm_rigidbody_plugin_gb300 import workloads as W
    out = []
    for s in systems:
        q, sg, ep = W.nonbonded(s)
        rc = W.cutoff_for(s.box)

        def force(R):
            f, e = oracle.lj_rf([0, s.num_atoms], [s.box], [rc], R, q, sg, ep, s.body_indices, nthreads=1)
            return f, float(e[0])

        o = oracle.Oracle(s.masses, s.body_indices, mode=0, robust=True)
        o.setup(s.positions, s.velocities, force(s.positions)[0])
        for _ in range(nsteps):
            o.part1(dt, force(o.R)[0])
            o.part2(dt, force(o.R)[0])
        out.append([force(o.R)[1], *o.kinetic()])
    return np.array(out)


def _rank_oracle(rank, world, port, result_path):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    from openmm_rigidbody_plugin_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        counts = W.batch_body_counts(6, lo=20, hi=60, seed=9)
        mine = partition.local_systems(counts, world, rank)
        systems = W.batch_systems(6, lo=20, hi=60, seed=9, only=mine)
        rows = partition.gather_by_system(_oracle_energies(systems), mine, len(counts))
        if rank == 0:
            np.save(result_path, rows)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_gloo_two_ranks_integrate_their_partitions_like_one_rank(tmp_path, oracle_mod):
    """The batched workload split by assign_systems over two gloo ranks, each rank integrating its
    own systems (the FP64 oracle's full steps): the per-system energies gathered in system order
    equal a single-rank run of all systems bit for bit."""
    import torch.multiprocessing as mp
    from openmm_rigidbody_plugin_gb300 import workloads as W
    out = str(tmp_path / "energies.npy")
    mp.start_processes(_rank_oracle, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    together = _oracle_energies(W.batch_systems(6, lo=20, hi=60, seed=9))
    assert np.array_equal(np.load(out), together)
