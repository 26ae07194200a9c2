"""Checkpoint/restore and continuous batching on the GPU.

A batch rebuilt from its systems' original structures and restored from a checkpoint continues
bit for bit as if it had never stopped. The server admits requests as the memory budget frees up,
so batch membership changes while systems are in flight; every served request must equal the same
request run alone with the same chunk boundaries, bit for bit (a chunk boundary ends a step with
part2 and starts the next with part1 instead of the fused kernel, so the chunking is part of the
trajectory's rounding).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import batch, build, serving
    from openmm_rigidbody_plugin_gb300 import workloads as W
    build.build_library()
    return batch, serving, W


@pytest.mark.parametrize("precision", ["mixed", "double"])
def test_checkpoint_restore_is_exact(mods, precision):
    batch, _, W = mods
    # both batches are set up from the same structures (they fix each body's frame)
    systems = [W.water_box(64, seed=3), W.water_box(125, seed=4), W.mixed_system(n_bodies=300, n_free=40, seed=5)]
    a = batch.BatchedSystems.from_systems(systems, precision=precision)
    a.step(25, 0.002)
    ckpt = a.checkpoint()
    b = batch.BatchedSystems.from_systems(systems, precision=precision)
    b.restore(ckpt)
    # the body rows are the device words: every float-float low word comes back as it was
    for (ra, _, _), (rb, _, _) in zip(ckpt, b.checkpoint()):
        assert ra.shape[1] == 112 and np.array_equal(ra, rb)
    for h in (a, b):
        h.step(20, 0.002)
    for u, w in zip(a.get_state(), b.get_state()):
        assert np.array_equal(u, w)
    assert np.array_equal(a.energies(), b.energies())


def test_served_requests_equal_requests_alone(mods):
    batch, serving, W = mods
    reqs = []
    for rid, (nw, steps) in enumerate([(20, 130), (150, 40), (60, 95), (210, 70), (40, 60), (90, 120)]):
        reqs.append(serving.Request(rid, W.water_box(nw, seed=100 + rid), steps, arrival=0.0))
    atoms = [r.num_atoms for r in reqs]
    # a budget that holds the largest request and two small ones at the largest bytes per atom the
    # server can measure (a batch of all the requests: its neighbour lists are sized for the largest),
    # so requests join as others finish
    bpa = 0.0
    for group in [reqs] + [[r] for r in reqs]:
        probe = batch.BatchedSystems.from_systems([r.system for r in group])
        bpa = max(bpa, 1.05 * probe.memory_bytes / sum(r.num_atoms for r in group))
        del probe
    server = serving.Server(budget_bytes=bpa * (max(atoms) + 2 * min(atoms) + 200), reserve_bytes=0,
                            chunk_steps=25, graph_steps=10)
    done = server.run(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert server.groups_created >= 3  # groups formed while others were in flight
    assert server.peak_bytes <= server.budget_used
    for r in done:
        assert r.failed is None and sum(r.chunks) == r.steps
        alone = serving.serve_alone(r)
        assert np.array_equal(alone["positions"], r.result["positions"])
        assert np.array_equal(alone["velocities"], r.result["velocities"])
        assert np.array_equal(alone["energies"], r.result["energies"])


def test_memory_report_counts_the_neighbour_lists(mods):
    """rbx_batch_memory: the bytes a batch holds grow with its atoms (the neighbour lists dominate)."""
    batch, _, W = mods
    small = batch.BatchedSystems.from_systems([W.water_box(200, seed=1)])
    large = batch.BatchedSystems.from_systems([W.water_box(2000, seed=1)])
    assert 0 < small.memory_bytes < large.memory_bytes
    assert large.memory_bytes / (3 * 2000) > 200  # lists, state, cells: hundreds of bytes per atom
