"""Batched systems on the GPU: cell-list LJ + reaction-field forces against the FP64 oracle, the
batched step against the same systems stepped alone, and full-step energy conservation against
the FP64 oracle's own full steps.

Tolerances: forces are accumulated in FP32 from FP32 positions, so 99.9 % of the atoms are held to
a force error of 2e-5 of the largest force. The rest may hold a pair whose distance lies within
FP32 rounding of the cutoff, where FP32 and FP64 disagree on whether it counts: the reaction-field
force does not vanish at the cutoff (K q_i q_j (1/rc^2 - 2 k_rf rc), 0.76 kJ/mol/nm for an O-H
pair at 0.9 nm), so such an atom's force jumps by up to 2e-3 of the largest force. Pair energies are formed in FP32 and summed with compensation; the FP32 rounding of
the positions (about 2e-7 nm) moves a box's energy by about sqrt(N) |F| 2e-7, a random walk over
its atoms, so the bound is absolute, 1e-5 kJ/mol per atom plus 1e-6 relative (a missing pair or
a wrong exclusion moves it by more than 1 kJ/mol; measured: 2.3e-3 kJ/mol on 512 waters, 2.3e-2
on a relaxed 4286-atom mixed box). A system gives bit-identical results alone and in a batch: its
cell lists, pair sums and per-body integration do not depend on the other systems.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import batch, build
    build.build_library()
    return batch


def oracle_forces(oracle_mod, systems, pos):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    offs = np.concatenate([[0], np.cumsum([s.num_atoms for s in systems])])
    q, sg, ep = (np.concatenate(x) for x in zip(*(W.nonbonded(s) for s in systems)))
    body = np.concatenate([s.body_indices + 100000 * i * (s.body_indices > 0) for i, s in enumerate(systems)])
    return oracle_mod.lj_rf(offs, [s.box for s in systems], [W.cutoff_for(s.box) for s in systems], pos, q, sg, ep,
                            body)


def merged_waters(W, seed):
    """A mixed box in which the 15 waters nearest one point form one rigid 45-atom body and the 40
    nearest another point one 120-atom body: groups larger than a warp pass and than the step
    kernel's per-thread sums, whose radii make the list cells large."""
    s = W.mixed_system(n_bodies=3000, n_free=300, seed=seed)
    bidx = s.body_indices.copy()
    ids, counts = np.unique(bidx[bidx > 0], return_counts=True)
    waters = ids[counts == 3]
    centre = {i: s.positions[bidx == i].mean(axis=0) for i in waters}
    free_id = bidx.max() + 1
    for n, point in ((15, 0.25 * s.box), (40, 0.75 * s.box)):
        near = sorted((i for i in waters if (bidx == i).any()), key=lambda i: np.sum((centre[i] - point) ** 2))[:n]
        for i in near:
            bidx[bidx == i] = free_id
        free_id += 1
    s.body_indices = bidx
    return s


@pytest.mark.parametrize("case", ["water512_one_cell", "mixed_cells", "batch_of_8", "large_groups"])
def test_forces_and_energies_match_oracle(B, oracle_mod, case):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    if case == "water512_one_cell":
        systems = [W.water_box(512, seed=1)]          # 2.48 nm box: fewer than 3 cells per edge
    elif case == "mixed_cells":
        systems = [W.mixed_system(n_bodies=3000, n_free=300, seed=12)]  # 5 cells per edge
    elif case == "large_groups":
        systems = [merged_waters(W, 13), W.mixed_system(n_bodies=400, n_free=40, seed=14)]
    else:
        systems = W.batch_systems(8, lo=64, hi=1500, seed=9)
    # generated mixed structures overlap (lattice sites 0.34 nm apart): relax them first
    b = B.BatchedSystems.from_systems(systems, relax_steps=0 if case == "water512_one_cell" else 300)
    x, _ = b.get_state()
    f, e = b.forces()
    fo, eo = oracle_forces(oracle_mod, systems, x)
    err = np.linalg.norm(f - fo, axis=1) / np.max(np.abs(fo))
    assert np.quantile(err, 0.999) < 2e-5 and np.max(err) < 2e-3, (np.quantile(err, 0.999), np.max(err))
    natoms = np.array([s.num_atoms for s in systems])
    assert np.all(np.abs(e - eo) <= 1e-6 * np.abs(eo) + 1e-5 * natoms), (e, eo)


@pytest.mark.parametrize("large", [False, True])
def test_system_alone_equals_system_in_batch(B, large):
    """With `large`, one system holds rigid bodies of 45 and 120 atoms: the batch then runs the step
    kernel form that sums such bodies by a warp, while the other systems alone run the ordinary
    form; their trajectories are the same bit for bit."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = W.batch_systems(5, lo=64, hi=1200, seed=10)
    if large:
        systems = systems[:3] + [merged_waters(W, 15)]
    together = B.BatchedSystems.from_systems(systems, relax_steps=100)
    x0, v0 = together.get_state()
    together.set_state(x0, v0)  # both runs set up from the same positions (they fix the body frames)
    together.step(30, 0.002)
    x_all, v_all = together.get_state()
    e_all = together.energies()
    off = together.offsets
    for k, s in enumerate(systems):
        alone = B.BatchedSystems.from_systems([s])
        alone.set_state(x0[off[k]:off[k + 1]], v0[off[k]:off[k + 1]])
        alone.step(30, 0.002)
        x, v = alone.get_state()
        assert np.array_equal(x, x_all[off[k]:off[k + 1]])
        assert np.array_equal(v, v_all[off[k]:off[k + 1]])
        assert np.array_equal(alone.energies()[0], e_all[k])


def test_graph_replay_equals_direct_launches(B):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = W.batch_systems(6, lo=64, hi=800, seed=11)
    direct = B.BatchedSystems.from_systems(systems, relax_steps=100)
    graphed = B.BatchedSystems.from_systems(systems, relax_steps=100)
    graphed.set_graph_steps(8)
    for b in (direct, graphed):
        b.step(20, 0.002)
        b.step(17, 0.002)
    for a, c in zip(direct.get_state(), graphed.get_state()):
        assert np.array_equal(a, c)
    assert graphed.last_launch_count == direct.last_launch_count


def test_step_calls_keep_the_last_forces(B):
    """A step call that follows another starts from the forces that call ended with (one force
    evaluation per step); after a restore it forms them itself, from lists built at the same
    positions by the same kernels, so both runs stay equal bit for bit."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = W.batch_systems(4, lo=64, hi=600, seed=21)
    a = B.BatchedSystems.from_systems(systems, relax_steps=60)
    b = B.BatchedSystems.from_systems(systems, relax_steps=60)
    for h in (a, b):
        h.step(10, 0.002)
    first = a.last_launch_count
    ck = b.checkpoint()
    b.restore(ck)
    a.step(10, 0.002)
    kept = a.last_launch_count
    b.step(10, 0.002)
    formed = b.last_launch_count
    assert kept < formed == first
    for u, w in zip(a.get_state(), b.get_state()):
        assert np.array_equal(u, w)
    e_kept = a.energies()  # formed by the step's last evaluation
    assert np.array_equal(e_kept, b.energies())
    a.restore(a.checkpoint())
    assert np.array_equal(a.energies(), e_kept)  # formed afresh at the same state


def test_degrees_of_freedom_per_system(B):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = [W.mixed_system(n_bodies=200, n_free=13, seed=3), W.water_box(27, seed=2)]
    b = B.BatchedSystems.from_systems(systems)
    assert list(b.num_dof) == [6 * 200 + 3 * 13, 6 * 27]


def test_water_full_steps_track_the_fp64_oracle(B, oracle_mod):
    """512 rigid waters, cutoff LJ + reaction field, 2 fs steps in mixed precision against the FP64
    oracle's own full steps (oracle integrator + oracle forces) from the same relaxed, thermalised
    state: positions within 1e-5 after 10 steps and 1e-4 after 100, velocities within 1e-3 and
    1e-2 (measured after 100 steps: 1.0e-3 for velocities; liquid dynamics amplify the
    FP32 force rounding; with identical forces the integrator itself meets 1e-6 after 100 steps,
    test_gpu_parity.py), and an energy drift over 500 steps no worse than the FP64 run's. Both
    runs drift by about 16 kJ/mol here: the unshifted Lennard-Jones term jumps as pairs cross the
    cutoff (as with OpenMM's CutoffPeriodic method without a switching function); their
    instantaneous energies part by about 1 kJ/mol as the two chaotic trajectories separate."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.water_box(512, seed=1)
    q, sg, ep = W.nonbonded(s)
    rc = W.cutoff_for(s.box)
    b = B.BatchedSystems.from_systems([s], relax_steps=100)
    x0, v0 = b.get_state()
    o = oracle_mod.Oracle(s.masses, s.body_indices, mode=0, robust=True)

    def force(R):
        return oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], R, q, sg, ep, s.body_indices)

    o.setup(x0, v0, force(x0)[0])
    dt = 0.002
    e_gpu, e_orc = [], []
    done = 0
    for n in (10, 90, 100, 100, 100, 100):
        b.step(n, dt)
        for _ in range(n):
            o.part1(dt, force(o.R)[0])
            o.part2(dt, force(o.R)[0])
        done += n
        u, kt, kr = b.energies()[0]
        e_gpu.append(u + kt + kr)
        e_orc.append(force(o.R)[1][0] + sum(o.kinetic()))
        if done in (10, 100):
            x, v = b.get_state()
            tol = 1e-5 if done == 10 else 1e-4
            assert rel_err(x, o.R) < tol, (done, rel_err(x, o.R))
            assert rel_err(v, o.V) < 100 * tol, (done, rel_err(v, o.V))
    e_gpu, e_orc = np.array(e_gpu), np.array(e_orc)
    assert abs(e_gpu[0] - e_orc[0]) < 1e-5 * abs(e_orc[0])  # after 10 steps: same state
    drift_gpu, drift_orc = abs(e_gpu[-1] - e_gpu[0]), abs(e_orc[-1] - e_orc[0])
    assert drift_gpu <= 1.25 * drift_orc + 1.0, (e_gpu, e_orc)


def test_autotune_changes_no_result(B):
    """The autotuner times schedules on the batch and restores its state exactly; every tile shape of
    the step kernel, block size of the cell kernel and graph run length gives the same trajectory
    bit for bit."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = W.batch_systems(6, lo=300, hi=2500, seed=14)
    runs = []
    for how in ("plain", "autotuned", 64, 256, "narrow tiles"):
        b = B.BatchedSystems.from_systems(systems, relax_steps=50)
        x0, v0 = b.get_state()
        b.set_state(x0, v0)
        b.step(3, 0.002)
        if how == "autotuned":
            choice = b.autotune(0.002, trial_steps=2)
            assert choice["cell_threads"] in (64, 128, 256) and choice["graph_steps"] in (0, 10, 50)
            assert choice["tile_threads"] in (128, 256)
        elif how == "narrow tiles":
            assert b.tile_threads == 256
            b.tile_threads = 128
            assert b.tile_threads == 128
        elif how != "plain":
            b.set_tuning(how, 10)
        b.step(25, 0.002)
        runs.append((b.get_state(), b.energies()))
    for (x, v), e in runs[1:]:
        assert np.array_equal(x, runs[0][0][0]) and np.array_equal(v, runs[0][0][1])
        assert np.array_equal(e, runs[0][1])
