"""The benchmark workload at its full size: 1,000,000 bodies (70 % 3-site waters, 20 % 5-atom
tetrahedra, 10 % 12-atom rings) and 100,000 free atoms, seeded sd 500 kJ/mol/nm forces, mixed
precision, rotation mode 0, 2 fs steps (part1, 19 fused steps, part2). The FP64 oracle is too slow
to follow the whole system, so it follows a sample: under fixed forces every body and free atom
moves independently, so 1000 bodies and 100 free atoms drawn at random from the full run are
stepped by the robust oracle on their own and compared with the device's positions and
velocities of the same atoms (mixed-precision bounds of the sd 500 kJ/mol/nm parity tests at 20
steps: positions 1e-6, velocities 3e-6 relative). The other tests check properties that hold at
every size:
  * bitwise determinism: two independent handles give identical positions, velocities, body
    states and kinetic energies (fixed-order reductions, no atomics);
  * rigidity: every body atom keeps its distance to its body's first atom. Bound 2e-6 nm: the
    rebuild r + At(q) d rounds d and At(q) to FP32, about 1e-7 nm on these bodies;
  * unit quaternions: ||q| - 1| < 1e-6 (q is renormalised every step in float-float);
  * translational kinetic energy: the device's fixed-order FP64 sum equals a host sum over the body
    state and the free atoms' velocities to 1e-9 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 0.002
STEPS = 20


@pytest.fixture(scope="module")
def full():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import build, kernel
    from openmm_rigidbody_plugin_gb300 import workloads as W
    build.build_library()
    s = W.mixed_system(n_bodies=1_000_000, n_free=100_000, seed=3)
    F = W.gaussian_forces(s.num_atoms, seed=5)

    def run():
        k = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=0, precision="mixed")
        buf = kernel.DeviceBuffers(s.num_atoms, precision="mixed")
        buf.set_positions(s.positions)
        buf.set_velocities(s.velocities, s.masses)
        buf.set_forces(F)
        k.upload_state(s.positions, s.velocities)
        k.part1(buf, DT)
        for _ in range(STEPS - 1):
            k.fused(buf, DT)
        k.part2(buf, DT)
        torch.cuda.synchronize()
        return k, buf

    k, buf = run()
    out = {"s": s, "F": F, "k": k, "x": buf.get_positions(), "v": buf.get_velocities(), "state": k.body_state(),
           "ke": k.kinetic_energies(buf)}
    k2, buf2 = run()
    out["again"] = (buf2.get_positions(), buf2.get_velocities(), k2.body_state(), k2.kinetic_energies(buf2))
    return out


def test_full_size_is_bitwise_deterministic(full):
    x, v, state, ke = full["again"]
    assert np.array_equal(x, full["x"])
    assert np.array_equal(v, full["v"])
    assert np.array_equal(state, full["state"])
    assert np.array_equal(ke, full["ke"])


def test_full_size_bodies_stay_rigid(full):
    s, k = full["s"], full["k"]
    first, atoms = k.body_atoms()
    assert k.num_bodies == 1_000_000 and len(atoms) == 4_300_000
    owner = np.repeat(np.arange(k.num_bodies), np.diff(first))
    anchor = atoms[first[owner]]
    d0 = np.linalg.norm(s.positions[atoms] - s.positions[anchor], axis=1)
    d1 = np.linalg.norm(full["x"][atoms] - full["x"][anchor], axis=1)
    assert np.abs(d1 - d0).max() < 2e-6
    assert np.isfinite(full["x"]).all() and np.isfinite(full["v"]).all()


def test_full_size_quaternions_stay_unit(full):
    q = full["state"][:, 6:10]
    assert np.abs(np.linalg.norm(q, axis=1) - 1.0).max() < 1e-6


def test_full_size_translational_kinetic_energy(full):
    s, k, state = full["s"], full["k"], full["state"]
    first, atoms = k.body_atoms()
    body_mass = np.add.reduceat(np.asarray(s.masses)[atoms], first[:-1])
    free = (np.asarray(s.body_indices) <= 0) & (np.asarray(s.masses) > 0)
    assert free.sum() == k.num_free == 100_000
    vb = state[:, 3:6]
    ke_t = 0.5 * np.sum(body_mass * np.sum(vb * vb, axis=1)) + \
        0.5 * np.sum(np.asarray(s.masses)[free] * np.sum(full["v"][free] ** 2, axis=1))
    assert abs(full["ke"][0] - ke_t) <= 1e-9 * ke_t


def test_full_size_sample_vs_robust_oracle(full, oracle_mod):
    from conftest import rel_err
    s, k = full["s"], full["k"]
    first, atoms = k.body_atoms()
    rng = np.random.default_rng(77)
    picked = np.sort(rng.choice(k.num_bodies, size=1000, replace=False))
    body_atoms = np.concatenate([atoms[first[b]:first[b + 1]] for b in picked])
    free = np.flatnonzero(np.asarray(s.body_indices) <= 0)
    sample = np.concatenate([body_atoms, np.sort(rng.choice(free, size=100, replace=False))])
    F = np.round(full["F"][sample] * 2.0 ** 32) / 2.0 ** 32  # the device's fixed-point forces
    o = oracle_mod.Oracle(np.asarray(s.masses)[sample], np.asarray(s.body_indices)[sample], mode=0, robust=True)
    o.setup(s.positions[sample], s.velocities[sample], F)
    assert o.num_bodies == 1000 and o.num_free == 100
    for _ in range(STEPS):
        o.part1(DT, F)
        o.part2(DT, F)
    ex, ev = rel_err(full["x"][sample], o.R), rel_err(full["v"][sample], o.V)
    assert ex < 1e-6 and ev < 3e-6, f"positions {ex:.3e}, velocities {ev:.3e}"
