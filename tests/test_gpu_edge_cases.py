"""Atom classes at the edges of RigidBodySystem::initialize (RigidBodySystem.cpp:23-49, :71-105)
on the GPU, against the robust FP64 oracle:
  * massless free atoms (OpenMM's virtual sites) are not integrated: position and velocity stay
    as they were (the counts skip them, :73-80);
  * a body index used by one atom only makes that atom free, as the comment at :23-26 intends (the
    reference code keeps a one-atom body with 6 DOF and zero inertia, defect D5);
  * degrees of freedom: 6 per body, 3 per integrated free atom.
Tolerances as the other oracle comparisons: positions 1e-9 (double), 1e-6 (mixed), 2e-4 (single),
velocities 10x those, after 20 steps under seeded sd 50 kJ/mol/nm forces.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-9, "mixed": 1e-6, "single": 2e-4}


@pytest.fixture(scope="module")
def rbx():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import build, kernel
    build.build_library()
    return kernel


def _edge_system():
    """27 waters, 4 free argon atoms, 2 massless atoms and 3 atoms whose body ids are used once."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    rng = np.random.default_rng(44)
    w = W.water_box(27, seed=5)
    nid = int(w.body_indices.max())
    masses = np.concatenate([w.masses, np.full(4, 39.95), np.zeros(2), np.array([12.0, 14.0, 16.0])])
    bidx = np.concatenate([w.body_indices, np.zeros(4, int), np.zeros(2, int), nid + 1 + np.arange(3) * 5])
    R = np.concatenate([w.positions, rng.uniform(0, 2.5, (9, 3))])
    V = np.concatenate([w.velocities, rng.normal(0, 0.5, (9, 3))])
    F = np.round(W.gaussian_forces(len(masses), seed=9, sd=50.0) * 2.0 ** 32) / 2.0 ** 32
    return masses, bidx, R, V, F


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
@pytest.mark.parametrize("mode", [0, 10])
def test_massless_and_singleton_atoms_vs_robust_oracle(rbx, oracle_mod, prec, mode):
    masses, bidx, R, V, F = _edge_system()
    k = rbx.IntegratorKernel(masses, bidx, rotation_mode=mode, precision=prec)
    buf = rbx.DeviceBuffers(len(masses), precision=prec)
    buf.set_positions(R)
    buf.set_velocities(V, masses)
    k.upload_state(R, V)
    buf.set_forces(F)
    o = oracle_mod.Oracle(masses, bidx, mode=mode, robust=True)
    o.setup(R, V, F)
    assert k.num_dof == o.num_dof == 6 * 27 + 3 * (4 + 3)
    for _ in range(20):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
        o.part1(0.002, F)
        o.part2(0.002, F)
    x, v = buf.get_positions(), buf.get_velocities()
    live = masses > 0
    assert rel_err(x[live], o.R[live]) < TOL[prec]
    assert rel_err(v[live], o.V[live]) < 10 * TOL[prec]
    stored = 1e-6 if prec == "single" else 1e-12  # FP32 storage of the untouched values in single
    assert np.abs(x[~live] - R[~live]).max() < stored
    assert np.abs(v[~live] - V[~live]).max() < stored
