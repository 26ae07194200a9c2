"""Constraints between free atoms on the CPU: the Context stand-in's SHAKE / RATTLE solvers and
the oracle's constrained step (ReferenceRigidBodyKernels.cpp:82-108), which the GPU paths are
compared with in test_gpu_constraints.py."""
import numpy as np

from conftest import constrained_system, oracle_constrained_run
from openmm_rigidbody_plugin_gb300.api import rattle_velocities, shake


def test_shake_and_rattle_enforce_the_bonds():
    rng = np.random.default_rng(0)
    x_old = rng.normal(size=(6, 3))
    pairs = np.array([[0, 1], [2, 3], [4, 5]])
    d = np.linalg.norm(x_old[pairs[:, 0]] - x_old[pairs[:, 1]], axis=1)
    x = x_old + 0.01 * rng.normal(size=x_old.shape)
    w = 1.0 / rng.uniform(1, 16, 6)
    xc = shake(x_old, x, w, pairs, d, 1e-10)
    np.testing.assert_allclose(np.linalg.norm(xc[pairs[:, 0]] - xc[pairs[:, 1]], axis=1), d, rtol=1e-9)
    # the centre of mass of each pair does not move (corrections are along the bond, mass-weighted)
    m = 1.0 / w
    com = lambda y: (m[pairs[:, 0], None] * y[pairs[:, 0]] + m[pairs[:, 1], None] * y[pairs[:, 1]])
    np.testing.assert_allclose(com(xc), com(x), atol=1e-12)
    v = rattle_velocities(xc, rng.normal(size=(6, 3)), w, pairs, 1e-12)
    rij = xc[pairs[:, 0]] - xc[pairs[:, 1]]
    vij = v[pairs[:, 0]] - v[pairs[:, 1]]
    assert np.max(np.abs(np.einsum("ij,ij->i", rij, vij))) < 1e-10


def test_constrained_oracle_run_keeps_bonds_and_energy():
    import oracle as oracle_mod
    sysc = constrained_system()
    masses, bidx, x0, v0, force, pairs, dist = sysc
    # energy after the first step (the setup projects body-atom velocities onto rigid motion)
    o = oracle_constrained_run(oracle_mod, sysc, 0.001, 1)
    e0 = force(o.R)[1] + o.kinetic().sum()
    o = oracle_constrained_run(oracle_mod, sysc, 0.001, 200)
    r = np.linalg.norm(o.R[pairs[:, 0]] - o.R[pairs[:, 1]], axis=1)
    np.testing.assert_allclose(r, dist, rtol=2e-5)
    # the energy of the constrained system stays within the velocity-Verlet fluctuation
    e1 = force(o.R)[1] + o.kinetic().sum()
    assert abs(e1 - e0) < 1e-3 * e0, (e0, e1)
