"""Invariants of the integrator that hold whatever the reference does, on the CUDA path.

The bounds below sit above values measured on a GB300 (in brackets), with margin:
  free rotation of 512 waters, exact rotation (mode 0), 1000 steps of 2 fs, no forces:
    relative change of the total kinetic energy   double 1e-13, mixed 1e-7 [1.3e-8]
                                                  (double: the increment-form exact rotation; 4e-14
                                                  for 512 such bodies in FP64 on the host)
    | |q| - 1 |                                   double 1e-13 [2e-16], mixed 1e-12 [4e-15]
    relative change of intra-body distances       double 1e-12 [5e-15], mixed 1e-6 [1.6e-7],
                                                  single 1e-5 [2.9e-6] (positions in FP32)
  NO-SQUISH with n substeps: the kinetic-energy error of free rotation is O((dt/n)^2), so
    halving the substep (n = 5 -> 10) divides the largest excursion by about 4
  time reversibility: 100 steps of +dt then 100 of -dt under fixed forces return the body
    state and atom positions to their start (double: rounding only; mixed: FP32 increments)
  degrees of freedom: 6 per non-linear body, 5 per linear body, 3 per free atom
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rbx():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import build, kernel
    build.build_library()
    return kernel


def make(rbx, s, mode, prec, F=None):
    k = rbx.IntegratorKernel(s.masses, s.body_indices, rotation_mode=mode, precision=prec)
    buf = rbx.DeviceBuffers(s.num_atoms, precision=prec)
    buf.set_positions(s.positions)
    buf.set_velocities(s.velocities, s.masses)
    buf.set_forces(np.zeros((s.num_atoms, 3)) if F is None else F)
    k.upload_state(s.positions, s.velocities)
    return k, buf


def body_distances(k, R):
    first, atoms = k.body_atoms()
    out = []
    for b in range(k.num_bodies):
        a = atoms[first[b]:first[b + 1]]
        i, j = np.triu_indices(len(a), 1)
        out.append(np.linalg.norm(R[a[i]] - R[a[j]], axis=1))
    return np.concatenate(out)


@pytest.fixture(scope="module")
def waters():
    from openmm_rigidbody_plugin_gb300 import workloads as W
    return W.water_box(512, seed=1)


@pytest.mark.parametrize("prec,tol_ke,tol_q,tol_d", [("double", 1e-13, 1e-13, 1e-12), ("mixed", 1e-7, 1e-12, 1e-6),
                                                     ("single", 1e-7, 1e-12, 1e-5)])
def test_free_rotation_conserves_energy_norm_and_shape(rbx, waters, prec, tol_ke, tol_q, tol_d):
    s = waters
    k, buf = make(rbx, s, 0, prec)
    ke0 = sum(k.kinetic_energies(buf))
    for _ in range(1000):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
    assert abs(sum(k.kinetic_energies(buf)) - ke0) / ke0 < tol_ke
    q = k.body_state()[:, 6:10]
    assert np.max(np.abs(np.linalg.norm(q, axis=1) - 1.0)) < tol_q
    d0 = body_distances(k, s.positions)
    assert np.max(np.abs(body_distances(k, buf.get_positions()) - d0) / d0) < tol_d


def test_nosquish_energy_error_is_second_order(rbx, waters):
    excursion = {}
    for n in (5, 10):
        k, buf = make(rbx, waters, n, "double")
        ke0 = sum(k.kinetic_energies(buf))
        worst = 0.0
        for step in range(400):
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
            if step % 20 == 19:
                worst = max(worst, abs(sum(k.kinetic_energies(buf)) - ke0) / ke0)
        excursion[n] = worst
    ratio = excursion[5] / excursion[10]
    assert 2.5 < ratio < 6.5, excursion


@pytest.mark.parametrize("prec,tol", [("double", 1e-9), ("mixed", 2e-6)])
@pytest.mark.parametrize("mode", [0, 10])
def test_time_reversibility(rbx, prec, tol, mode):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=2000, n_free=200, seed=11)
    F = W.gaussian_forces(s.num_atoms, seed=3, sd=50.0)
    k, buf = make(rbx, s, mode, prec, F)
    state0 = k.body_state()
    for dt in (0.002, -0.002):
        for _ in range(100):
            k.part1(buf, dt)
            k.part2(buf, dt)
    R = buf.get_positions()
    assert np.max(np.abs(R - s.positions)) / np.max(np.abs(s.positions)) < tol
    state = k.body_state()
    for cols in (slice(0, 3), slice(3, 6), slice(6, 10), slice(10, 14)):  # r, v, q, pi
        ref = state0[:, cols]
        assert np.max(np.abs(state[:, cols] - ref)) / np.max(np.abs(ref)) < 10 * tol


def test_degrees_of_freedom(rbx, golden):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    g = golden("linear10_mode10")
    k, _ = make(rbx, type("S", (), dict(masses=g["masses"], body_indices=g["body_indices"], positions=g["R0"],
                                        velocities=g["V0"], num_atoms=len(g["masses"])))(), 10, "mixed")
    assert k.num_dof == 5 * 10 == int(g["dof"])
    s = W.mixed_system(n_bodies=500, n_free=70, seed=2)
    k, _ = make(rbx, s, 0, "mixed")
    assert k.num_dof == 6 * 500 + 3 * 70
