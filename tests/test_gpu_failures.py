"""Failure detection on the device, tested by planting the failure on the host (no GPU fault).

The reference lets NaN through silently (openmmapi/include/internal/ellipticFunctions.h:38-39,
:64-66). Here every step kernel checks each body's and free atom's new state, and the batched force
kernel checks each force against OpenMM's fixed-point range:
  * a single handle reports flagged bodies and free atoms through rbx_check_state;
  * a batch reports each failed system through rbx_batch_status, and its other systems go on
    bit for bit as they would without the failed one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rbx():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import batch, build, kernel
    build.build_library()
    return kernel, batch


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
def test_non_finite_body_state_is_flagged(rbx, prec):
    kernel, _ = rbx
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=400, n_free=30, seed=5)
    k = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=0, precision=prec)
    buf = kernel.DeviceBuffers(s.num_atoms, precision=prec)
    buf.set_positions(s.positions)
    buf.set_velocities(s.velocities, s.masses)
    buf.set_forces(W.gaussian_forces(s.num_atoms, seed=2, sd=50.0))
    k.upload_state(s.positions, s.velocities)
    for _ in range(3):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
    assert k.check_state() == (0, 0)
    state = k.body_state()
    state[17, 10] = np.nan   # the quaternion momentum of body 17
    state[250, 4] = np.inf   # the COM velocity of body 250
    k.set_body_state(state)
    assert k.check_state() == (0, 0)  # a new state clears the detector
    k.part1(buf, 0.002)
    k.part2(buf, 0.002)
    nb, nf = k.check_state()
    assert nb == 2 and nf == 0
    from openmm_rigidbody_plugin_gb300 import _lib
    with pytest.raises(_lib.RbxError, match="first: body 17"):
        _lib.check(k._lib.rbx_check_state(k._h, None, None, None))
    k.upload_state(s.positions, s.velocities)
    assert k.check_state() == (0, 0)


def test_non_finite_free_atom_is_flagged(rbx):
    kernel, _ = rbx
    import torch
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=100, n_free=50, seed=6)
    k = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=0, precision="mixed")
    buf = kernel.DeviceBuffers(s.num_atoms, precision="mixed")
    buf.set_positions(s.positions)
    buf.set_velocities(s.velocities, s.masses)
    k.upload_state(s.positions, s.velocities)
    free = np.flatnonzero(np.asarray(s.body_indices) == 0)
    buf.velm[int(buf.location[free[7]]), 1] = float("nan")  # one free atom's velocity
    torch.cuda.synchronize()
    k.part1(buf, 0.002)
    k.part2(buf, 0.002)
    assert k.check_state() == (0, 1)


def _batch_of(batch, systems, overlap=None):
    """The systems, set up twice (the second time from the positions and velocities the first set-up
    gives back), so that a run with and a run without a planted overlap share the same history."""
    b = batch.BatchedSystems.from_systems(systems)
    x, v = b.get_state()
    if overlap is not None:  # two atoms of different molecules put on top of each other
        a, c = overlap
        x[c] = x[a] + 1e-4
    b.set_state(x, v)
    return b


def test_failed_system_is_reported_and_the_others_are_unchanged(rbx):
    _, batch = rbx
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = [W.water_box(64, seed=s) for s in (1, 2, 3)]
    ref = _batch_of(batch, systems)
    ref.step(30, 0.002)
    assert not ref.status().any()
    # the same three systems, the middle one with two oxygens of different waters 1e-4 nm apart:
    # its forces leave the fixed-point range at the first evaluation
    off = 64 * 3
    bad = _batch_of(batch, systems, overlap=(off + 0, off + 3))
    bad.step(30, 0.002)
    st = bad.status()
    assert list(st) == [0, 5, 0]
    x_ref, v_ref = ref.get_state()
    x_bad, v_bad = bad.get_state()
    for k in (0, 2):
        sl = slice(64 * 3 * k, 64 * 3 * (k + 1))
        assert np.array_equal(x_bad[sl], x_ref[sl]) and np.array_equal(v_bad[sl], v_ref[sl])
    e_ref, e_bad = ref.energies(), bad.energies()
    assert np.array_equal(e_bad[[0, 2]], e_ref[[0, 2]])


def test_non_finite_restored_state_fails_only_its_system(rbx):
    _, batch = rbx
    from openmm_rigidbody_plugin_gb300 import workloads as W
    systems = [W.water_box(27, seed=s) for s in (4, 5, 6, 7)]
    ref = _batch_of(batch, systems)
    b = _batch_of(batch, systems)
    states = b.checkpoint()
    body, x, v = states[3]
    body = body.copy()
    body.view(np.float32)[5, 11] = np.nan  # pi.x of body 5, high word (mixed precision)
    states[3] = (body, x, v)
    b.restore(states)
    assert not b.status().any()
    b.step(10, 0.002)
    ref.step(10, 0.002)
    assert list(b.status()) == [0, 0, 0, 5]
    xr, vr = ref.get_state()
    xb, vb = b.get_state()
    n = 3 * 27 * 3
    assert np.array_equal(xb[:n], xr[:n]) and np.array_equal(vb[:n], vr[:n])
