"""Body setup on the device (rbx_upload_state_device) against the host setup (rbx_upload_state).

Both run the arithmetic of csrc/rbx_setup.cuh (the device build without FP contraction), so fed
the same positions and velocities -- those the device reads from posq (+ correction) and velm --
they give the same body state, moments and body-frame coordinates bit for bit, for asymmetric,
symmetric, spherical and linear bodies, and trajectories that stay identical, including across an
atom reordering (which fetches the device geometry back to the host and re-plans)."""
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


def _systems(golden):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    m = W.mixed_system(n_bodies=1500, n_free=120, seed=17)
    g = golden("linear10_mode10")
    lin = type("S", (), dict(masses=g["masses"], body_indices=g["body_indices"], positions=g["R0"],
                             velocities=g["V0"], num_atoms=len(g["masses"])))()
    return {"mixed": m, "linear": lin}


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
@pytest.mark.parametrize("name", ["mixed", "linear"])
def test_device_setup_equals_host_setup(rbx, golden, prec, name):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = _systems(golden)[name]
    F = W.gaussian_forces(s.num_atoms, seed=2, sd=50.0)
    runs = []
    for where in ("host", "device"):
        k = rbx.IntegratorKernel(s.masses, s.body_indices, rotation_mode=0 if name == "mixed" else 10, precision=prec)
        buf = rbx.DeviceBuffers(s.num_atoms, precision=prec)
        buf.set_positions(s.positions)
        buf.set_velocities(s.velocities, s.masses)
        buf.set_forces(F)
        if where == "host":
            k.upload_state(buf.get_positions(), buf.get_velocities())  # what the device sees
        else:
            k.upload_state_device(buf)
        runs.append((k, buf))
    (kh, bh), (kd, bd) = runs
    assert kd.num_dof == kh.num_dof
    assert np.array_equal(kd.body_state(), kh.body_state())
    Ih, dh = kh.geometry()
    Id, dd = kd.geometry()
    assert np.array_equal(Id, Ih)
    if prec == "double":
        assert np.array_equal(dd, dh)
    else:  # the device keeps d in FP32; its host copy is read back from there
        assert np.array_equal(dd, dh.astype(np.float32).astype(np.float64))
    perm = np.random.default_rng(5).permutation(s.num_atoms)
    for n in range(12):
        if n == 6:  # reordering after a device setup: the geometry comes back to the host first
            for k, b in runs:
                b.relocate(perm)
                k.set_atom_locations(perm)
        for k, b in runs:
            k.part1(b, 0.002)
            k.part2(b, 0.002)
    assert np.array_equal(bd.get_positions(), bh.get_positions())
    assert np.array_equal(bd.get_velocities(), bh.get_velocities())
    assert np.array_equal(kd.body_state(), kh.body_state())
