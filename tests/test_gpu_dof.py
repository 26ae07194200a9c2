"""Degree-of-freedom counts through the C ABI: rbx_get_num_dof_reference reports the reference's
own integer (openmmapi/src/RigidBodySystem.cpp:130), bit for bit, for every golden vector the
reference produced, after a host state upload and after a device-side one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDENS_WITH_DOF = ["water64_mode0", "water64_sd50_mode10", "water27_tether_mode0", "linear10_mode10",
                    "cross48_mode0_dt1fs", "cross48_mode16_dt4fs"]


@pytest.fixture(scope="module")
def rbx():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import build, kernel
    build.build_library()
    return kernel


def counts(rbx, masses, bidx, R, V, device_setup, prec="mixed"):
    k = rbx.IntegratorKernel(masses, bidx, rotation_mode=0, precision=prec)
    if device_setup:
        buf = rbx.DeviceBuffers(len(masses), precision=prec)
        buf.set_positions(R)
        buf.set_velocities(V, masses)
        k.upload_state_device(buf)
    else:
        k.upload_state(R, V)
    return k.num_dof, k.num_dof_reference, k


@pytest.mark.parametrize("device_setup", [False, True])
@pytest.mark.parametrize("name", GOLDENS_WITH_DOF)
def test_reference_count_equals_golden(rbx, golden, name, device_setup):
    g = golden(name)
    nd, ref, k = counts(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], device_setup)
    assert ref == int(g["dof"])
    assert nd == ref + 2 * k.num_free  # the library counts three per free atom


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
@pytest.mark.parametrize("device_setup", [False, True])
def test_reference_count_with_one_atom_bodies(rbx, golden, prec, device_setup):
    """Unique body indices (one-atom bodies in the reference, 5 or 6 DOF each by the rounding of its
    centre-of-mass arithmetic), a linear body, free and massless atoms."""
    g = golden("singleton_dof")
    off = g["offsets"]
    for c in range(len(off) - 1):
        a, b = off[c], off[c + 1]
        _, ref, _ = counts(rbx, g["masses"][a:b], g["body_indices"][a:b], g["R0"][a:b], g["V0"][a:b], device_setup,
                           prec)
        if prec == "double" or not device_setup:
            assert ref == int(g["dof"][c])
        else:  # device positions rounded to FP32 (single) or float pairs (mixed): still 5 or 6 per atom
            assert abs(ref - int(g["dof"][c])) <= np.count_nonzero(np.bincount(g["body_indices"][a:b])[1:] == 1)
