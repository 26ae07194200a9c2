"""The API mirror driving the library on the GPU: RigidBodyIntegrator.step on a Context with
position-dependent forces reproduces the reference's own trajectory (golden tethered waters,
computed by the reference's CPU code), with the tolerances of test_gpu_parity.py; binding rules
follow RigidBodyIntegrator.cpp:26-46."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import api, build
    build.build_library()
    return api


@pytest.mark.parametrize("prec,tol_x,tol_v", [("double", 1e-9, 1e-8), ("mixed", 1e-6, 5e-6)])
@pytest.mark.parametrize("mode", [0, 4])
def test_integrator_step_reproduces_reference_tethers(api, golden, mode, prec, tol_x, tol_v):
    g = golden(f"water27_tether_mode{mode}")
    R0, k = g["R0"], float(g["k"])
    intg = api.RigidBodyIntegrator(float(g["dt"]), g["body_indices"])
    intg.setRotationMode(int(g["mode"]))
    ctx = api.Context(api.System(g["masses"]), intg, lambda R: (-k * (R - R0), 0.5 * k * np.sum((R - R0) ** 2)),
                      precision=prec)
    ctx.setPositions(R0)
    ctx.setVelocities(g["V0"])
    assert intg.getRigidBodySystem().getNumDOF() == int(g["dof"])  # waters only: no free atoms
    for block in range(len(g["R"])):
        intg.step(10)
    st = ctx.getState(getPositions=True, getVelocities=True, getEnergy=True)
    assert rel_err(st.getPositions(), g["R"][-1]) < tol_x
    assert rel_err(st.getVelocities(), g["V"][-1]) < tol_v
    np.testing.assert_allclose(intg.getKineticEnergies(), g["energy"][-1][1:], rtol=10 * tol_v)
    np.testing.assert_allclose(st.getPotentialEnergy(), g["energy"][-1][0], rtol=10 * tol_v)


def test_binding_rules(api):
    intg = api.RigidBodyIntegrator(0.002, [1, 1, 1, 0])
    ctx = api.Context(api.System([16.0, 1.0, 1.0, 40.0]), intg, lambda R: (np.zeros_like(R), 0.0))
    with pytest.raises(api.OpenMMException, match="already bound"):
        intg.setRotationMode(2)
    with pytest.raises(api.OpenMMException, match="already bound"):
        api.Context(api.System([16.0, 1.0, 1.0, 40.0]), intg, lambda R: (np.zeros_like(R), 0.0))
    with pytest.raises(api.OpenMMException, match="differs"):
        api.Context(api.System([16.0, 1.0]), api.RigidBodyIntegrator(0.002, [1, 1, 1]), lambda R: (R, 0.0))
    del ctx
