"""Constrained free atoms on the GPU against the oracle's constrained step (the Reference
platform's execute: part1, SHAKE, forces, part2 with its (R - savedPos)/dt velocity term, RATTLE;
ReferenceRigidBodyKernels.cpp:82-108, RigidBodySystem.cpp:170-204), both paths using the same
SHAKE/RATTLE solver:
  * the API mirror's Context, which applies the solvers to the owned buffers between the halves;
  * the C ABI's posDelta protocol of the OpenMM shim (rbx_free_atoms_delta, the solver on
    posDelta, rbx_integrate_part1_delta), with the solver standing in for OpenMM's applyConstraints.
Tolerances as test_gpu_parity.py's tethered cases: positions 1e-6 (mixed) and 1e-9 (double),
velocities 10x those, after 30 steps of 1 fs.
"""
import numpy as np
import pytest

from conftest import constrained_system, oracle_constrained_run, rel_err

pytestmark = pytest.mark.gpu

DT = 0.001
TOL = {"mixed": 1e-6, "double": 1e-9, "single": 2e-4}


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import api, build
    build.build_library()
    return api


@pytest.mark.parametrize("prec", ["mixed", "double"])
@pytest.mark.parametrize("mode", [0, 4])
def test_context_with_constraints_matches_oracle(api, oracle_mod, prec, mode):
    sysc = constrained_system()
    masses, bidx, x0, v0, force, pairs, dist = sysc
    system = api.System(masses)
    for (i, j), d in zip(pairs, dist):
        system.addConstraint(int(i), int(j), float(d))
    intg = api.RigidBodyIntegrator(DT, bidx)
    intg.setRotationMode(mode)
    ctx = api.Context(system, intg, force, precision=prec)
    ctx.setPositions(x0)
    ctx.setVelocities(v0)
    nb = len(set(bidx[bidx > 0].tolist()))
    assert intg.getRigidBodySystem().getNumDOF() == 6 * nb + 3 * 2 * len(pairs) - len(pairs)
    intg.step(30)
    st = ctx.getState(getPositions=True, getVelocities=True)
    o = oracle_constrained_run(oracle_mod, sysc, DT, 30, mode=mode)
    assert rel_err(st.getPositions(), o.R) < TOL[prec]
    assert rel_err(st.getVelocities(), o.V) < 10 * TOL[prec]
    x = st.getPositions()
    np.testing.assert_allclose(np.linalg.norm(x[pairs[:, 0]] - x[pairs[:, 1]], axis=1), dist, rtol=3e-5)


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
def test_posdelta_protocol_matches_oracle(api, oracle_mod, prec):
    from openmm_rigidbody_plugin_gb300 import kernel as K
    sysc = constrained_system(seed=6)
    masses, bidx, x0, v0, force, pairs, dist = sysc
    w = 1.0 / masses
    k = K.IntegratorKernel(masses, bidx, rotation_mode=0, precision=prec)
    k.set_constraints(pairs)
    buf = K.DeviceBuffers(len(masses), precision=prec)
    buf.set_positions(x0)
    buf.set_velocities(v0, masses)
    k.upload_state(x0, v0)
    buf.set_forces(force(x0)[0])
    for _ in range(30):
        xs = buf.get_positions()
        k.free_atoms_delta(buf, DT)
        d = buf.get_pos_delta()
        buf.set_pos_delta(api.shake(xs, xs + d, w, pairs, dist, 1e-5) - xs)  # OpenMM's applyConstraints
        k.part1_delta(buf, DT)
        buf.set_forces(force(buf.get_positions())[0])
        k.part2(buf, DT)
        buf.set_velocities(api.rattle_velocities(buf.get_positions(), buf.get_velocities(), w, pairs, 1e-5), masses)
    o = oracle_constrained_run(oracle_mod, sysc, DT, 30)
    assert rel_err(buf.get_positions(), o.R) < TOL[prec]
    assert rel_err(buf.get_velocities(), o.V) < 10 * TOL[prec]


def test_constraint_rules(api):
    sysc = constrained_system()
    masses, bidx, x0, v0, force, pairs, dist = sysc
    body_atom = int(np.flatnonzero(bidx > 0)[0])
    system = api.System(masses)
    system.addConstraint(body_atom, int(pairs[0, 0]), 0.1)
    with pytest.raises(api.OpenMMException, match="Constraints involving rigid-body atoms are not allowed"):
        api.Context(system, api.RigidBodyIntegrator(DT, bidx), force)
    system = api.System(masses)
    system.addConstraint(int(pairs[0, 0]), int(pairs[0, 1]), 0.1)
    intg = api.RigidBodyIntegrator(DT, bidx)
    intg.setComputeRefinedEnergies(True)
    with pytest.raises(api.OpenMMException, match="not available with constrained"):
        api.Context(system, intg, force)
