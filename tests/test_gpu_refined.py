"""Refined ("shadow") energies on the GPU, through the API mirror and the C ABI, against the FP64
oracle's restatement of the reference's COMPMOD path (tests/test_oracle_refined.py pins the oracle).

Systems: rigid bodies of 3-5 atoms plus free atoms on harmonic tethers (a smooth force field with
torques), forces evaluated on the host at every half step, 2 fs steps.

Tolerances. The kernels write per-body corrections to the plain kinetic energy, so they are
compared as corrections (refined minus plain), which are 1e-4..1e-3 of the kinetic energy here:
  double: corrections and the potential refinement within 1e-6 relative (FP64 throughout; the
          oracle's position stencils cancel to about 1e-11 of the corrections);
  mixed:  the translational correction is formed without cancellation (1e-4 relative after 30
          steps of an FP32-force trajectory); the rotational correction is a difference of two FP32
          per-body energies (about 1e-7 of each body's rotational energy), so it is held to 2e-2 of
          itself plus 1e-6 of the rotational energy; the potential refinement to 1e-4.
"""
import numpy as np
import pytest

from conftest import tether_system

pytestmark = pytest.mark.gpu

DT = 0.002


@pytest.fixture(scope="module")
def api():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import api, build
    build.build_library()
    return api


def gpu_run(api, prec, rot, nsteps, dt=DT, refined=True, **kw):
    m, bidx, x0, v0, force = tether_system(**kw)
    intg = api.RigidBodyIntegrator(dt, bidx)
    intg.setRotationMode(rot)
    intg.setComputeRefinedEnergies(refined)
    ctx = api.Context(api.System(m), intg, force, precision=prec)
    ctx.setPositions(x0)
    ctx.setVelocities(v0)
    out = []
    for _ in range(nsteps):
        intg.step(1)
        u = ctx.getState(getEnergy=True).getPotentialEnergy()
        out.append([u, *intg.getKineticEnergies(), *intg.getRefinedKineticEnergies(),
                    intg.getPotentialEnergyRefinement()])
    return np.array(out)


def oracle_run(oracle_mod, rot, nsteps, dt=DT, weights=1, **kw):
    m, bidx, x0, v0, force = tether_system(**kw)
    o = oracle_mod.Oracle(m, bidx, mode=rot, robust=True)
    o.setup(x0, v0, force(x0)[0])
    o.set_refined(weights)
    out = []
    for _ in range(nsteps):
        o.part1(dt, force(o.R)[0])
        F, U = force(o.R)
        o.part2(dt, F)
        out.append([U, *o.kinetic(), *o.refined(dt, F)])
    return np.array(out)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("rot", [0, 4])
def test_refined_energies_match_oracle(api, oracle_mod, prec, rot):
    g = gpu_run(api, prec, rot, 30)
    o = oracle_run(oracle_mod, rot, 30)
    for n in (0, 9, 29):
        _, kt, kr, rt, rr, ur = g[n]
        _, okt, okr, ort, orr, our = o[n]
        dt_g, dt_o = rt - kt, ort - okt
        dr_g, dr_o = rr - kr, orr - okr
        if prec == "double":
            assert abs(dt_g - dt_o) <= 1e-6 * abs(dt_o), (n, dt_g, dt_o)
            assert abs(dr_g - dr_o) <= 1e-6 * abs(dr_o), (n, dr_g, dr_o)
            assert abs(ur - our) <= 1e-6 * abs(our), (n, ur, our)
        else:
            assert abs(dt_g - dt_o) <= 1e-4 * abs(dt_o) + 1e-7 * okt, (n, dt_g, dt_o)
            assert abs(dr_g - dr_o) <= 2e-2 * abs(dr_o) + 1e-6 * okr, (n, dr_g, dr_o)
            assert abs(ur - our) <= 1e-4 * abs(our), (n, ur, our)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("rot", [0, 4])
def test_body_stencils_match_the_reference_weights(api, oracle_mod, prec, rot):
    """Rigid bodies only (no free atoms, so the free-atom stencil that this library corrects, defect
    D9, plays no part): the refined energies against the oracle run with the reference's own
    stencil weights (mode 2, the literal restatement of rigidbodyintegrator.cu:285-292, :318-321,
    :380-384, :433-469), to the tolerances of test_refined_energies_match_oracle."""
    g = gpu_run(api, prec, rot, 30, n_free=0)
    o = oracle_run(oracle_mod, rot, 30, weights=2, n_free=0)
    for n in (0, 9, 29):
        _, kt, kr, rt, rr, ur = g[n]
        _, okt, okr, ort, orr, our = o[n]
        dt_g, dt_o = rt - kt, ort - okt
        dr_g, dr_o = rr - kr, orr - okr
        tk, tr, tu = (1e-6, 1e-6, 1e-6) if prec == "double" else (1e-4, 2e-2, 1e-4)
        assert abs(dt_g - dt_o) <= tk * abs(dt_o) + (0 if prec == "double" else 1e-7 * okt), (n, dt_g, dt_o)
        assert abs(dr_g - dr_o) <= tr * abs(dr_o) + (0 if prec == "double" else 1e-6 * okr), (n, dr_g, dr_o)
        assert abs(ur - our) <= tu * abs(our), (n, ur, our)


@pytest.mark.parametrize("rot", [0, 4])
def test_shadow_energy_conserved_better_in_mixed(api, rot):
    """200 steps of 4 fs: the refined total energy U + U_ref + KE_ref fluctuates far less than
    U + KE (FP64 oracle: 9x less)."""
    g = gpu_run(api, "mixed", rot, 200, dt=0.004)
    H = g[:, 0] + g[:, 1] + g[:, 2]
    Hr = g[:, 0] + g[:, 5] + g[:, 3] + g[:, 4]
    assert Hr.std() < H.std() / 5, (H.std(), Hr.std())


def test_refined_off_returns_plain_energies(api):
    g = gpu_run(api, "mixed", 0, 3, refined=False)
    np.testing.assert_array_equal(g[:, 3:5], g[:, 1:3])
    assert np.all(g[:, 5] == 0.0)


def test_refined_query_needs_a_step(api):
    m, bidx, x0, v0, force = tether_system(n_bodies=4, n_free=2)
    intg = api.RigidBodyIntegrator(DT, bidx)
    intg.setComputeRefinedEnergies(True)
    ctx = api.Context(api.System(m), intg, force)
    ctx.setPositions(x0)
    ctx.setVelocities(v0)
    with pytest.raises(RuntimeError, match="completed step"):
        intg.getRefinedKineticEnergies()
    intg.step(1)
    intg.getRefinedKineticEnergies()
    ctx.setVelocities(v0)  # a state change restarts the stencils
    with pytest.raises(RuntimeError, match="completed step"):
        intg.getPotentialEnergyRefinement()


@pytest.mark.parametrize("prec", ["mixed", "double"])
def test_reordering_between_the_halves_keeps_the_stencils(api, prec):
    """Atoms moved to new slots between part1 and part2 (as OpenMM's reordering does): the
    library moves each body's and free atom's stencil sums with it."""
    from openmm_rigidbody_plugin_gb300 import kernel as K
    m, bidx, x0, v0, force = tether_system(seed=8, n_bodies=40, n_free=30)
    res = []
    for move in (False, True):
        k = K.IntegratorKernel(m, bidx, rotation_mode=0, precision=prec)
        k.set_compute_refined_energies(True)
        buf = K.DeviceBuffers(len(m), precision=prec)
        buf.set_positions(x0)
        buf.set_velocities(v0, m)
        k.upload_state(x0, v0)
        buf.set_forces(force(x0)[0])
        rng = np.random.default_rng(3)
        for n in range(4):
            k.part1(buf, DT)
            if move:
                loc = rng.permutation(len(m))
                buf.relocate(loc)
                k.set_atom_locations(loc)
            buf.set_forces(force(buf.get_positions())[0])
            k.part2(buf, DT)
        res.append(np.concatenate([k.refined_kinetic_energies(buf), [k.potential_energy_refinement(buf)]]))
    np.testing.assert_allclose(res[1], res[0], rtol=1e-12)


def test_fused_steps_accumulate_the_same_stencils(api):
    """The host-buffer step (part1, fused x (n-1), part2) closes the same stencils as n separate
    part1/part2 steps under a fixed force array (fused kicks round differently: 1e-6)."""
    from openmm_rigidbody_plugin_gb300 import kernel as K
    m, bidx, x0, v0, force = tether_system(seed=9, n_bodies=30, n_free=20)
    F = np.ascontiguousarray(force(x0)[0])
    res = []
    for fused in (False, True):
        k = K.IntegratorKernel(m, bidx, rotation_mode=0, precision="mixed")
        k.set_compute_refined_energies(True)
        k.context_set_state(x0, v0)
        if fused:
            R, V = np.zeros_like(x0), np.zeros_like(v0)
            k.step_host(10, DT, F, R, V)
        else:
            k.context_set_forces(F)
            for _ in range(10):
                k.context_step("part1", DT)
                k.context_step("part2", DT)
        res.append(np.concatenate([k.context_kinetic_energies(), k.context_refined_kinetic_energies(),
                                   [k.context_potential_energy_refinement()]]))
    corr = [r[2:4] - r[0:2] for r in res]
    np.testing.assert_allclose(corr[1], corr[0], rtol=1e-3, atol=1e-7 * res[0][0:2].sum())
    np.testing.assert_allclose(res[1][4], res[0][4], rtol=1e-6)
