"""The API mirror on the CPU: serialization (the reference's own serialization test values),
integrator parameter errors, ForceField rigid-body templates, StateDataReporter columns."""
import io

import numpy as np
import pytest

from openmm_rigidbody_plugin_gb300 import api


def test_serialization_round_trip_as_the_reference_tests_it():
    # serialization/tests/TestSerializeRigidBodyIntegrator.cpp:48-62
    intg = api.RigidBodyIntegrator(0.00342, [5, 4, 3, 2, 1])
    text = api.serialize(intg)
    assert 'version="1"' in text
    intg2 = api.deserialize(text)
    assert intg2.getConstraintTolerance() == intg.getConstraintTolerance()
    assert intg2.getStepSize() == intg.getStepSize()
    assert intg2.getBodyIndices() == [5, 4, 3, 2, 1]
    assert intg2.getRotationMode() == 0


def test_rotation_mode_is_serialized_as_version_2():
    intg = api.RigidBodyIntegrator(0.002, [1, 1, 1, 0])
    intg.setRotationMode(10)
    intg.setConstraintTolerance(2e-6)
    back = api.deserialize(api.serialize(intg))
    assert back.getRotationMode() == 10 and back.getConstraintTolerance() == 2e-6
    with pytest.raises(api.OpenMMException, match="Unsupported version"):
        api.deserialize(api.serialize(intg).replace('version="2"', 'version="3"'))


def test_integrator_parameter_errors():
    intg = api.RigidBodyIntegrator(0.002, [1, 1, 0])
    with pytest.raises(api.OpenMMException, match="Rotation mode cannot be negative"):
        intg.setRotationMode(-1)
    with pytest.raises(api.OpenMMException, match="not bound"):
        intg.step(1)
    with pytest.raises(api.OpenMMException, match="not bound"):
        intg.getRefinedKineticEnergies()
    with pytest.raises(api.OpenMMException, match="not bound"):
        intg.getPotentialEnergyRefinement()
    intg.setComputeRefinedEnergies(True)
    assert intg.getComputeRefinedEnergies()


def _waters_and_ligand():
    top = api.Topology()
    for _ in range(3):
        top.addResidue("HOH", ["O", "H1", "H2"])
    top.addResidue("LIG", ["C1", "C2", "H1", "H2", "EP"])
    ff = api.ForceField({"HOH": {"atoms": ["O", "H1", "H2"]},
                         "LIG": {"atoms": ["C1", "C2", "H1", "H2", "EP"], "virtualSites": ["EP"]}})
    return top, ff


def test_force_field_templates_resolve_and_merge_bodies():
    top, ff = _waters_and_ligand()
    ff.registerBodyTemplate("water", "HOH")
    ff.registerBodyTemplate("ring", "LIG", "(C1|C2)")
    with pytest.raises(ValueError):
        ff.registerBodyTemplate("water", "HOH")
    with pytest.raises(ValueError):
        ff.registerBodyTemplate("x", "XYZ")
    idx = ff.resolveBodies(top)
    assert idx == [1, 1, 1, 2, 2, 2, 3, 3, 3, 4, 4, 0, 0, 0]
    # merged sets take their smallest index; overlapping merge sets are joined first
    assert ff.resolveBodies(top, merge=[[2, 3], [3, 4]]) == [1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 0, 0, 0]
    assert ff.resolveBodies(top, merge=[1, 4]) == [1, 1, 1, 2, 2, 2, 3, 3, 3, 1, 1, 0, 0, 0]
    with pytest.raises(ValueError):
        ff.resolveBodies(top, merge=5)
    ff2 = api.ForceField({"HOH": {"atoms": ["O", "H1", "H2"]}})
    ff2.registerBodyTemplate("none", "HOH", "Q.*")
    with pytest.raises(ValueError, match="no atom"):
        ff2.resolveBodies(top)


def test_intra_body_constraints_and_interactions_are_removed():
    top, ff = _waters_and_ligand()
    ff.registerBodyTemplate("water", "HOH")
    idx = ff.resolveBodies(top)
    system = api.System([16.0, 1.0, 1.0] * 3 + [12.0, 12.0, 1.0, 1.0, 0.0])
    nb = api.NonbondedForce()
    for _ in range(system.getNumParticles()):
        nb.addParticle(0.1, 0.3, 0.5)
    system.addForce(nb)
    system.addConstraint(0, 1, 0.1)
    system.addConstraint(9, 10, 0.14)   # ligand atoms: not in a body here
    system.addConstraint(3, 9, 0.5)     # one body atom
    ff.removeConstraints(system, idx)
    assert system.constraints == [(9, 10, 0.14)]
    ff.removeForces(system, idx)
    assert nb.getNumExceptions() == 3 * 3  # three pairs in each of three waters
    assert all(v == (0.0, 1.0, 0.0) for v in nb.exceptions.values())
    assert sorted(ff._intraBodyPairs([1, 1, 0, 2, 2, 2])) == [(0, 1), (3, 4), (3, 5), (4, 5)]


class _FakeIntegrator:
    """Stands in for the bound integrator: the library's count is `dof`, the reference's count
    (one per free atom instead of three) 20 less."""

    def __init__(self, dof):
        self._dof = dof

    def getRigidBodySystem(self):
        return type("S", (), {"getNumDOF": lambda s, reference=False: self._dof - (20 if reference else 0)})()

    def getKineticEnergies(self):
        return [30.0, 12.0]

    def getRefinedKineticEnergies(self):
        return [31.0, 11.5]

    def getPotentialEnergyRefinement(self):
        return -0.25


class _FakeContext:
    def __init__(self, dof, cmm):
        self.integrator = _FakeIntegrator(dof)
        self.system = api.System([1.0])
        if cmm:
            self.system.addForce(api.CMMotionRemover())

    def getState(self, getEnergy=False):
        return api.State(potential=-5.0)


@pytest.mark.parametrize("cmm", [False, True])
def test_state_data_reporter_columns_and_temperature(cmm):
    out = io.StringIO()
    rep = api.StateDataReporter(out, 10, translationalEnergy=True, rotationalEnergy=True)
    rep.report(_FakeContext(60, cmm), 10)
    header, line = out.getvalue().splitlines()
    assert header.split(",") == ['#"Step"', "Potential Energy (kJ/mole)", "Kinetic Energy (kJ/mole)",
                                 "Total Energy (kJ/mole)", "Temperature (K)", "Translational Energy (kJ/mole)",
                                 "Rotational Energy (kJ/mole)"]
    v = [float(x) for x in line.split(",")]
    dof = 60 - (3 if cmm else 0)
    np.testing.assert_allclose(v, [10, -5.0, 42.0, 37.0, 2 * 42.0 / (dof * api.KB), 30.0, 12.0])


def test_state_data_reporter_temperature_with_the_reference_count():
    """referenceDOF=True divides by the reference's own count (RigidBodySystem.cpp:130), as the
    plugin's reporter does (python/statedatareporter.py:19-28)."""
    out = io.StringIO()
    rep = api.StateDataReporter(out, 10, step=False, potentialEnergy=False, kineticEnergy=False, totalEnergy=False,
                                referenceDOF=True)
    rep.report(_FakeContext(60, True), 10)
    np.testing.assert_allclose(float(out.getvalue().splitlines()[1]), 2 * 42.0 / ((60 - 20 - 3) * api.KB))


def test_state_data_reporter_refined_columns():
    """Refined columns in the reference's order (python/statedatareporter.py:30-48): potential plus
    refinement, refined kinetic, their total, refined temperature, refined translational/rotational."""
    out = io.StringIO()
    rep = api.StateDataReporter(out, 10, step=False, potentialEnergy=False, kineticEnergy=False, totalEnergy=False,
                                temperature=False, refinedPotentialEnergy=True, refinedKineticEnergy=True,
                                refinedTotalEnergy=True, refinedTemperature=True, refinedTranslationalEnergy=True,
                                refinedRotationalEnergy=True)
    rep.report(_FakeContext(60, True), 10)
    header, line = out.getvalue().splitlines()
    assert header.split(",") == ["Refined Potential Energy (kJ/mole)", "Refined Kinetic Energy (kJ/mole)",
                                 "Refined Total Energy (kJ/mole)", "Refined Temperature (K)",
                                 "Refined Translational Energy (kJ/mole)", "Refined Rotational Energy (kJ/mole)"]
    v = [float(x) for x in line.split(",")]
    np.testing.assert_allclose(v, [-5.25, 42.5, 37.25, 2 * 42.5 / (57 * api.KB), 31.0, 11.5])
