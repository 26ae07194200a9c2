"""The plugin's user-facing API, mirrored on top of the library (OpenMM itself is not a dependency).

* ``RigidBodyIntegrator`` -- RigidBodyIntegrator(stepSize, bodyIndices) with setRotationMode,
  step, getKineticEnergies, getRigidBodySystem (openmmapi/src/RigidBodyIntegrator.cpp:18-93),
  bound to a ``Context``.
* ``RigidBodySystem`` -- the counts the plugin exposes (openmmapi/include/RigidBodySystem.h:38-50).
* ``serialize`` / ``deserialize`` -- the XML form of serialization/src/RigidBodyIntegratorProxy.cpp:
  40-67 (version 1: stepSize, constraintTolerance, bodyIndices); a non-zero rotation mode is
  written as version 2 with a rotationMode attribute, and both versions are read.
* ``ForceField`` -- rigid-body templates over residue templates: registerBodyTemplate,
  resolveBodies with merge lists, removeConstraints, removeForces (python/forcefield.py:3-180).
* ``StateDataReporter`` -- the extra columns of python/statedatareporter.py:5-90 (translational
  and rotational energies, the refined ("shadow") energies and temperature; temperature from the
  rigid-body degrees of freedom, minus 3 with a centre-of-mass motion remover).

``Context`` stands in for an OpenMM Context on one device: a ``System`` (masses, constraints,
forces), the integrator, positions, velocities and a force provider, a callable positions ->
(forces, potential energy) evaluated on the host between the two halves of each step, the way the
Reference platform drives RigidBodySystem::integratePart1/2 (RigidBodySystem.cpp:170-204).
Constraints between free atoms are enforced, as OpenMM's solvers do, by ``shake`` after part1 and
``rattle_velocities`` after part2 (ReferenceRigidBodyKernels.cpp:82-108); constraints on body atoms
are rejected (RigidBodySystem.cpp:107-113).
Refined ("shadow") energies: setComputeRefinedEnergies before the integrator is bound, then
getRefinedKineticEnergies / getPotentialEnergyRefinement after a step (RigidBodyIntegrator.cpp:
34-38, 84-90), computed on the device by the step kernels.
"""
import re
import xml.etree.ElementTree as ET

import numpy as np

from . import kernel as _kernel
from .workloads import KB

__all__ = ["System", "NonbondedForce", "CMMotionRemover", "Topology", "Context", "RigidBodyIntegrator",
           "RigidBodySystem", "serialize", "deserialize", "ForceField", "StateDataReporter", "shake",
           "rattle_velocities"]


class OpenMMException(RuntimeError):
    """The plugin's misuse errors (OpenMMException in the reference)."""


# --------------------------------------------------------------------------------------------
# Constraint solvers of the Context stand-in (OpenMM's own enforce constraints in a real Context)
# --------------------------------------------------------------------------------------------
def shake(x_old, x, inv_mass, pairs, dist, tol=1e-5, max_iter=200):
    """Positions x with |x_i - x_j| = d for every constrained pair, corrected along the bonds of
    x_old (SHAKE, Ryckaert, Ciccotti and Berendsen 1977); tol is relative, as OpenMM's."""
    x = np.array(x, dtype=np.float64)
    i, j = pairs[:, 0], pairs[:, 1]
    wi, wj = inv_mass[i], inv_mass[j]
    r0 = x_old[i] - x_old[j]
    d2 = dist * dist
    for _ in range(max_iter):
        rij = x[i] - x[j]
        diff = d2 - np.einsum("ij,ij->i", rij, rij)
        if np.all(np.abs(diff) <= 2.0 * tol * d2):
            break
        g = diff / (2.0 * np.einsum("ij,ij->i", rij, r0) * (wi + wj))
        np.add.at(x, i, (g * wi)[:, None] * r0)
        np.subtract.at(x, j, (g * wj)[:, None] * r0)
    return x


def rattle_velocities(x, v, inv_mass, pairs, tol=1e-5, max_iter=200):
    """Velocities v with no relative component along any constrained bond (RATTLE, Andersen 1983)."""
    v = np.array(v, dtype=np.float64)
    i, j = pairs[:, 0], pairs[:, 1]
    wi, wj = inv_mass[i], inv_mass[j]
    rij = x[i] - x[j]
    r2 = np.einsum("ij,ij->i", rij, rij)
    for _ in range(max_iter):
        rv = np.einsum("ij,ij->i", rij, v[i] - v[j])
        if np.all(np.abs(rv) <= tol * r2):
            break
        k = rv / (r2 * (wi + wj))
        np.subtract.at(v, i, (k * wi)[:, None] * rij)
        np.add.at(v, j, (k * wj)[:, None] * rij)
    return v


# --------------------------------------------------------------------------------------------
# Minimal System / force / topology description (the parts the plugin's API reads)
# --------------------------------------------------------------------------------------------
class NonbondedForce:
    def __init__(self):
        self.particles = []     # (charge, sigma, epsilon)
        self.exceptions = {}    # (i, j) with i < j -> (chargeProd, sigma, epsilon)

    def addParticle(self, charge, sigma, epsilon):
        self.particles.append((charge, sigma, epsilon))
        return len(self.particles) - 1

    def addException(self, i, j, chargeProd, sigma, epsilon, replace=False):
        key = (min(i, j), max(i, j))
        if key in self.exceptions and not replace:
            raise OpenMMException(f"There is already an exception for particles {i} and {j}")
        self.exceptions[key] = (chargeProd, sigma, epsilon)

    def getNumExceptions(self):
        return len(self.exceptions)


class CMMotionRemover:
    pass


class System:
    def __init__(self, masses=()):
        self.masses = [float(m) for m in masses]
        self.constraints = []   # (i, j, distance)
        self.forces = []

    def addParticle(self, mass):
        self.masses.append(float(mass))
        return len(self.masses) - 1

    def getNumParticles(self):
        return len(self.masses)

    def getParticleMass(self, i):
        return self.masses[i]

    def addConstraint(self, i, j, distance):
        self.constraints.append((i, j, distance))

    def getNumConstraints(self):
        return len(self.constraints)

    def getConstraintParameters(self, k):
        return self.constraints[k]

    def removeConstraint(self, k):
        del self.constraints[k]

    def addForce(self, force):
        self.forces.append(force)
        return len(self.forces) - 1

    def getNumForces(self):
        return len(self.forces)

    def getForce(self, k):
        return self.forces[k]


class Topology:
    """Residues (name, atom names) in atom order; atom indices are assigned in that order."""

    class Atom:
        def __init__(self, name, index):
            self.name, self.index = name, index

    class Residue:
        def __init__(self, name, atoms):
            self.name, self._atoms = name, atoms

        def atoms(self):
            return iter(self._atoms)

    def __init__(self):
        self._residues = []
        self._n = 0

    def addResidue(self, name, atom_names):
        atoms = []
        for a in atom_names:
            atoms.append(Topology.Atom(a, self._n))
            self._n += 1
        self._residues.append(Topology.Residue(name, atoms))

    def residues(self):
        return iter(self._residues)

    def getNumAtoms(self):
        return self._n


# --------------------------------------------------------------------------------------------
# Integrator, rigid-body system, context
# --------------------------------------------------------------------------------------------
class RigidBodySystem:
    """Counts of the bound integrator's rigid-body system."""

    def __init__(self, k, body_indices):
        self._k = k
        self._bidx = np.asarray(body_indices)

    def getNumDOF(self, reference=False):
        """Degrees of freedom: three per free atom, and the atoms of unique body indices free (the
        library's count); with reference=True, the integer RigidBodySystem::getNumDOF reports
        (openmmapi/src/RigidBodySystem.cpp:130: one per free atom, unique indices as one-atom
        bodies)."""
        return self._k.num_dof_reference if reference else self._k.num_dof

    def getNumBodies(self):
        return self._k.num_bodies

    def getNumFree(self):
        return self._k.num_free

    def getNumActualAtoms(self):
        return int(np.count_nonzero(self._k.masses > 0))

    def getNumBodyAtoms(self):
        return self.getNumActualAtoms() - self.getNumFree()


class RigidBodyIntegrator:
    def __init__(self, stepSize, bodyIndices):
        self._dt = float(stepSize)
        self._tol = 1e-5
        self._bodyIndices = [int(i) for i in bodyIndices]
        self._mode = 0
        self._refined = False
        self._context = None
        self._kernel = None
        self._cons = None

    # parameters (RigidBodyIntegrator.cpp:18-38)
    def getStepSize(self):
        return self._dt

    def setStepSize(self, dt):
        self._dt = float(dt)

    def getConstraintTolerance(self):
        return self._tol

    def setConstraintTolerance(self, tol):
        self._tol = float(tol)

    def setRotationMode(self, mode):
        if mode < 0:
            raise OpenMMException("Rotation mode cannot be negative")
        if self._context is not None:
            raise OpenMMException("Cannot set rotation mode: integrator already bound to a context")
        self._mode = int(mode)

    def getRotationMode(self):
        return self._mode

    def setComputeRefinedEnergies(self, compute):
        if self._context is not None:
            raise OpenMMException("Cannot set refined energy computation: integrator already bound to a context")
        self._refined = bool(compute)

    def getComputeRefinedEnergies(self):
        return self._refined

    def getBodyIndices(self):
        return list(self._bodyIndices)

    # binding and stepping
    def _bind(self, context):
        if self._context is not None and self._context is not context:
            raise OpenMMException("This Integrator is already bound to a context")
        if context.system.getNumParticles() != len(self._bodyIndices):
            raise OpenMMException("Number of body indices differs from that of atoms in Context")
        self._context = context
        self._kernel = _kernel.IntegratorKernel(context.system.masses, self._bodyIndices, rotation_mode=self._mode,
                                                precision=context.precision, device=context.device)
        self._kernel.set_compute_refined_energies(self._refined)
        cons = context.system.constraints
        if cons:
            if self._refined:
                raise OpenMMException("Refined energies are not available with constrained free atoms")
            try:
                self._kernel.set_constraints([(c[0], c[1]) for c in cons])
            except RuntimeError as e:
                raise OpenMMException(str(e).split(" [")[0]) from None
            m = np.asarray(context.system.masses, dtype=np.float64)
            self._cons = (np.array([(c[0], c[1]) for c in cons], dtype=np.int64),
                          np.array([c[2] for c in cons], dtype=np.float64),
                          np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0))
        else:
            self._cons = None

    def getRigidBodySystem(self):
        self._require()
        self._context._ensure_state()
        return RigidBodySystem(self._kernel, self._bodyIndices)

    def _require(self):
        if self._context is None:
            raise OpenMMException("This Integrator is not bound to a context")

    def step(self, steps):
        """`steps` velocity-Verlet steps: part1, forces at the new positions, part2; with constraints,
        SHAKE after part1 with the (R - savedPos)/dt velocity correction and RATTLE after part2
        (ReferenceRigidBodyKernels.cpp:82-108, RigidBodySystem.cpp:170-204)."""
        self._require()
        c, k = self._context, self._kernel
        c._ensure_state()
        dt = self._dt
        for _ in range(int(steps)):
            if self._cons is not None:
                x0, _ = k.context_get_state()
            k.context_step("part1", dt)
            x, v = k.context_get_state()
            if self._cons is not None:
                pairs, dist, w = self._cons
                xc = shake(x0, x, w, pairs, dist, self._tol)
                v = v + (xc - x) / dt
                k.context_load(xc, v)
                x = xc
            c._apply_forces(x)
            k.context_step("part2", dt)
            if self._cons is not None:
                x, v = k.context_get_state()
                k.context_load(x, rattle_velocities(x, v, self._cons[2], self._cons[0], self._tol))
        c._stale = True

    def getKineticEnergies(self):
        """[translational, rotational] kinetic energy (kJ/mol)."""
        self._require()
        self._context._ensure_state()
        return [float(e) for e in self._kernel.context_kinetic_energies()]

    def computeKineticEnergy(self):
        return sum(self.getKineticEnergies())

    def getRefinedKineticEnergies(self):
        """[translational, rotational] refined kinetic energy (kJ/mol) after the last step; the plain
        kinetic energies while refined energies are off (CudaRigidBodyKernels.cpp:469-476)."""
        self._require()
        self._context._ensure_state()
        return [float(e) for e in self._kernel.context_refined_kinetic_energies()]

    def getPotentialEnergyRefinement(self):
        """-dt^2/24 (sum |F|^2/m + tau.I^-1.tau) after the last step; 0 while refined energies are off
        (CudaRigidBodyKernels.cpp:481-494)."""
        self._require()
        self._context._ensure_state()
        return self._kernel.context_potential_energy_refinement()


class State:
    def __init__(self, positions=None, velocities=None, potential=None, kinetic=None):
        self._x, self._v, self._u, self._k = positions, velocities, potential, kinetic

    def getPositions(self, asNumpy=True):
        return self._x

    def getVelocities(self, asNumpy=True):
        return self._v

    def getPotentialEnergy(self):
        return self._u

    def getKineticEnergy(self):
        return self._k


class Context:
    """One simulation on one device: System + RigidBodyIntegrator + positions, velocities and a
    host force provider f(positions) -> (forces [N, 3] kJ/mol/nm, potential energy kJ/mol)."""

    def __init__(self, system, integrator, forces, precision="mixed", device=0):
        self.system = system
        self.integrator = integrator
        self.precision = precision
        self.device = device
        self._forces = forces
        n = system.getNumParticles()
        self._x = np.zeros((n, 3))
        self._v = np.zeros((n, 3))
        self._u = 0.0
        self._dirty = True
        self._stale = False
        integrator._bind(self)

    def setPositions(self, positions):
        self._x = np.array(positions, dtype=np.float64).reshape(-1, 3)
        self._dirty = True

    def setVelocities(self, velocities):
        self._v = np.array(velocities, dtype=np.float64).reshape(-1, 3)
        self._dirty = True

    def _apply_forces(self, x):
        f, u = self._forces(x)
        self._u = float(u)
        self.integrator._kernel.context_set_forces(f)

    def _ensure_state(self):
        """Rebuild the bodies after a position or velocity change (RigidBodyIntegrator::stateChanged,
        RigidBodyIntegrator.cpp:63-74): forces at the new positions, geometry and momenta."""
        if self._dirty:
            k = self.integrator._kernel
            k.context_set_state(self._x, self._v)
            self._apply_forces(self._x)
            self._dirty = False
            self._stale = False

    def getState(self, getPositions=False, getVelocities=False, getEnergy=False):
        self._ensure_state()
        if self._stale:
            self._x, self._v = self.integrator._kernel.context_get_state()
            self._stale = False
        ke = self.integrator.computeKineticEnergy() if getEnergy else None
        return State(self._x.copy() if getPositions else None, self._v.copy() if getVelocities else None,
                     self._u if getEnergy else None, ke)


# --------------------------------------------------------------------------------------------
# Serialization (RigidBodyIntegratorProxy.cpp:40-67)
# --------------------------------------------------------------------------------------------
def serialize(integrator):
    version = 1 if integrator.getRotationMode() == 0 else 2
    root = ET.Element("RigidBodyIntegrator", {"constraintTolerance": repr(integrator.getConstraintTolerance()),
                                              "stepSize": repr(integrator.getStepSize()),
                                              "type": "RigidBodyIntegrator", "version": str(version)})
    if version == 2:
        root.set("rotationMode", str(integrator.getRotationMode()))
    node = ET.SubElement(root, "bodyIndices")
    for index in integrator.getBodyIndices():
        ET.SubElement(node, "bodyIndex", {"index": str(index)})
    return '<?xml version="1.0" ?>\n' + ET.tostring(root, encoding="unicode")


def deserialize(text):
    root = ET.fromstring(text)
    version = int(root.get("version"))
    if version not in (1, 2):
        raise OpenMMException("Unsupported version number")
    integrator = RigidBodyIntegrator(float(root.get("stepSize")),
                                     [int(b.get("index")) for b in root.find("bodyIndices")])
    integrator.setConstraintTolerance(float(root.get("constraintTolerance")))
    if version == 2:
        integrator.setRotationMode(int(root.get("rotationMode")))
    return integrator


# --------------------------------------------------------------------------------------------
# ForceField rigid-body templates (python/forcefield.py)
# --------------------------------------------------------------------------------------------
class ForceField:
    """Rigid-body templates over residue templates {residue: {"atoms": [names],
    "virtualSites": [names]}}."""

    class _BodyTemplate:
        def __init__(self, residue, pattern, virtualSites):
            self.residue, self.pattern, self.virtualSites = residue, pattern, virtualSites

    def __init__(self, residue_templates):
        self._templates = dict(residue_templates)
        self._bodyTemplates = {}

    def getBodyTemplate(self, name):
        return self._bodyTemplates[name]

    def registerBodyTemplate(self, name, residue, pattern=".+"):
        if name in self._bodyTemplates:
            raise ValueError("A rigid body template named %s has already been registered." % name)
        if residue not in self._templates:
            raise ValueError("Unknown residue %s in rigid body registration." % residue)
        vs = set(self._templates[residue].get("virtualSites", ()))
        self._bodyTemplates[name] = ForceField._BodyTemplate(residue, pattern if pattern is not None else ".+", vs)

    @staticmethod
    def _disjointSets(sets):
        """Merge overlapping sets until all are disjoint."""
        sets = [set(s) for s in sets]
        changed = True
        while changed:
            changed = False
            out = []
            for s in sets:
                for t in out:
                    if not t.isdisjoint(s):
                        t |= s
                        changed = True
                        break
                else:
                    out.append(set(s))
            sets = out
        return sets

    def resolveBodies(self, topology, merge=None):
        """Body index of every atom (0 = free); bodies numbered in residue order, one per matching
        template and residue; `merge` lists (or one list) of body indices to merge, each merged
        set taking its smallest index."""
        index = [0] * topology.getNumAtoms()
        n = 0
        for res in topology.residues():
            for body in (b for b in self._bodyTemplates.values() if b.residue == res.name):
                n += 1
                atoms = [a for a in res.atoms() if a.name not in body.virtualSites and re.match(body.pattern, a.name)]
                if not atoms:
                    raise ValueError("no atom in residue %s matches pattern %s" % (res.name, body.pattern))
                for a in atoms:
                    index[a.index] = n
        if merge is not None:
            if not hasattr(merge, "__iter__"):
                raise ValueError("merge parameter is not a sequence")
            if all(hasattr(m, "__iter__") for m in merge):
                sets = self._disjointSets([set(m) for m in merge])
            else:
                sets = [set(merge)]
            for s in sets:
                target = min(s)
                index = [target if b in s else b for b in index]
        return index

    @staticmethod
    def _intraBodyPairs(bodyIndices):
        members = {}
        for i, b in enumerate(bodyIndices):
            if b != 0:
                members.setdefault(b, []).append(i)
        return [(i, j) for atoms in members.values() for a, i in enumerate(atoms) for j in atoms[a + 1:]]

    def removeConstraints(self, system, bodyIndices):
        for k in reversed(range(system.getNumConstraints())):
            i, j, _ = system.getConstraintParameters(k)
            if bodyIndices[i] != 0 or bodyIndices[j] != 0:
                system.removeConstraint(k)

    def removeForces(self, system, bodyIndices):
        nonbonded = [f for f in system.forces if isinstance(f, NonbondedForce)]
        for i, j in self._intraBodyPairs(bodyIndices):
            for f in nonbonded:
                f.addException(i, j, 0.0, 1.0, 0.0, replace=True)


# --------------------------------------------------------------------------------------------
# StateDataReporter columns (python/statedatareporter.py)
# --------------------------------------------------------------------------------------------
class StateDataReporter:
    """Writes one comma-separated line per report: step, potential, kinetic and total energy,
    temperature (rigid-body degrees of freedom, minus 3 with a CMMotionRemover in the System),
    and optionally the translational and rotational kinetic energies and the refined energies, in
    the column order of python/statedatareporter.py:30-48. With referenceDOF=True the temperature
    divides by the reference's own degree-of-freedom count (getNumDOF(reference=True)), so the
    column equals the plugin's reporter on the same state."""

    _NAMES = {"step": '#"Step"', "potentialEnergy": "Potential Energy (kJ/mole)",
              "kineticEnergy": "Kinetic Energy (kJ/mole)", "totalEnergy": "Total Energy (kJ/mole)",
              "temperature": "Temperature (K)", "translationalEnergy": "Translational Energy (kJ/mole)",
              "rotationalEnergy": "Rotational Energy (kJ/mole)",
              "refinedPotentialEnergy": "Refined Potential Energy (kJ/mole)",
              "refinedKineticEnergy": "Refined Kinetic Energy (kJ/mole)",
              "refinedTotalEnergy": "Refined Total Energy (kJ/mole)",
              "refinedTemperature": "Refined Temperature (K)",
              "refinedTranslationalEnergy": "Refined Translational Energy (kJ/mole)",
              "refinedRotationalEnergy": "Refined Rotational Energy (kJ/mole)"}

    def __init__(self, file, reportInterval, step=True, potentialEnergy=True, kineticEnergy=True,
                 totalEnergy=True, temperature=True, translationalEnergy=False, rotationalEnergy=False,
                 refinedPotentialEnergy=False, refinedKineticEnergy=False, refinedTotalEnergy=False,
                 refinedTemperature=False, refinedTranslationalEnergy=False, refinedRotationalEnergy=False,
                 referenceDOF=False):
        self._out = file
        self._reference_dof = bool(referenceDOF)
        self._interval = int(reportInterval)
        self._cols = dict(step=step, potentialEnergy=potentialEnergy, kineticEnergy=kineticEnergy,
                          totalEnergy=totalEnergy, temperature=temperature, translationalEnergy=translationalEnergy,
                          rotationalEnergy=rotationalEnergy, refinedPotentialEnergy=refinedPotentialEnergy,
                          refinedKineticEnergy=refinedKineticEnergy, refinedTotalEnergy=refinedTotalEnergy,
                          refinedTemperature=refinedTemperature, refinedTranslationalEnergy=refinedTranslationalEnergy,
                          refinedRotationalEnergy=refinedRotationalEnergy)
        self._header = False
        self._dof = None

    def headers(self):
        return [self._NAMES[k] for k, on in self._cols.items() if on]

    def report(self, context, step):
        if self._dof is None:
            self._dof = context.integrator.getRigidBodySystem().getNumDOF(reference=self._reference_dof)
            if any(isinstance(f, CMMotionRemover) for f in context.system.forces):
                self._dof -= 3
        if not self._header:
            self._out.write(",".join(self.headers()) + "\n")
            self._header = True
        st = context.getState(getEnergy=True)
        integ = context.integrator
        kt, kr = integ.getKineticEnergies()
        u = st.getPotentialEnergy()
        vals = {"step": step, "potentialEnergy": u, "kineticEnergy": kt + kr, "totalEnergy": u + kt + kr,
                "temperature": 2.0 * (kt + kr) / (self._dof * KB), "translationalEnergy": kt, "rotationalEnergy": kr}
        c = self._cols
        if c["refinedPotentialEnergy"] or c["refinedTotalEnergy"]:
            vals["refinedPotentialEnergy"] = u + integ.getPotentialEnergyRefinement()
        if any(c[k] for k in ("refinedKineticEnergy", "refinedTotalEnergy", "refinedTemperature",
                              "refinedTranslationalEnergy", "refinedRotationalEnergy")):
            rt, rr = integ.getRefinedKineticEnergies()
            vals.update(refinedKineticEnergy=rt + rr, refinedTranslationalEnergy=rt, refinedRotationalEnergy=rr,
                        refinedTemperature=2.0 * (rt + rr) / (self._dof * KB))
            if c["refinedTotalEnergy"]:
                vals["refinedTotalEnergy"] = rt + rr + vals["refinedPotentialEnergy"]
        self._out.write(",".join(str(vals[k]) for k, on in c.items() if on) + "\n")
