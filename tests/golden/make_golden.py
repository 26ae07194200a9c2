"""Generate the golden fixtures of tests/golden/ by running the reference plugin's own CPU code.

The reference's openmmapi sources (RigidBodySystem, RigidBody, MatVec, eigenDecomposition) are
compiled unmodified by ``oracle/Makefile`` into ``oracle/_ref/librefrb.so``; this script drives
that library (through ``oracle/oracle.py``) on seeded synthetic inputs and stores the inputs and
outputs as ``.npz`` files. Run it where the reference tree is available:

    make -C oracle ref REF=/path/to/openmm_rigidbody_plugin && python tests/golden/make_golden.py

Every force array is quantised to the 2^-32 fixed point that OpenMM's CUDA platform uses, so the
CUDA path sees exactly the same forces as the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import Reference, reference_available  # noqa: E402
from openmm_rigidbody_plugin_gb300 import workloads as W  # noqa: E402


def quantise(f):
    return np.round(np.asarray(f, dtype=np.float64) * 2.0 ** 32) / 2.0 ** 32


def water_fixed_force(mode, nsteps=100, dt=0.002, sd=500.0):
    """64 rigid waters + 8 free argon atoms, fixed seeded Gaussian forces of standard deviation sd
    (kJ/mol/nm)."""
    s = W.mixed_system(n_bodies=64, n_free=8, fractions=(1.0, 0.0, 0.0), seed=11)
    F = quantise(W.gaussian_forces(s.num_atoms, seed=5, sd=sd))
    r = Reference(s.masses, s.body_indices, mode)
    r.setup(s.positions, s.velocities, F)
    ke0 = r.kinetic()
    dof = r.num_dof
    traj_R, traj_V, ke = [], [], []
    for n in range(nsteps):
        r.part1(dt, F)
        r.part2(dt, F)
        if (n + 1) % 10 == 0:
            traj_R.append(r.R.copy()); traj_V.append(r.V.copy()); ke.append(r.kinetic())
    return dict(masses=s.masses, body_indices=s.body_indices, R0=s.positions, V0=s.velocities, F=F, dt=dt,
                mode=mode, nsteps=nsteps, ke0=ke0, dof=dof, R=np.array(traj_R), V=np.array(traj_V), ke=np.array(ke))


def water_tether(mode=0, nsteps=200, dt=0.002, k=1000.0):
    """27 waters held by harmonic tethers F = -k (R - R0): position-dependent conservative forces."""
    s = W.water_box(27, seed=1)
    R0 = s.positions.copy()

    def force(R):
        return quantise(-k * (R - R0))

    r = Reference(s.masses, s.body_indices, mode)
    r.setup(s.positions, s.velocities, force(s.positions))
    F = force(s.positions)
    energy, Rs, Vs = [], [], []
    for n in range(nsteps):
        r.part1(dt, F)
        F = force(r.R)
        r.part2(dt, F)
        if (n + 1) % 10 == 0:
            U = 0.5 * k * np.sum((r.R - R0) ** 2)
            energy.append([U, *r.kinetic()])
            Rs.append(r.R.copy()); Vs.append(r.V.copy())
    return dict(masses=s.masses, body_indices=s.body_indices, R0=s.positions, V0=s.velocities, k=k, dt=dt, mode=mode,
                nsteps=nsteps, energy=np.array(energy), R=np.array(Rs), V=np.array(Vs), dof=r.num_dof)


def single_bond(nsteps=1000, dt=0.01):
    """The reference's own known-answer test (tests/TestRigidBodyIntegrator.h:49-83): two free atoms
    of mass 2 joined by a harmonic bond (r0 1.5, k 1), dt 0.01, 1000 steps."""
    masses = np.array([2.0, 2.0])
    bidx = np.array([0, 0], dtype=np.int32)
    R = np.array([[-1.0, 0, 0], [1.0, 0, 0]])
    V = np.zeros((2, 3))

    def force(x):
        d = x[1] - x[0]
        r = np.linalg.norm(d)
        f = -1.0 * (r - 1.5) * d / r
        return quantise(np.array([-f, f]))

    ref = Reference(masses, bidx, 0)
    F = force(R)
    ref.setup(R, V, F)
    Rs, Vs = [R.copy()], [V.copy()]
    for n in range(nsteps):
        ref.part1(dt, F)
        F = force(ref.R)
        ref.part2(dt, F)
        Rs.append(ref.R.copy()); Vs.append(ref.V.copy())
    return dict(masses=masses, body_indices=bidx, R0=R, V0=V, dt=dt, nsteps=nsteps, R=np.array(Rs), V=np.array(Vs))


def linear_bodies(mode=10, nsteps=20, dt=0.002):
    """Ten rigid CO2-like molecules (reference keeps a transposed principal frame for them)."""
    rng = np.random.default_rng(0)
    R, M, B = [], [], []
    for k in range(10):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        c = rng.uniform(0, 3, size=3)
        R += [c - 0.116 * u, c, c + 0.116 * u]
        M += [16.0, 12.0, 16.0]
        B += [k + 1] * 3
    R, M, B = np.array(R), np.array(M), np.array(B, dtype=np.int32)
    V = rng.normal(size=R.shape) * 0.3
    F = quantise(rng.normal(size=R.shape) * 100)
    ref = Reference(M, B, mode)
    ref.setup(R, V, F)
    for n in range(nsteps):
        ref.part1(dt, F)
        ref.part2(dt, F)
    return dict(masses=M, body_indices=B, R0=R, V0=V, F=F, dt=dt, mode=mode, nsteps=nsteps, R=ref.R, V=ref.V,
                ke=ref.kinetic(), dof=ref.num_dof)


def near_degenerate(mode, dt, nsteps=100, sd=50.0):
    """48 planar 4-atom crosses whose two in-plane principal moments differ by a factor 1+eps, eps
    log-uniform in [1e-4, 1e-2], built in their principal frame (inertia tensors diagonal in the
    space frame, where the reference's eigen-solver is exact), 300 K velocities, fixed seeded
    Gaussian forces of standard deviation sd (kJ/mol/nm); final positions, velocities and kinetic
    energies after nsteps steps of dt."""
    s = W.near_degenerate_system(48, 0, eps_range=(1e-4, 1e-2), seed=17, principal_frame=True)
    F = quantise(W.gaussian_forces(s.num_atoms, seed=9, sd=sd))
    r = Reference(s.masses, s.body_indices, mode)
    r.setup(s.positions, s.velocities, F)
    for n in range(nsteps):
        r.part1(dt, F)
        r.part2(dt, F)
    return dict(masses=s.masses, body_indices=s.body_indices, R0=s.positions, V0=s.velocities, F=F, dt=dt,
                mode=mode, nsteps=nsteps, eps=s.eps, R=r.R, V=r.V, ke=r.kinetic(), dof=r.num_dof)


def singleton_dof(ncases=12):
    """Degrees of freedom the reference reports for systems that hold one-atom bodies (indices used
    once, which it keeps as bodies), linear bodies, free and massless atoms: ncases seeded systems,
    stored as concatenated arrays with atom offsets."""
    rng = np.random.default_rng(41)
    M, B, R, V, off, dof = [], [], [], [], [0], []
    for c in range(ncases):
        s = W.mixed_system(n_bodies=6, n_free=3, fractions=(0.5, 0.3, 0.2), seed=100 + c)
        ns = 1 + c % 4
        m = np.concatenate([s.masses, rng.uniform(1, 20, ns), [16.0, 12.0, 16.0], [0.0]])
        b = np.concatenate([s.body_indices, 1000 + np.arange(ns), [900, 900, 900], [0]]).astype(np.int32)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        x = np.concatenate([s.positions, rng.uniform(-3, 3, (ns, 3)), 1.0 + np.outer([-0.116, 0, 0.116], u),
                            rng.uniform(0, 2, (1, 3))])
        v = rng.normal(size=x.shape)
        r = Reference(m, b, 0)
        r.setup(x, v, np.zeros_like(x))
        M.append(m); B.append(b); R.append(x); V.append(v); off.append(off[-1] + len(m)); dof.append(r.num_dof)
    return dict(masses=np.concatenate(M), body_indices=np.concatenate(B), R0=np.concatenate(R), V0=np.concatenate(V),
                offsets=np.array(off), dof=np.array(dof))


def main():
    only = sys.argv[1:]  # optional case names; all cases by default
    if not reference_available():
        sys.exit("oracle/_ref/librefrb.so missing: build it with `make -C oracle ref`")
    cases = {f"water64_mode{m}": water_fixed_force(m) for m in (0, 1, 10)}
    for m in (0, 10):
        cases[f"water64_sd50_mode{m}"] = water_fixed_force(m, sd=50.0)
    cases["water27_tether_mode0"] = water_tether(0)
    cases["water27_tether_mode4"] = water_tether(4)
    cases["single_bond"] = single_bond()
    cases["linear10_mode10"] = linear_bodies(10)
    cases["singleton_dof"] = singleton_dof()
    for m in (0, 1, 4, 16):
        for dt_fs in (1, 4):
            cases[f"cross48_mode{m}_dt{dt_fs}fs"] = near_degenerate(m, dt_fs * 1e-3)
    for name, data in cases.items():
        if only and name not in only:
            continue
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print(f"{path}: {os.path.getsize(path)} bytes")


if __name__ == "__main__":
    main()
