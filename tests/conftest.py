import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and librbx.so")


@pytest.fixture(scope="session")
def oracle_mod():
    import subprocess

    import oracle
    if not os.path.exists(oracle.ORACLE_SO):
        oracle.build()
    else:  # rebuild the C restatement if its sources are newer (make checks)
        subprocess.run(["make", "-s", "-C", oracle.HERE, "oracle"], check=True)
    return oracle


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
            return {k: z[k] for k in z.files}
    return load


def rel_err(a, b):
    """Normwise relative difference max|a-b| / max|b| used by every parity test."""
    import numpy as np
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def tether_system(seed=3, n_bodies=20, n_free=10, k=2000.0):
    """Rigid bodies of 3-5 atoms and free atoms, each atom tied by a harmonic spring (stiffness k,
    kJ/mol/nm^2) to a point near its start: a smooth force field with torques, for energy checks.
    Returns masses, body indices, positions, velocities and force(R) -> (F, U)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    masses, bidx, pos = [], [], []
    for b in range(n_bodies):
        c = rng.uniform(0, 3, 3)
        for _ in range(3 + b % 3):
            masses.append(rng.uniform(1, 16))
            bidx.append(b + 1)
            pos.append(c + rng.normal(0, 0.1, 3))
    for _ in range(n_free):
        masses.append(rng.uniform(1, 16))
        bidx.append(0)
        pos.append(rng.uniform(0, 3, 3))
    masses, bidx, x0 = np.array(masses), np.array(bidx, dtype=np.int32), np.array(pos)
    anchor = x0 + rng.normal(0, 0.05, x0.shape)
    v0 = rng.normal(0, 2, x0.shape) / np.sqrt(masses)[:, None]

    def force(R):
        d = R - anchor
        return -k * d, 0.5 * k * float(np.sum(d * d))
    return masses, bidx, x0, v0, force


def constrained_system(seed=4, n_bodies=12, n_pairs=15, bond=0.1, k=2000.0):
    """The bodies of tether_system plus free diatomic molecules whose bond length is constrained
    (pairs of free atoms at distance `bond`), all tethered. Returns masses, body indices, positions,
    velocities (bond-relative components removed), force(R) -> (F, U), constrained pairs [n, 2] and
    their distances."""
    import numpy as np
    from openmm_rigidbody_plugin_gb300.api import rattle_velocities
    m, bidx, x, v, _ = tether_system(seed=seed, n_bodies=n_bodies, n_free=0, k=k)
    rng = np.random.default_rng(seed + 100)
    u = rng.normal(size=(n_pairs, 3))
    u /= np.linalg.norm(u, axis=1)[:, None]
    c = rng.uniform(0, 3, (n_pairs, 3))
    xp = np.stack([c + 0.5 * bond * u, c - 0.5 * bond * u], axis=1).reshape(-1, 3)
    mp = rng.uniform(1, 16, 2 * n_pairs)
    n0 = len(m)
    masses = np.concatenate([m, mp])
    bidx = np.concatenate([bidx, np.zeros(2 * n_pairs, dtype=bidx.dtype)])
    x0 = np.concatenate([x, xp])
    pairs = n0 + np.arange(2 * n_pairs).reshape(-1, 2)
    dist = np.full(n_pairs, bond)
    v0 = np.concatenate([v, rng.normal(0, 2, (2 * n_pairs, 3)) / np.sqrt(mp)[:, None]])
    v0 = rattle_velocities(x0, v0, 1.0 / masses, pairs, 1e-12)
    anchor = x0 + rng.normal(0, 0.05, x0.shape)

    def force(R):
        d = R - anchor
        return -k * d, 0.5 * k * float(np.sum(d * d))
    return masses, bidx, x0, v0, force, pairs, dist


def oracle_constrained_run(oracle_mod, system, dt, nsteps, mode=0, tol=1e-5):
    """The Reference platform's step with constraints (ReferenceRigidBodyKernels.cpp:82-108): part1,
    SHAKE from the pre-step positions, forces, part2 (with its (R - savedPos)/dt term), RATTLE."""
    from openmm_rigidbody_plugin_gb300.api import rattle_velocities, shake
    masses, bidx, x0, v0, force, pairs, dist = system
    w = 1.0 / masses
    o = oracle_mod.Oracle(masses, bidx, mode=mode, robust=True)
    o.setup(x0, v0, force(x0)[0])
    for _ in range(nsteps):
        xold = o.R.copy()
        o.part1(dt, force(o.R)[0])
        o.R[:] = shake(xold, o.R, w, pairs, dist, tol)
        o.part2(dt, force(o.R)[0])
        o.V[:] = rattle_velocities(o.R, o.V, w, pairs, tol)
    return o
