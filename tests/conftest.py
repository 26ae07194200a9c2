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
