"""CUDA path (through the C ABI) against the reference's golden vectors and the oracle.

Tolerances (normwise relative, max|gpu - ref| / max|ref|), from the target "positions and
velocities within 1e-6 relative after 100 steps in mixed/FP64":
  double: positions 1e-9, velocities 1e-8 after 100 steps (FP64 throughout; differences are
          rounding order)
  mixed:  positions 1e-6, velocities 1e-6 after 100 steps under moderate forces (seeded Gaussian
          forces of sd 50 kJ/mol/nm, harmonic tethers). With FIXED forces the FP32 rounding of the
          per-atom forces and of the stored body-frame coordinates repeats identically every step
          and its effect grows linearly: in the FP64 oracle, FP32-rounded fixed forces alone move
          the velocities by 3.8e-7 after 100 steps and FP32-rounded body-frame coordinates alone by
          3.2e-7, so the fixed-force cases allow 1.5e-6 for velocities (positions stay at 1e-6);
          position-dependent forces (tethers) are held to 1e-6. Under the sd 500 kJ/mol/nm forces of the
          integrator-only benchmark each rigid body is a strongly driven top whose trajectory
          amplifies any perturbation exponentially: in the FP64 oracle itself a 1e-7 relative
          force perturbation (FP32 rounding) grows to 3e-8 after 20 steps, 3e-6 after 50 and
          2e-5 after 100. Those cases are compared after 20 steps (positions 1e-6, velocities
          3e-6), where the comparison still measures the implementation, not the chaos.
"""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {"double": (1e-9, 1e-8, 1e-9), "mixed": (1e-6, 1e-6, 1e-6)}
TOL_FIXED = {"double": (1e-9, 1e-8, 1e-9), "mixed": (1e-6, 1.5e-6, 1e-6)}  # sd 50, fixed forces
TOL_STRONG = {"double": (1e-9, 1e-8, 1e-9), "mixed": (1e-6, 3e-6, 1e-6)}  # sd 500 forces
STEPS_STRONG = {"double": 100, "mixed": 20}


@pytest.fixture(scope="module")
def rbx():
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import build, kernel
    build.build_library()
    return kernel


def make(rbx, masses, bidx, R, V, mode, prec, location=None):
    k = rbx.IntegratorKernel(masses, bidx, rotation_mode=mode, precision=prec)
    buf = rbx.DeviceBuffers(len(masses), precision=prec)
    if location is not None:
        buf.location = np.asarray(location)
        k.set_atom_locations(location)
    buf.set_positions(R)
    buf.set_velocities(V, masses)
    k.upload_state(R, V)
    return k, buf


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("mode", [0, 1, 10])
def test_water_fixed_force_vs_reference(rbx, golden, mode, prec):
    g = golden(f"water64_mode{mode}")
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], mode, prec)
    buf.set_forces(g["F"])
    dt = float(g["dt"])
    # the reference counts one degree of freedom per free atom (RigidBodySystem.cpp:130), the
    # library three
    assert k.num_dof == int(g["dof"]) + 2 * k.num_free
    nsteps = STEPS_STRONG[prec]
    for n in range(nsteps):
        k.part1(buf, dt)
        k.part2(buf, dt)
    snap = nsteps // 10 - 1
    tp, tv, tk = TOL_STRONG[prec]
    assert rel_err(buf.get_positions(), g["R"][snap]) < tp
    assert rel_err(buf.get_velocities(), g["V"][snap]) < tv
    np.testing.assert_allclose(k.kinetic_energies(buf), g["ke"][snap], rtol=tk)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("mode", [0, 10])
def test_water_moderate_force_100_steps(rbx, golden, mode, prec):
    """The 1e-6-after-100-steps criterion, sd 50 kJ/mol/nm forces."""
    g = golden(f"water64_sd50_mode{mode}")
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], mode, prec)
    buf.set_forces(g["F"])
    dt = float(g["dt"])
    for n in range(int(g["nsteps"])):
        k.part1(buf, dt)
        k.part2(buf, dt)
    tp, tv, tk = TOL_FIXED[prec]
    assert rel_err(buf.get_positions(), g["R"][-1]) < tp
    assert rel_err(buf.get_velocities(), g["V"][-1]) < tv
    np.testing.assert_allclose(k.kinetic_energies(buf), g["ke"][-1], rtol=tk)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("mode", [0, 10])
def test_fused_steps_equal_split_steps(rbx, golden, mode, prec):
    """part1, fused x (n-1), part2 == n x (part1, part2) with fixed forces."""
    g = golden(f"water64_sd50_mode{mode}")
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], mode, prec)
    buf.set_forces(g["F"])
    dt, n = float(g["dt"]), int(g["nsteps"])
    k.part1(buf, dt)
    for _ in range(n - 1):
        k.fused(buf, dt)
    k.part2(buf, dt)
    tp, tv, tk = TOL_FIXED[prec]
    assert rel_err(buf.get_positions(), g["R"][-1]) < tp
    assert rel_err(buf.get_velocities(), g["V"][-1]) < tv
    np.testing.assert_allclose(k.kinetic_energies(buf), g["ke"][-1], rtol=tk)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("name", ["water27_tether_mode0", "water27_tether_mode4"])
def test_position_dependent_forces_vs_reference(rbx, golden, name, prec):
    """Harmonic tethers F = -k (R - R0), k = 1000 kJ/mol/nm^2, 200 steps. The tether force depends
    on displacements of 0.01-0.1 nm, so the ~1e-8 nm rounding of an FP32 position rebuild (mixed
    precision rebuilds r + At(q) d with FP32 arithmetic) is a ~1e-6 relative force error every
    step; mixed velocities are therefore held to 5e-6 here, positions and energies to 1e-6."""
    g = golden(name)
    kk, dt, R0 = float(g["k"]), float(g["dt"]), g["R0"]
    k, buf = make(rbx, g["masses"], g["body_indices"], R0, g["V0"], int(g["mode"]), prec)
    buf.set_forces(-kk * (R0 - R0))
    for n in range(int(g["nsteps"])):
        k.part1(buf, dt)
        R = buf.get_positions()
        buf.set_forces(-kk * (R - R0))
        k.part2(buf, dt)
        if (n + 1) % 10 == 0:
            j = (n + 1) // 10 - 1
            U = 0.5 * kk * np.sum((R - R0) ** 2)
            np.testing.assert_allclose([U, *k.kinetic_energies(buf)], g["energy"][j], rtol=TOL[prec][2])
    assert rel_err(buf.get_positions(), g["R"][-1]) < TOL[prec][0]
    assert rel_err(buf.get_velocities(), g["V"][-1]) < (5e-6 if prec == "mixed" else TOL[prec][1])


def test_single_bond_free_atoms(rbx, golden):
    """Free atoms only (the reference's testSingleBond), mixed precision, against the reference run."""
    g = golden("single_bond")
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], 0, "mixed")
    dt = float(g["dt"])

    def force(x):
        d = x[1] - x[0]
        r = np.linalg.norm(d)
        f = -1.0 * (r - 1.5) * d / r
        return np.array([-f, f])

    buf.set_forces(force(g["R0"]))
    for n in range(int(g["nsteps"])):
        k.part1(buf, dt)
        buf.set_forces(force(buf.get_positions()))
        k.part2(buf, dt)
    np.testing.assert_allclose(buf.get_positions(), g["R"][-1], atol=1e-9)
    np.testing.assert_allclose(buf.get_velocities(), g["V"][-1], atol=1e-9)


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
def test_single_bond_known_answer_in_every_precision(rbx, golden, prec):
    """The reference's testSingleBond (tests/TestRigidBodyIntegrator.h:49-83), which its CUDA tests
    run in single, mixed and double precision (platforms/cuda/tests/CMakeLists.txt:20-22): two free
    atoms of mass 2 on a harmonic bond (r0 1.5, k 1) against the analytic oscillator, positions and
    velocities within 0.02 and energy within 0.01 at every step, 1000 steps of 0.01 (time 10.0)."""
    g = golden("single_bond")
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], 0, prec)
    dt, nsteps, m = float(g["dt"]), int(g["nsteps"]), np.asarray(g["masses"])

    def force(x):
        d = x[1] - x[0]
        r = np.linalg.norm(d)
        f = -1.0 * (r - 1.5) * d / r
        return np.array([-f, f])

    def energy(x, v):
        return 0.5 * (np.linalg.norm(x[1] - x[0]) - 1.5) ** 2 + 0.5 * np.sum(m[:, None] * v ** 2)

    e0 = energy(g["R0"], g["V0"])
    buf.set_forces(force(g["R0"]))
    for n in range(nsteps):
        k.part1(buf, dt)
        buf.set_forces(force(buf.get_positions()))
        k.part2(buf, dt)
        x, v = buf.get_positions(), buf.get_velocities()
        t = (n + 1) * dt
        dist, speed = 1.5 + 0.5 * np.cos(t), -0.5 * np.sin(t)
        np.testing.assert_allclose(x, [[-0.5 * dist, 0, 0], [0.5 * dist, 0, 0]], atol=0.02)
        np.testing.assert_allclose(v, [[-0.5 * speed, 0, 0], [0.5 * speed, 0, 0]], atol=0.02)
        assert abs(energy(x, v) - e0) < 0.01
    assert abs(nsteps * dt - 10.0) < 1e-12


def _mixed_case(seed=3):
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=300, n_free=40, fractions=(0.5, 0.3, 0.2), seed=seed)
    F = np.round(W.gaussian_forces(s.num_atoms, seed=5) * 2.0 ** 32) / 2.0 ** 32
    return s, F


@pytest.mark.parametrize("prec,size", [("mixed", 1024), ("single", 1024), ("double", 512)])
def test_largest_body_vs_robust_oracle(rbx, oracle_mod, prec, size):
    """A body filling a whole tile (1024 atoms in single/mixed, 512 in double), with waters and free
    atoms around it, against the robust FP64 oracle: 20 steps under sd 50 kJ/mol/nm forces."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    rng = np.random.default_rng(31)
    w = W.water_box(27, seed=3)
    blob = rng.normal(0, 0.6, (size, 3)) + 5.0
    masses = np.concatenate([w.masses, rng.uniform(1, 16, size), np.full(7, 39.95)])
    bidx = np.concatenate([w.body_indices, np.full(size, w.body_indices.max() + 1), np.zeros(7, dtype=int)])
    R = np.concatenate([w.positions, blob, rng.uniform(0, 3, (7, 3))])
    V = rng.normal(0, 0.3, R.shape)
    F = W.gaussian_forces(len(masses), seed=8, sd=50.0)
    k, buf = make(rbx, masses, bidx, R, V, 0, prec)
    buf.set_forces(F)
    o = oracle_mod.Oracle(masses, bidx, mode=0, robust=True)
    o.setup(R, V, F)
    for _ in range(20):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
        o.part1(0.002, F)
        o.part2(0.002, F)
    tol = {"double": 1e-9, "mixed": 1e-6, "single": 2e-4}[prec]
    assert rel_err(buf.get_positions(), o.R) < tol
    assert rel_err(buf.get_velocities(), o.V) < 10 * tol


def _blobs(sizes, seed):
    """Rigid bodies of the given atom counts (random clouds, 0.3 nm spread), one per id from 1."""
    rng = np.random.default_rng(seed)
    R = np.concatenate([rng.normal(0, 0.3, (n, 3)) + rng.uniform(0, 6, 3) for n in sizes])
    bidx = np.concatenate([np.full(n, i + 1) for i, n in enumerate(sizes)])
    return R, bidx, rng.uniform(1, 16, len(bidx)), rng.normal(0, 0.3, R.shape)


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("mode", [0, 10])
def test_many_large_bodies_per_tile(rbx, oracle_mod, prec, mode):
    """Bodies of more than 32 atoms are summed by a warp each. Twelve of 33-40 atoms share one tile
    (more large bodies than warps, so a warp takes several), among 27 waters: 20 steps against the
    robust oracle under sd 50 forces; then the same bodies without the waters (other tiles, other
    warps): their trajectories are bit-identical."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    sizes = [33, 40, 34, 39, 35, 38, 36, 37, 33, 40, 34, 39]
    Rb, bb, mb, Vb = _blobs(sizes, seed=41)
    w = W.water_box(27, seed=5)
    R = np.concatenate([w.positions, Rb])
    bidx = np.concatenate([w.body_indices, bb + w.body_indices.max()])
    masses = np.concatenate([w.masses, mb])
    V = np.concatenate([w.velocities, Vb])
    F = np.round(W.gaussian_forces(len(masses), seed=9, sd=50.0) * 2.0 ** 32) / 2.0 ** 32
    k, buf = make(rbx, masses, bidx, R, V, mode, prec)
    buf.set_forces(F)
    o = oracle_mod.Oracle(masses, bidx, mode=mode, robust=True)
    o.setup(R, V, F)
    for _ in range(20):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
        o.part1(0.002, F)
        o.part2(0.002, F)
    tol = {"double": 1e-9, "mixed": 1e-6}[prec]
    x, v = buf.get_positions(), buf.get_velocities()
    assert rel_err(x, o.R) < tol
    assert rel_err(v, o.V) < 10 * tol
    n = len(w.masses)
    k2, buf2 = make(rbx, mb, bb, Rb, Vb, mode, prec)
    buf2.set_forces(F[n:])
    for _ in range(20):
        k2.part1(buf2, 0.002)
        k2.part2(buf2, 0.002)
    assert np.array_equal(buf2.get_positions(), x[n:])
    assert np.array_equal(buf2.get_velocities(), v[n:])


@pytest.mark.parametrize("prec", ["double", "mixed"])
@pytest.mark.parametrize("mode", [0, 10])
def test_mixed_body_types_vs_robust_oracle(rbx, oracle_mod, mode, prec):
    """Waters, spherical-top tetrahedra and symmetric-top rings (the reference gives NaN or
    distorted bodies for the last two): parity against the robust FP64 oracle."""
    s, F = _mixed_case()
    k, buf = make(rbx, s.masses, s.body_indices, s.positions, s.velocities, mode, prec)
    buf.set_forces(F)
    o = oracle_mod.Oracle(s.masses, s.body_indices, mode=mode, robust=True)
    o.setup(s.positions, s.velocities, F)
    assert k.num_dof == o.num_dof
    dt = 0.002
    for n in range(STEPS_STRONG[prec]):
        k.part1(buf, dt)
        k.part2(buf, dt)
        o.part1(dt, F)
        o.part2(dt, F)
    tp, tv, tk = TOL_STRONG[prec]
    assert rel_err(buf.get_positions(), o.R) < tp
    assert rel_err(buf.get_velocities(), o.V) < tv
    np.testing.assert_allclose(k.kinetic_energies(buf), o.kinetic(), rtol=tk)


@pytest.mark.parametrize("prec", ["double", "mixed"])
def test_atom_reordering_is_transparent(rbx, golden, prec):
    """Device slots permuted as OpenMM's reordering would: identical user-order results."""
    g = golden("water64_sd50_mode0")
    perm = np.random.default_rng(7).permutation(len(g["masses"]))
    k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], 0, prec, location=perm)
    buf.set_forces(g["F"])
    for _ in range(int(g["nsteps"])):
        k.part1(buf, float(g["dt"]))
        k.part2(buf, float(g["dt"]))
    assert rel_err(buf.get_positions(), g["R"][-1]) < TOL_FIXED[prec][0]
    assert rel_err(buf.get_velocities(), g["V"][-1]) < TOL_FIXED[prec][1]


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
def test_reordering_mid_run_is_bit_exact(rbx, prec):
    """Atoms moved to new slots between steps (buffers moved as OpenMM moves them, then
    rbx_set_atom_locations): the library re-plans its body order for the new slots and carries
    the body state over bit for bit, so the trajectory equals an unmoved run exactly."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=3000, n_free=400, seed=13)
    F = W.gaussian_forces(s.num_atoms, seed=4, sd=50.0)
    runs = []
    for move in (False, True):
        k, buf = make(rbx, s.masses, s.body_indices, s.positions, s.velocities, 0, prec)
        buf.set_forces(F)
        rng = np.random.default_rng(21)
        for n in range(12):
            if move and n % 4 == 2:
                loc = rng.permutation(s.num_atoms)
                buf.relocate(loc)
                k.set_atom_locations(loc)
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
        runs.append((buf.get_positions(), buf.get_velocities(), k.body_state()))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["mixed", "double"])
def test_reordering_into_padded_slots_is_bit_exact(rbx, prec):
    """OpenMM pads its atom buffers: slots above the atom count, and gaps between used slots. The
    re-plan on the device sorts by slot across the whole slot range."""
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=2000, n_free=300, seed=17)
    n = s.num_atoms
    F = W.gaussian_forces(n, seed=6, sd=50.0)
    runs = []
    for move in (False, True):
        k = rbx.IntegratorKernel(s.masses, s.body_indices, rotation_mode=4, precision=prec)
        buf = rbx.DeviceBuffers(n, precision=prec, stride=3 * n + 32)
        buf.set_positions(s.positions)
        buf.set_velocities(s.velocities, s.masses)
        k.upload_state(s.positions, s.velocities)
        buf.set_forces(F)
        rng = np.random.default_rng(5)
        for step in range(9):
            if move and step % 3 == 1:
                loc = rng.choice(3 * n + 32, size=n, replace=False)
                buf.relocate(loc)
                k.set_atom_locations(loc)
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
        runs.append((buf.get_positions(), buf.get_velocities(), k.body_state(), k.kinetic_energies(buf)))
    for a, b in zip(runs[0][:3], runs[1][:3]):
        assert np.array_equal(a, b)
    # the energy sums run in library order, which the re-plan changes: equal to rounding
    np.testing.assert_allclose(runs[1][3], runs[0][3], rtol=1e-13)


def test_invalid_locations_are_rejected_and_change_nothing(rbx):
    from openmm_rigidbody_plugin_gb300 import _lib
    from openmm_rigidbody_plugin_gb300 import workloads as W
    s = W.mixed_system(n_bodies=500, n_free=50, seed=19)
    n = s.num_atoms
    F = W.gaussian_forces(n, seed=7, sd=50.0)
    runs = []
    for bad in (False, True):
        k, buf = make(rbx, s.masses, s.body_indices, s.positions, s.velocities, 0, "mixed")
        buf.set_forces(F)
        for step in range(4):
            if bad and step == 2:
                dup = np.arange(n)
                dup[7] = dup[3]  # one slot for two atoms
                with pytest.raises(_lib.RbxError, match="two atoms"):
                    k.set_atom_locations(dup)
                neg = np.arange(n)
                neg[11] = -1
                with pytest.raises(_lib.RbxError, match="negative location for atom 11"):
                    k.set_atom_locations(neg)
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
        runs.append((buf.get_positions(), buf.get_velocities(), k.body_state()))
    for a, b in zip(runs[0], runs[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["single", "mixed", "double"])
def test_host_buffer_step(rbx, golden, prec):
    """rbx_step_host (host arrays in, host arrays out) against the reference."""
    g = golden("water64_sd50_mode10")
    k = rbx.IntegratorKernel(g["masses"], g["body_indices"], rotation_mode=10, precision=prec)
    k.context_set_state(g["R0"], g["V0"])
    R = np.zeros_like(g["R0"])
    V = np.zeros_like(g["V0"])
    F = np.ascontiguousarray(g["F"])
    k.step_host(int(g["nsteps"]), float(g["dt"]), F, R, V)
    tol = {"single": 1e-4, "mixed": 1e-6, "double": 1e-9}[prec]
    assert rel_err(R, g["R"][-1]) < tol
    assert rel_err(V, g["V"][-1]) < tol * 10
    np.testing.assert_allclose(k.context_kinetic_energies(), g["ke"][-1], rtol=tol * 10)


@pytest.mark.parametrize("prec", ["single", "mixed"])
@pytest.mark.parametrize("mode", [0, 10])
def test_tile_shapes_give_identical_results(rbx, prec, mode):
    """The step kernel's two tile shapes (256 threads / 1024 body atoms and 128 / 512) integrate
    every body alike: 600 bodies of three kinds, a 32-atom body and 40 free atoms, 20 split and 10
    fused steps, with the shape switched mid-run in one of the runs. Bodies of more than 32 atoms
    (summed by a warp), and double precision, have the wide shape only."""
    from openmm_rigidbody_plugin_gb300 import _lib, workloads as W
    s = W.mixed_system(n_bodies=600, n_free=40, fractions=(0.5, 0.3, 0.2), seed=8)
    Rb, bb, mb, Vb = _blobs([32], seed=2)
    R = np.concatenate([s.positions, Rb])
    bidx = np.concatenate([s.body_indices, bb + s.body_indices.max()])
    masses = np.concatenate([s.masses, mb])
    V = np.concatenate([s.velocities, Vb])
    F = np.round(W.gaussian_forces(len(masses), seed=4, sd=50.0) * 2.0 ** 32) / 2.0 ** 32
    outs = []
    for shape in ((256, 256), (128, 128), (256, 128)):
        k, buf = make(rbx, masses, bidx, R, V, mode, prec)
        assert k.tile_threads == 256
        k.tile_threads = shape[0]
        buf.set_forces(F)
        for n in range(20):
            if n == 10:
                k.tile_threads = shape[1]
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
        k.part1(buf, 0.002)
        for _ in range(10):
            k.fused(buf, 0.002)
        k.part2(buf, 0.002)
        assert k.tile_threads == shape[1]
        outs.append((buf.get_positions(), buf.get_velocities(), k.kinetic_energies(buf)))
    for out in outs[1:]:
        for a, b in zip(outs[0], out):
            assert np.array_equal(a, b)
    big = np.concatenate([bidx, np.full(33, bidx.max() + 1)])
    k = rbx.IntegratorKernel(np.concatenate([masses, np.ones(33)]), big, rotation_mode=mode, precision=prec)
    with pytest.raises(_lib.RbxError, match="bodies of at most 32 atoms"):
        k.tile_threads = 128
    k = rbx.IntegratorKernel(masses, bidx, rotation_mode=mode, precision="double")
    with pytest.raises(_lib.RbxError, match="one tile shape"):
        k.tile_threads = 128


def test_determinism(rbx, golden):
    """Two identical runs give bit-identical results (fixed-order reductions, no atomics)."""
    g = golden("water64_mode0")
    outs = []
    for _ in range(2):
        k, buf = make(rbx, g["masses"], g["body_indices"], g["R0"], g["V0"], 0, "mixed")
        buf.set_forces(g["F"])
        for _ in range(20):
            k.part1(buf, 0.002)
            k.part2(buf, 0.002)
        outs.append((buf.get_positions(), buf.get_velocities(), k.kinetic_energies(buf)))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", ["mixed", "double"])
def test_pipelined_host_steps_equal_synchronous_ones(rbx, golden, prec):
    """rbx_step_host_async (copies overlapped across calls) gives the synchronous results."""
    import torch
    g = golden("water64_sd50_mode0")
    rng = np.random.default_rng(3)
    forces = [np.ascontiguousarray(g["F"] * (1.0 + 0.1 * k)) for k in range(5)]
    out = {}
    for mode in ("sync", "async"):
        k = rbx.IntegratorKernel(g["masses"], g["body_indices"], rotation_mode=0, precision=prec)
        k.context_set_state(g["R0"], g["V0"])
        pinned = [(torch.zeros((len(g["masses"]), 3), dtype=torch.float64).pin_memory().numpy(),
                   torch.zeros((len(g["masses"]), 3), dtype=torch.float64).pin_memory().numpy()) for _ in forces]
        for f, (x, v) in zip(forces, pinned):
            if mode == "sync":
                k.step_host(2, 0.002, f, x, v)
            else:
                k.step_host_async(2, 0.002, f, x, v)
        if mode == "async":
            k.step_host_wait()
        out[mode] = [(x.copy(), v.copy()) for x, v in pinned]
    for (xs, vs), (xa, va) in zip(out["sync"], out["async"]):
        assert np.array_equal(xs, xa) and np.array_equal(vs, va)
