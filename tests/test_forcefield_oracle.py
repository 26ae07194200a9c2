"""The FP64 force-field checker itself (oracle/ff_oracle.c), on the CPU.

Forces must be minus the gradient of the energy (central differences, away from the cutoff
discontinuity of the unshifted LJ term), sum to zero in each box (pair forces are equal and
opposite), leave pairs of one rigid body out, and not depend on the other systems of a batch.
"""
import numpy as np

from openmm_rigidbody_plugin_gb300 import workloads as W


def _system(n=27, seed=1):
    s = W.water_box(n, seed=seed)
    q, sg, ep = W.nonbonded(s)
    return s, q, sg, ep


def _ff(oracle_mod, systems):
    offs = np.concatenate([[0], np.cumsum([s.num_atoms for s, *_ in systems])])
    cat = lambda k: np.concatenate([x[k] for x in systems])
    pos = np.concatenate([s.positions for s, *_ in systems])
    body = np.concatenate([s.body_indices + 1000 * i * (s.body_indices > 0) for i, (s, *_) in enumerate(systems)])
    boxes = [s.box for s, *_ in systems]
    return oracle_mod.lj_rf(offs, boxes, [W.cutoff_for(b) for b in boxes], pos, cat(1), cat(2), cat(3), body)


def test_forces_are_minus_energy_gradient(oracle_mod):
    s, q, sg, ep = _system(64, seed=3)
    rc = W.cutoff_for(s.box)
    f, e = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], s.positions, q, sg, ep, s.body_indices)
    rng = np.random.default_rng(0)
    h = 1e-6
    checked = 0
    for i in rng.choice(s.num_atoms, 12, replace=False):
        for c in range(3):
            p = s.positions.copy()
            p[i, c] += h
            _, ep_ = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], p, q, sg, ep, s.body_indices)
            p[i, c] -= 2 * h
            _, em_ = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], p, q, sg, ep, s.body_indices)
            num = -(ep_[0] - em_[0]) / (2 * h)
            if abs(ep_[0] - em_[0]) > 1.0:  # a pair crossed the cutoff: the LJ term is not shifted
                continue
            assert abs(num - f[i, c]) < 1e-4 * max(1.0, abs(f[i, c])), (i, c, num, f[i, c])
            checked += 1
    assert checked >= 30


def test_net_force_vanishes_and_exclusions_apply(oracle_mod):
    s, q, sg, ep = _system(64, seed=4)
    rc = W.cutoff_for(s.box)
    f, e = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], s.positions, q, sg, ep, s.body_indices)
    assert np.max(np.abs(f.sum(0))) < 1e-9 * np.max(np.abs(f))
    # without the exclusions the intra-water O-H and H-H Coulomb terms dominate
    f2, e2 = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], s.positions, q, sg, ep, np.zeros(s.num_atoms))
    assert abs(e2[0] - e[0]) > 100.0


def test_systems_are_independent(oracle_mod):
    a = _system(27, seed=5)
    b = _system(64, seed=6)
    fab, eab = _ff(oracle_mod, [a, b])
    fa, ea = _ff(oracle_mod, [a])
    fb, eb = _ff(oracle_mod, [b])
    np.testing.assert_array_equal(fab[:a[0].num_atoms], fa)
    np.testing.assert_array_equal(fab[a[0].num_atoms:], fb)
    assert eab[0] == ea[0] and eab[1] == eb[0]


def test_selected_atoms_match_full_evaluation(oracle_mod):
    s, q, sg, ep = _system(64, seed=7)
    rc = W.cutoff_for(s.box)
    f, _ = oracle_mod.lj_rf([0, s.num_atoms], [s.box], [rc], s.positions, q, sg, ep, s.body_indices)
    sel = np.array([0, 5, 17, 100, s.num_atoms - 1])
    fs = oracle_mod.lj_rf_atoms(sel, s.box, rc, s.positions, q, sg, ep, s.body_indices)
    np.testing.assert_allclose(fs, f[sel], rtol=1e-12, atol=1e-10)
