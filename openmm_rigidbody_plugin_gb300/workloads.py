"""Seeded synthetic systems of rigid bodies and free atoms (units: nm, ps, amu, kJ/mol).

No public dataset is involved: every workload is generated here from a seed.

* ``water_box`` -- rigid 3-site waters on a cubic lattice at 1 g/cm^3, random orientations,
  Maxwell-Boltzmann velocities (the 512-water plain-method case).
* ``mixed_system`` -- the single-large-system case: 70 % waters, 20 % 5-atom tetrahedra
  (C + 4 H at 0.109 nm, masses 12/1), 10 % 12-atom planar rings (6 C on a 0.14 nm hexagon,
  6 H radially outside at 0.109 nm, masses 12.011/1.008), plus free LJ atoms (mass 39.95).
  Molecules sit on a cubic lattice at 1 g/cm^3 with random orientations, except that the rings
  take sites two lattice spacings apart and a staggered orientation (plane normal along a random
  body diagonal, carbons between the neighbours), so that no carbons of neighbouring molecules
  start inside each other's Lennard-Jones core.
* ``gaussian_forces`` -- seeded per-atom Gaussian forces (sd 500 kJ/mol/nm by default) for
  integrator-only timing.
* ``batch_systems`` -- many independent mixed systems, each in its own box at 1 g/cm^3, with
  body counts log-uniform in a range (the batched-replicas case).

Every builder returns a ``System`` with masses, body indices (1-based per molecule, 0 = free
atom, atoms of a molecule contiguous), positions, velocities, the cubic box edge and the
species of each atom, from which ``nonbonded`` gives charges and Lennard-Jones parameters.

Nonbonded parameters (cutoff LJ + reaction field): water O -0.834 e, sigma 0.315061 nm,
epsilon 0.636386 kJ/mol; water H +0.417 e, no LJ; argon 0 e, 0.34 nm, 0.996 kJ/mol. The
tetrahedra and rings have no published parameters; this project fixes them as neutral, with LJ
on carbon only (sigma 0.34 nm, epsilon 0.36 kJ/mol) and none on their hydrogens. The cutoff is
0.9 nm, clamped to 0.49 box edges for boxes too small for it (below 1.84 nm).
"""
from dataclasses import dataclass, field

import numpy as np

KB = 0.00831446261815324  # kJ/mol/K
AVOGADRO = 6.02214076e23

WATER_OH = 0.09572
WATER_HOH_DEG = 104.52
WATER_MASSES = (15.999, 1.008, 1.008)
WATER_CHARGES = (-0.834, 0.417, 0.417)
WATER_SIGMA = 0.315061
WATER_EPSILON = 0.636386

TETRA_ARM = 0.109
TETRA_MASSES = (12.0, 1.0, 1.0, 1.0, 1.0)
RING_CC = 0.14
RING_CH = 0.109
RING_MASSES = (12.011,) * 6 + (1.008,) * 6
ARGON_MASS = 39.95
ARGON_SIGMA = 0.34
ARGON_EPSILON = 0.996
CARBON_SIGMA = 0.34
CARBON_EPSILON = 0.36
CUTOFF = 0.9

# species codes and their (charge, sigma, epsilon)
WATER_O, WATER_H, TETRA_C, TETRA_H, RING_C, RING_H, ARGON = range(7)
NONBONDED = {WATER_O: (WATER_CHARGES[0], WATER_SIGMA, WATER_EPSILON), WATER_H: (WATER_CHARGES[1], 1.0, 0.0),
             TETRA_C: (0.0, CARBON_SIGMA, CARBON_EPSILON), TETRA_H: (0.0, 1.0, 0.0),
             RING_C: (0.0, CARBON_SIGMA, CARBON_EPSILON), RING_H: (0.0, 1.0, 0.0),
             ARGON: (0.0, ARGON_SIGMA, ARGON_EPSILON)}
SPECIES = {"water": (WATER_O, WATER_H, WATER_H), "tetra": (TETRA_C,) + (TETRA_H,) * 4,
           "ring": (RING_C,) * 6 + (RING_H,) * 6}


@dataclass
class System:
    masses: np.ndarray
    body_indices: np.ndarray
    positions: np.ndarray
    velocities: np.ndarray
    box: float
    kinds: dict = field(default_factory=dict)
    species: np.ndarray = None

    @property
    def num_atoms(self):
        return len(self.masses)

    @property
    def num_bodies(self):
        return int(len(np.unique(self.body_indices[self.body_indices > 0])))


def water_template():
    half = np.deg2rad(WATER_HOH_DEG) / 2
    return np.array([[0.0, 0.0, 0.0],
                     [WATER_OH * np.sin(half), WATER_OH * np.cos(half), 0.0],
                     [-WATER_OH * np.sin(half), WATER_OH * np.cos(half), 0.0]])


def tetra_template():
    dirs = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], dtype=np.float64) / np.sqrt(3.0)
    return np.vstack([np.zeros(3), TETRA_ARM * dirs])


def ring_template():
    ang = np.arange(6) * np.pi / 3
    c = RING_CC * np.stack([np.cos(ang), np.sin(ang), np.zeros(6)], axis=1)
    h = (RING_CC + RING_CH) * np.stack([np.cos(ang), np.sin(ang), np.zeros(6)], axis=1)
    return np.vstack([c, h])


def random_rotations(rng, n):
    """Uniform random rotation matrices from uniform unit quaternions (Shoemake)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    q = np.stack([a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)], axis=1)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def _lattice(n, box, rng=None):
    k = int(np.ceil(n ** (1.0 / 3.0)))
    g = (np.arange(k) + 0.5) * (box / k)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)[:n]
    return pts


def _mb_velocities(rng, masses, temperature):
    sd = np.sqrt(KB * temperature / masses)
    return rng.standard_normal((len(masses), 3)) * sd[:, None]


def _box_for_mass(total_amu, density_g_cm3=1.0):
    grams = total_amu / AVOGADRO
    cm3 = grams / density_g_cm3
    return (cm3 * 1e21) ** (1.0 / 3.0)  # 1 cm^3 = 1e21 nm^3


def _assemble(templates, masses_of, kinds, n_free, rng, temperature, box=None, free_mass=ARGON_MASS):
    """Place molecules of the given kinds (in the given order) plus free atoms on a lattice."""
    nmol = len(kinds)
    total_mass = sum(sum(masses_of[k]) for k in kinds) + n_free * free_mass
    if box is None:
        box = _box_for_mass(total_mass)
    sites = _lattice(nmol + n_free, box)
    order = rng.permutation(nmol + n_free)
    rot = random_rotations(rng, nmol)
    pos, mass, bidx, spec = [], [], [], []
    body = 0
    kind_count = {}
    for slot in order:
        centre = sites[slot]
        if slot < nmol:
            k = kinds[slot]
            t = templates[k]
            m = np.asarray(masses_of[k])
            t = t - (m[:, None] * t).sum(0) / m.sum()
            body += 1
            pos.append(centre + t @ rot[slot].T)
            mass.append(m)
            bidx.append(np.full(len(m), body, dtype=np.int32))
            spec.append(np.array(SPECIES[k], dtype=np.int8))
            kind_count[k] = kind_count.get(k, 0) + 1
        else:
            pos.append(centre[None, :])
            mass.append(np.array([free_mass]))
            bidx.append(np.zeros(1, dtype=np.int32))
            spec.append(np.array([ARGON], dtype=np.int8))
    masses = np.concatenate(mass)
    vel = _mb_velocities(rng, masses, temperature)
    kind_count["free"] = n_free
    return System(masses, np.concatenate(bidx), np.vstack(pos), vel, box, kind_count, np.concatenate(spec))


TEMPLATES = {"water": water_template(), "tetra": tetra_template(), "ring": ring_template()}
MASSES = {"water": WATER_MASSES, "tetra": TETRA_MASSES, "ring": RING_MASSES}


def water_box(n_waters=512, seed=1, temperature=300.0, box=None):
    """Rigid waters on a cubic lattice at 1 g/cm^3 (seeded orientations and velocities)."""
    rng = np.random.default_rng(seed)
    kinds = ["water"] * n_waters
    return _assemble(TEMPLATES, MASSES, kinds, 0, rng, temperature, box)


def mixed_system(n_bodies=1_000_000, n_free=100_000, fractions=(0.7, 0.2, 0.1), seed=3,
                 temperature=300.0, grouped=False):
    """Waters, tetrahedra and planar rings in the given fractions plus free LJ atoms.

    The molecules sit on seeded random lattice sites either way; `grouped` lists them in the
    atom order by kind (waters, tetrahedra, rings, then free atoms, as a PDB file usually lists
    residues), otherwise the kinds are interleaved in a seeded random order."""
    rng = np.random.default_rng(seed)
    nw = int(round(fractions[0] * n_bodies))
    nt = int(round(fractions[1] * n_bodies))
    nr = n_bodies - nw - nt
    kinds = ["water"] * nw + ["tetra"] * nt + ["ring"] * nr
    return _assemble_fast(kinds, n_free, rng, temperature, grouped=grouped)


def _mixed_sites(kid, ntot, box, rng):
    """Lattice site of each slot (molecules, then free atoms). Rings take random points of the
    sublattice of all-even grid indices (not touching across the periodic boundary), so that no
    two rings are nearest neighbours (their carbon hexagons would interpenetrate); the grid is
    refined until that sublattice holds every ring. The other slots take the remaining points
    with the fewest ring neighbours first, so that small boxes leave their vacancies next to
    rings."""
    ring_slots = np.nonzero(kid == 2)[0]
    sub_count = lambda k: ((k - 1) // 2 + (1 if k % 2 == 0 else 0)) ** 3 if k > 1 else 1
    k = int(np.ceil(ntot ** (1.0 / 3.0) - 1e-9))
    while sub_count(k) < len(ring_slots):
        k += 1
    g = (np.arange(k) + 0.5) * (box / k)
    ii, jj, kk = (a.ravel() for a in np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij"))
    grid = np.stack([g[ii], g[jj], g[kk]], axis=1)
    top = k - 1 if k % 2 else k  # with an odd edge, indices 0 and k-1 are periodic neighbours
    even = lambda a: (a % 2 == 0) & (a < top)
    sub = np.nonzero(even(ii) & even(jj) & even(kk))[0]
    site_of = np.empty(ntot, dtype=np.int64)
    site_of[ring_slots] = rng.choice(sub, len(ring_slots), replace=False)
    others = np.setdiff1d(np.arange(ntot), ring_slots)
    taken = np.zeros(k ** 3, dtype=bool)
    taken[site_of[ring_slots]] = True
    # ring neighbours of each point (the 26 surrounding points, periodic)
    near = np.zeros((k, k, k), dtype=np.int32)
    rmask = taken.reshape(k, k, k).astype(np.int32)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                if dx or dy or dz:
                    near += np.roll(rmask, (dx, dy, dz), axis=(0, 1, 2))
    free_points = np.nonzero(~taken)[0]
    key = near.ravel()[free_points] + rng.random(len(free_points))  # random among equals
    site_of[others] = free_points[np.argsort(key)[:len(others)]]
    return grid[site_of]


def _ring_rotations(rng, n):
    """Ring orientations: the plane normal along a random body diagonal of the lattice and the
    hexagon turned so that its carbons point between the in-plane projections of the six face
    neighbours (30 degrees from them)."""
    normal = rng.choice([-1.0, 1.0], size=(n, 3)) / np.sqrt(3.0)
    x = np.array([1.0, 0.0, 0.0])
    e1 = x - normal * (normal @ x)[:, None]
    e1 /= np.linalg.norm(e1, axis=1)[:, None]
    e2 = np.cross(normal, e1)
    u = np.cos(np.pi / 6) * e1 + np.sin(np.pi / 6) * e2
    v = np.cross(normal, u)
    return np.stack([u, v, normal], axis=2)  # columns: images of the template's x, y, z axes


def _assemble_fast(kinds, n_free, rng, temperature, free_mass=ARGON_MASS, grouped=False):
    """Vectorised version of _assemble for millions of molecules."""
    names = ["water", "tetra", "ring"]
    kid = np.array([names.index(k) for k in kinds], dtype=np.int8) if kinds else np.zeros(0, np.int8)
    nmol = len(kid)
    sizes = np.array([len(MASSES[n]) for n in names])
    total_mass = sum(np.sum(MASSES[n]) * np.count_nonzero(kid == i) for i, n in enumerate(names))
    total_mass += n_free * free_mass
    box = _box_for_mass(total_mass)
    sites = _mixed_sites(kid, nmol + n_free, box, rng)
    order = rng.permutation(nmol + n_free)
    rot = random_rotations(rng, nmol)
    rings = np.nonzero(kid == 2)[0]
    rot[rings] = _ring_rotations(rng, len(rings))
    if grouped:  # list order: molecules by kind, then free atoms; lattice sites stay random
        site_of = order.copy()
        order = np.arange(nmol + n_free)
        sites = sites[np.argsort(site_of)]
    # slot -> (kind, n atoms)
    slot_kind = np.full(nmol + n_free, 3, dtype=np.int8)  # 3 = free atom
    slot_kind[:nmol] = kid
    seq_kind = slot_kind[order]
    seq_n = np.where(seq_kind == 3, 1, sizes[np.minimum(seq_kind, 2)])
    starts = np.concatenate([[0], np.cumsum(seq_n)[:-1]])
    natoms = int(seq_n.sum())
    pos = np.empty((natoms, 3))
    mass = np.empty(natoms)
    bidx = np.zeros(natoms, dtype=np.int32)
    spec = np.full(natoms, ARGON, dtype=np.int8)
    is_mol = seq_kind != 3
    body_id = np.zeros(len(order), dtype=np.int64)
    body_id[is_mol] = np.arange(1, int(is_mol.sum()) + 1)
    free_sel = ~is_mol
    pos[starts[free_sel]] = sites[order[free_sel]]
    mass[starts[free_sel]] = free_mass
    for i, n in enumerate(names):
        sel = np.nonzero(seq_kind == i)[0]
        if len(sel) == 0:
            continue
        t = TEMPLATES[n]
        m = np.asarray(MASSES[n])
        t = t - (m[:, None] * t).sum(0) / m.sum()
        slots = order[sel]
        R = rot[slots]  # (k, 3, 3)
        placed = sites[slots][:, None, :] + np.einsum("aj,kij->kai", t, R)
        idx = starts[sel][:, None] + np.arange(len(m))[None, :]
        pos[idx] = placed
        mass[idx] = m[None, :]
        bidx[idx] = body_id[sel][:, None]
        spec[idx] = np.array(SPECIES[n], dtype=np.int8)[None, :]
    vel = _mb_velocities(rng, mass, temperature)
    counts = {n: int(np.count_nonzero(kid == i)) for i, n in enumerate(names)}
    counts["free"] = n_free
    return System(mass, bidx, pos, vel, box, counts, spec)


def gaussian_forces(n_atoms, seed=5, sd=500.0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n_atoms, 3)) * sd


def near_degenerate_system(n_bodies=8192, n_waters=20000, eps_range=(1e-8, 1e-2), seed=7, temperature=300.0,
                           arm=0.1, principal_frame=False):
    """Rigid bodies with nearly degenerate inertia among waters (the precision-study case): each
    body is a planar cross of four carbon-like atoms (mass 12, LJ on all four) with arms a and
    a*sqrt(1+eps), so that two of its principal moments differ by the factor 1+eps, eps
    log-uniform in eps_range; all molecules on one lattice at 1 g/cm^3. Orientations are random,
    or, with principal_frame, the crosses keep their arms along the x and y axes, so that their
    inertia tensors are diagonal in the space frame (the reference's eigen-solver is exact only
    there for such bodies: Smith's closed-form eigenvalues lose about 1e-9 relative,
    openmmapi/src/eigenDecomposition.cpp:72-101)."""
    rng = np.random.default_rng(seed)
    eps = np.exp(rng.uniform(np.log(eps_range[0]), np.log(eps_range[1]), size=n_bodies))
    nmol = n_bodies + n_waters
    m_body = np.full(4, 12.0)
    total = n_bodies * m_body.sum() + n_waters * sum(WATER_MASSES)
    box = _box_for_mass(total)
    sites = _lattice(nmol, box)[rng.permutation(nmol)]
    rot = random_rotations(rng, nmol)
    wt = water_template()
    wm = np.asarray(WATER_MASSES)
    wt = wt - (wm[:, None] * wt).sum(0) / wm.sum()
    pos, mass, bidx, spec = [], [], [], []
    for k in range(nmol):
        if k < n_bodies:
            b = arm * np.sqrt(1.0 + eps[k])
            t = np.array([[arm, 0, 0], [-arm, 0, 0], [0, b, 0], [0, -b, 0]])
            m, sp = m_body, (TETRA_C,) * 4
            if principal_frame:
                pos.append(sites[k] + t)
                mass.append(m)
                bidx.append(np.full(len(m), k + 1, dtype=np.int32))
                spec.append(np.array(sp, dtype=np.int8))
                continue
        else:
            t, m, sp = wt, wm, SPECIES["water"]
        pos.append(sites[k] + t @ rot[k].T)
        mass.append(m)
        bidx.append(np.full(len(m), k + 1, dtype=np.int32))
        spec.append(np.array(sp, dtype=np.int8))
    masses = np.concatenate(mass)
    s = System(masses, np.concatenate(bidx), np.vstack(pos), _mb_velocities(rng, masses, temperature), box,
               {"cross": n_bodies, "water": n_waters}, np.concatenate(spec))
    s.eps = eps
    return s


def nonbonded(system):
    """Per-atom (charge, sigma, epsilon) arrays of a system from its species."""
    table = np.array([NONBONDED[k] for k in range(len(NONBONDED))])
    p = table[system.species.astype(np.int64)]
    return p[:, 0].copy(), p[:, 1].copy(), p[:, 2].copy()


def cutoff_for(box):
    """The 0.9 nm cutoff, clamped to 0.49 box edges where the box is too small for it."""
    return min(CUTOFF, 0.49 * box)


def batch_body_counts(n_systems=4096, lo=64, hi=4096, seed=6):
    """Body counts of the batched-replicas workload: log-uniform in [lo, hi], seeded."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=n_systems)).astype(np.int64)


def batch_system(k, n_bodies, fractions=(0.7, 0.2, 0.1), seed=6, temperature=300.0):
    """System k of the batched-replicas workload (seeded from `seed` and k), without free atoms."""
    return mixed_system(n_bodies=int(n_bodies), n_free=0, fractions=fractions, seed=seed * 100003 + k,
                        temperature=temperature)


def batch_systems(n_systems=4096, lo=64, hi=4096, fractions=(0.7, 0.2, 0.1), seed=6, temperature=300.0, only=None):
    """Independent mixed systems without free atoms, body counts log-uniform in [lo, hi], each in
    its own cubic box at 1 g/cm^3 and seeded from `seed` and its index; `only` (indices) builds a
    subset of them."""
    counts = batch_body_counts(n_systems, lo, hi, seed)
    idx = range(n_systems) if only is None else only
    return [batch_system(int(k), counts[k], fractions, seed, temperature) for k in idx]
