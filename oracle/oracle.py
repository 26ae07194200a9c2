"""ctypes front-ends for the CPU checkers built by ``oracle/Makefile``.

TEST INFRASTRUCTURE ONLY. ``Oracle`` wraps this project's C restatement (``liboracle.so``) and
``Reference`` wraps the reference plugin's own CPU code compiled from its sources
(``_ref/librefrb.so``, present only where the reference tree was available at build time).
Only the tests, the smoke check and bench.py's CPU arm import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "librefrb.so")
BODY_RECORD = 36

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def build(reference_root=None):
    """Compile liboracle.so, and oracle/_ref/librefrb.so from the reference plugin's sources when
    their tree is given (`reference_root`, else the RBX_REFERENCE_ROOT environment variable; there
    is no default location). Without it the compiled reference is skipped, and the tests that
    need it skip themselves."""
    cmd = ["make", "-s", "-C", HERE, "oracle"]
    subprocess.run(cmd, check=True)
    ref = reference_root or os.environ.get("RBX_REFERENCE_ROOT")
    if ref and os.path.isdir(ref):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, _dp, _ip, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_setup.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_part1.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]
        L.orc_part2.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]
        L.orc_kinetic.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_set_refined.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_refined.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, _dp]
        for f in ("orc_num_dof", "orc_num_bodies", "orc_num_free", "orc_num_body_atoms"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.orc_atom_index.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_get_body.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_get_body_fixed.argtypes = [ctypes.c_void_p, _dp]
        L.orc_set_body_state.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_set_body_geometry.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc_run_fixed_force.restype = ctypes.c_double
        L.orc_run_fixed_force.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_exact_rotation.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int]
        L.orc_nosquish_rotation.argtypes = [_dp, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_int]
        L.orc_jacobi_sncndn.argtypes = [ctypes.c_double, ctypes.c_double, _dp, _dp, _dp]
        L.orc_carlson_rc.restype = ctypes.c_double
        L.orc_carlson_rc.argtypes = [ctypes.c_double] * 2
        L.orc_carlson_rf.restype = ctypes.c_double
        L.orc_carlson_rf.argtypes = [ctypes.c_double] * 3
        L.orc_carlson_rj.restype = ctypes.c_double
        L.orc_carlson_rj.argtypes = [ctypes.c_double] * 4
        L.orc_eigen.argtypes = [_dp, _dp, _dp, ctypes.c_int]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_lj_rf.argtypes = [ctypes.c_int, _ip, _dp, _dp, ctypes.c_double, _dp, _dp, _dp, _dp, _ip, _dp, _dp,
                                ctypes.c_int]
        L.orc_lj_rf_atoms.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      _dp, _dp, _dp, _dp, _ip, ctypes.c_int, _ip, _dp]
        _lib = L
    return _lib


EPS_SOLVENT = 78.3  # OpenMM's default reaction-field dielectric


def lj_rf(atom_offsets, boxes, cutoffs, positions, charges, sigmas, epsilons, bodies, eps_solvent=EPS_SOLVENT,
          nthreads=None):
    """FP64 cutoff LJ + reaction-field forces and per-system energies (ff_oracle.c)."""
    off = np.ascontiguousarray(atom_offsets, dtype=np.int32)
    S = len(off) - 1
    n = int(off[-1])
    f = np.zeros((n, 3))
    e = np.zeros(S)
    cast = lambda a, t=np.float64: np.ascontiguousarray(a, dtype=t)
    pos, q, sg, ep = cast(positions), cast(charges), cast(sigmas), cast(epsilons)
    bd = cast(bodies, np.int32)
    bx, rc = cast(np.broadcast_to(boxes, (S,))), cast(np.broadcast_to(cutoffs, (S,)))
    lib().orc_lj_rf(S, _i(off), _d(bx), _d(rc), eps_solvent, _d(pos), _d(q), _d(sg), _d(ep), _i(bd), _d(f), _d(e),
                    nthreads or (os.cpu_count() or 1))
    return f, e


def lj_rf_atoms(selected, box, cutoff, positions, charges, sigmas, epsilons, bodies, eps_solvent=EPS_SOLVENT):
    """FP64 forces on the selected atoms of one box (all atoms of `positions` in that box)."""
    sel = np.ascontiguousarray(selected, dtype=np.int32)
    cast = lambda a, t=np.float64: np.ascontiguousarray(a, dtype=t)
    pos, q, sg, ep, bd = cast(positions), cast(charges), cast(sigmas), cast(epsilons), cast(bodies, np.int32)
    f = np.zeros((len(sel), 3))
    lib().orc_lj_rf_atoms(0, len(pos), box, cutoff, eps_solvent, _d(pos), _d(q), _d(sg), _d(ep), _i(bd), len(sel),
                          _i(sel), _d(f))
    return f


class _Base:
    """Common state holder: user-order arrays R, V (natoms x 3, float64)."""

    def _arrays(self, R, V, F):
        self.R = np.ascontiguousarray(R, dtype=np.float64).copy()
        self.V = np.ascontiguousarray(V, dtype=np.float64).copy()
        F = np.ascontiguousarray(F, dtype=np.float64)
        return F

    @staticmethod
    def _f(F):
        return np.ascontiguousarray(F, dtype=np.float64)


class Oracle(_Base):
    """The project's C restatement. ``robust`` selects the robust FP64 oracle."""

    def __init__(self, masses, body_indices, mode=0, robust=False):
        L = lib()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.bidx = np.ascontiguousarray(body_indices, dtype=np.int32)
        self.n = len(self.masses)
        self.h = L.orc_create(self.n, _d(self.masses), _i(self.bidx), int(mode), int(bool(robust)))
        if not self.h:
            raise ValueError(L.orc_last_error().decode())
        self.mode = mode

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def setup(self, R, V, F):
        F = self._arrays(R, V, F)
        lib().orc_setup(self.h, _d(self.R), _d(self.V), _d(F))

    def part1(self, dt, F):
        lib().orc_part1(self.h, dt, _d(self._f(F)), _d(self.V), _d(self.R))

    def part2(self, dt, F):
        lib().orc_part2(self.h, dt, _d(self.R), _d(self._f(F)), _d(self.V))

    def step(self, dt, force_fn, nsteps=1):
        for _ in range(nsteps):
            self.part1(dt, force_fn(self.R, 0))
            self.part2(dt, force_fn(self.R, 1))

    def kinetic(self):
        out = np.zeros(2)
        lib().orc_kinetic(self.h, _d(self.V), _d(out))
        return out

    def set_refined(self, mode=1):
        """Refined energies on (1), off (0), or on with the reference's free-atom weights (2)."""
        lib().orc_set_refined(self.h, int(mode))

    def refined(self, dt, F):
        """[KE_t, KE_r, U_refinement] after a part2 whose force array was F."""
        out = np.zeros(3)
        lib().orc_refined(self.h, _d(self.V), _d(self._f(F)), float(dt), _d(out))
        return out

    @property
    def num_dof(self):
        return lib().orc_num_dof(self.h)

    @property
    def num_bodies(self):
        return lib().orc_num_bodies(self.h)

    @property
    def num_free(self):
        return lib().orc_num_free(self.h)

    @property
    def num_body_atoms(self):
        return lib().orc_num_body_atoms(self.h)

    def atom_index(self):
        L = lib()
        n = self.num_free + self.num_body_atoms
        return np.array([L.orc_atom_index(self.h, i) for i in range(n)], dtype=np.int64)

    def bodies(self):
        out = np.zeros((self.num_bodies, BODY_RECORD))
        for b in range(self.num_bodies):
            lib().orc_get_body(self.h, b, _d(out[b]))
        return out

    def body_fixed(self):
        out = np.zeros((self.num_body_atoms, 3))
        lib().orc_get_body_fixed(self.h, _d(out))
        return out

    def set_body_state(self, b, rcm, pcm, q, pi):
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (rcm, pcm, q, pi)]
        lib().orc_set_body_state(self.h, b, *[_d(x) for x in a])

    def set_body_geometry(self, b, I, d):
        I = np.ascontiguousarray(I, dtype=np.float64)
        d = np.ascontiguousarray(d, dtype=np.float64)
        lib().orc_set_body_geometry(self.h, b, _d(I), _d(d))

    def run_fixed_force(self, dt, F, nsteps, nthreads=1):
        return lib().orc_run_fixed_force(self.h, dt, _d(self._f(F)), _d(self.V), _d(self.R), nsteps, nthreads)


_ref = None


def reference_available():
    return os.path.exists(REF_SO)


def reflib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_SO)
        L.refrb_create.restype = ctypes.c_void_p
        L.refrb_create.argtypes = [ctypes.c_int, _dp, _ip, ctypes.c_int]
        L.refrb_destroy.argtypes = [ctypes.c_void_p]
        L.refrb_set_state.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.refrb_part1.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]
        L.refrb_part2.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, _dp, _dp]
        L.refrb_kinetic.argtypes = [ctypes.c_void_p, _dp, _dp]
        for f in ("refrb_num_dof", "refrb_num_bodies", "refrb_num_free", "refrb_num_body_atoms"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.refrb_atom_index.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.refrb_get_body.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.refrb_get_body_fixed.argtypes = [ctypes.c_void_p, _dp]
        L.refrb_last_error.restype = ctypes.c_char_p
        _ref = L
    return _ref


class Reference(_Base):
    """The reference plugin's own CPU integrator (RigidBodySystem) compiled from its sources."""

    def __init__(self, masses, body_indices, mode=0):
        L = reflib()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.bidx = np.ascontiguousarray(body_indices, dtype=np.int32)
        self.n = len(self.masses)
        self.h = L.refrb_create(self.n, _d(self.masses), _i(self.bidx), int(mode))
        self.mode = mode

    def __del__(self):
        if getattr(self, "h", None):
            reflib().refrb_destroy(self.h)
            self.h = None

    def setup(self, R, V, F):
        F = self._arrays(R, V, F)
        if reflib().refrb_set_state(self.h, _d(self.R), _d(self.V), _d(F)) != 0:
            raise RuntimeError(reflib().refrb_last_error().decode())

    def part1(self, dt, F):
        reflib().refrb_part1(self.h, dt, _d(self._f(F)), _d(self.V), _d(self.R))

    def part2(self, dt, F):
        reflib().refrb_part2(self.h, dt, _d(self.R), _d(self._f(F)), _d(self.V))

    def step(self, dt, force_fn, nsteps=1):
        for _ in range(nsteps):
            self.part1(dt, force_fn(self.R, 0))
            self.part2(dt, force_fn(self.R, 1))

    def kinetic(self):
        out = np.zeros(2)
        reflib().refrb_kinetic(self.h, _d(self.V), _d(out))
        return out

    @property
    def num_dof(self):
        return reflib().refrb_num_dof(self.h)

    @property
    def num_bodies(self):
        return reflib().refrb_num_bodies(self.h)

    @property
    def num_free(self):
        return reflib().refrb_num_free(self.h)

    @property
    def num_body_atoms(self):
        return reflib().refrb_num_body_atoms(self.h)

    def atom_index(self):
        L = reflib()
        n = self.num_free + self.num_body_atoms
        return np.array([L.refrb_atom_index(self.h, i) for i in range(n)], dtype=np.int64)

    def bodies(self):
        out = np.zeros((self.num_bodies, BODY_RECORD))
        for b in range(self.num_bodies):
            reflib().refrb_get_body(self.h, b, _d(out[b]))
        return out

    def body_fixed(self):
        out = np.zeros((self.num_body_atoms, 3))
        reflib().refrb_get_body_fixed(self.h, _d(out))
        return out
