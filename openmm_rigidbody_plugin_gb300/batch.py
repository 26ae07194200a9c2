"""Batched systems: many independent periodic systems stepped together (rbx_batch_* C ABI).

Each system is a rigid-body system in its own cubic box; forces come from the library's neighbour-list
cutoff Lennard-Jones + reaction-field kernels (the CutoffPeriodic form of OpenMM's
NonbondedForce), and the whole set advances with one integrator launch per step. Runs of steps
can replay a captured CUDA graph (``graph_steps``).
"""
import ctypes

import numpy as np

from . import _lib

EPS_SOLVENT = 78.3
BODY_ROW_BYTES = 112  # exact body-state row of a checkpoint (rbx_get_body_state_raw)


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _stream(stream):
    import torch
    return ctypes.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


class BatchedSystems:
    """Independent systems (each with masses, body_indices, positions, velocities, box and
    per-atom charge/sigma/epsilon) integrated as one batch on one device."""

    def __init__(self, masses, body_indices, atom_offsets, boxes, cutoffs, charges, sigmas, epsilons,
                 rotation_mode=0, precision="mixed", eps_solvent=EPS_SOLVENT, device=0):
        self._lib = _lib.load()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.offsets = np.ascontiguousarray(atom_offsets, dtype=np.int32)
        self.num_systems = len(self.offsets) - 1
        self.num_atoms = int(self.offsets[-1])
        cast = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.boxes = cast(boxes)
        self.cutoffs = cast(cutoffs)
        bidx = np.asarray(body_indices)
        # bodies per system as the library counts them: ids shared by at least two atoms
        self.bodies_per_system = np.array([
            int(np.count_nonzero(np.bincount(np.maximum(bidx[a:b], 0))[1:] >= 2)) if b > a else 0
            for a, b in zip(self.offsets[:-1], self.offsets[1:])])
        h = ctypes.c_void_p()
        _lib.check(self._lib.rbx_batch_create(
            ctypes.byref(h), self.num_systems, _i(self.offsets), _d(self.boxes), _d(self.cutoffs),
            _i(np.ascontiguousarray(body_indices, dtype=np.int32)), _d(cast(masses)), _d(cast(charges)),
            _d(cast(sigmas)), _d(cast(epsilons)), float(eps_solvent), int(rotation_mode),
            _lib.PRECISIONS[precision], int(device)))
        self._h = h

    @classmethod
    def from_systems(cls, systems, rotation_mode=0, precision="mixed", device=0, relax_steps=0, temperature=300.0,
                     seed=0):
        """Batch of workloads.System objects, with their species' nonbonded parameters and the
        0.9 nm cutoff clamped to 0.49 box edges. With relax_steps > 0 the generated structures are
        first relaxed (``relax``) and then given Maxwell-Boltzmann velocities at `temperature`."""
        from . import workloads as W
        q, s, e = zip(*(W.nonbonded(x) for x in systems))
        offsets = np.concatenate([[0], np.cumsum([x.num_atoms for x in systems])])
        b = cls(np.concatenate([x.masses for x in systems]), np.concatenate([x.body_indices for x in systems]),
                offsets, [x.box for x in systems], [W.cutoff_for(x.box) for x in systems], np.concatenate(q),
                np.concatenate(s), np.concatenate(e), rotation_mode=rotation_mode, precision=precision,
                device=device)
        b.set_state(np.concatenate([x.positions for x in systems]), np.concatenate([x.velocities for x in systems]))
        if relax_steps > 0:
            b.relax(relax_steps)
            b.thermalize(temperature, seed)
        return b

    def relax(self, nsteps=400, dt=0.002, max_force=2000.0, damping=0.7, stream=None):
        """Damped dynamics (forces capped at max_force, momenta scaled by `damping` each step) that
        removes the overlaps of generated starting structures; leaves every momentum at zero."""
        _lib.check(self._lib.rbx_batch_relax(self._h, _stream(stream), int(nsteps), float(dt), float(max_force),
                                             float(damping)))

    def thermalize(self, temperature=300.0, seed=0, stream=None):
        """Seeded Maxwell-Boltzmann velocities at the current positions (projected onto rigid motion
        by the state upload)."""
        from .workloads import KB
        x, _ = self.get_state(stream)
        rng = np.random.default_rng(seed)
        sd = np.sqrt(KB * temperature / np.where(self.masses > 0, self.masses, 1.0))
        v = rng.standard_normal((self.num_atoms, 3)) * sd[:, None] * (self.masses > 0)[:, None]
        self.set_state(x, v, stream)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rbx_batch_destroy(h)
            self._h = None

    def set_state(self, positions, velocities, stream=None):
        x = np.ascontiguousarray(positions, dtype=np.float64)
        v = np.ascontiguousarray(velocities, dtype=np.float64)
        _lib.check(self._lib.rbx_batch_set_state(self._h, _stream(stream), _d(x), _d(v)))

    def get_state(self, stream=None):
        x = np.zeros((self.num_atoms, 3))
        v = np.zeros((self.num_atoms, 3))
        _lib.check(self._lib.rbx_batch_get_state(self._h, _stream(stream), _d(x), _d(v)))
        return x, v

    def get_system_state(self, s, stream=None):
        """Positions and velocities of system s only."""
        n = int(self.offsets[s + 1] - self.offsets[s])
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        _lib.check(self._lib.rbx_batch_get_system_state(self._h, _stream(stream), int(s), _d(x), _d(v)))
        return x, v

    def checkpoint(self, stream=None):
        """Exact state of every system: a list of (body rows [nb_s, 112] bytes, positions, velocities).
        The body rows are the state's device words (rbx_get_body_state_raw): 14 doubles, or the 14
        high then 14 low floats of the float-float state."""
        bs = np.zeros((int(self.bodies_per_system.sum()), BODY_ROW_BYTES), dtype=np.uint8)
        _lib.check(self._lib.rbx_batch_get_body_state(self._h, bs.ctypes.data_as(ctypes.c_void_p)))
        x, v = self.get_state(stream)
        b_off = np.concatenate([[0], np.cumsum(self.bodies_per_system)])
        return [(bs[b_off[k]:b_off[k + 1]].copy(), x[self.offsets[k]:self.offsets[k + 1]].copy(),
                 v[self.offsets[k]:self.offsets[k + 1]].copy()) for k in range(self.num_systems)]

    def restore(self, states, stream=None):
        """Put back per-system states from ``checkpoint`` (bit for bit). The batch must hold the same
        systems, set up from the positions the checkpointed batch was last set up from."""
        bs = np.ascontiguousarray(np.concatenate([s[0] for s in states]) if states else
                                  np.zeros((0, BODY_ROW_BYTES), dtype=np.uint8), dtype=np.uint8)
        x = np.ascontiguousarray(np.concatenate([s[1] for s in states]))
        v = np.ascontiguousarray(np.concatenate([s[2] for s in states]))
        _lib.check(self._lib.rbx_batch_restore(self._h, _stream(stream), bs.ctypes.data_as(ctypes.c_void_p), _d(x),
                                               _d(v)))

    def step(self, nsteps, dt, stream=None):
        """nsteps velocity-Verlet steps of every system; a call that follows another step call
        starts from the forces that call ended with (one force evaluation per step)."""
        _lib.check(self._lib.rbx_batch_step(self._h, _stream(stream), int(nsteps), float(dt)))

    def energies(self, stream=None):
        """[U, KE_t, KE_r] per system (kJ/mol), shape (num_systems, 3)."""
        out = np.zeros((self.num_systems, 3))
        _lib.check(self._lib.rbx_batch_energies(self._h, _stream(stream), _d(out)))
        return out

    def forces(self, stream=None):
        """Forces at the current positions (user order, kJ/mol/nm) and the potential energies."""
        f = np.zeros((self.num_atoms, 3))
        e = np.zeros(self.num_systems)
        _lib.check(self._lib.rbx_batch_forces(self._h, _stream(stream), _d(f), _d(e)))
        return f, e

    @property
    def num_dof(self):
        out = np.zeros(self.num_systems, dtype=np.int32)
        _lib.check(self._lib.rbx_batch_get_num_dof(self._h, _i(out)))
        return out

    def status(self, stream=None):
        """Failure status per system (0, or 5 = RBX_ERR_NUMERIC for a system whose state became
        non-finite or whose forces left the fixed-point range) since the last set_state/restore."""
        out = np.zeros(self.num_systems, dtype=np.int32)
        n = ctypes.c_int()
        rc = self._lib.rbx_batch_status(self._h, _stream(stream), _i(out), ctypes.byref(n))
        if rc not in (0, _lib.RBX_ERR_NUMERIC):
            _lib.check(rc)
        return out

    def list_builds(self, stream=None):
        """Neighbour-list builds of each system so far (rbx_batch_list_builds)."""
        out = np.zeros(self.num_systems, dtype=np.uint32)
        _lib.check(self._lib.rbx_batch_list_builds(self._h, _stream(stream),
                                                   out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint))))
        return out

    @property
    def memory_bytes(self):
        """Device bytes the batch and its integrator hold (rbx_batch_memory)."""
        n = ctypes.c_size_t()
        _lib.check(self._lib.rbx_batch_memory(self._h, ctypes.byref(n)))
        return int(n.value)

    def set_graph_steps(self, k):
        _lib.check(self._lib.rbx_batch_set_graph_steps(self._h, int(k)))

    def autotune(self, dt=0.002, trial_steps=3, stream=None):
        """Pick the step kernel's tile shape, the cell list-build kernel's block size and the steps per
        captured graph by timing them on this batch; the state is restored exactly afterwards.
        Returns the choice."""
        out = np.zeros(2, dtype=np.int32)
        _lib.check(self._lib.rbx_batch_autotune(self._h, _stream(stream), float(dt), int(trial_steps),
                                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return {"tile_threads": self.tile_threads, "cell_threads": int(out[0]), "graph_steps": int(out[1])}

    @property
    def tile_threads(self):
        """Block size of the step kernel's tiles (results do not depend on it)."""
        out = ctypes.c_int()
        _lib.check(self._lib.rbx_batch_get_tile_threads(self._h, ctypes.byref(out)))
        return out.value

    @tile_threads.setter
    def tile_threads(self, threads):
        _lib.check(self._lib.rbx_batch_set_tile_threads(self._h, int(threads)))

    def set_tuning(self, cell_threads, graph_steps):
        _lib.check(self._lib.rbx_batch_set_tuning(self._h, int(cell_threads), int(graph_steps)))

    def set_timing(self, on):
        _lib.check(self._lib.rbx_batch_set_timing(self._h, int(bool(on))))

    def kernel_times(self):
        """(ms in force kernels, ms in integrator kernels, launch groups) since the last call."""
        f, i, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _lib.check(self._lib.rbx_batch_kernel_times(self._h, ctypes.byref(f), ctypes.byref(i), ctypes.byref(n)))
        return f.value, i.value, n.value

    @property
    def last_launch_count(self):
        return self._lib.rbx_batch_last_launch_count(self._h)
