"""Python handle on the C ABI: one integrator kernel plus OpenMM-layout device buffers.

``IntegratorKernel`` is the object the C++ OpenMM shim would hold (the role of
CudaIntegrateRigidBodyStepKernel, platforms/cuda/src/CudaRigidBodyKernels.h:45-133);
``DeviceBuffers`` allocates the arrays an OpenMM CudaContext would lend it (posq,
posqCorrection, velm, fixed-point force) with PyTorch, which serves only as the allocator and
stream provider here.
"""
import ctypes

import numpy as np

from . import _lib

FIXED_POINT_SCALE = float(2 ** 32)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _stream_handle(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


class DeviceBuffers:
    """posq / posqCorrection / velm / force arrays in the OpenMM CUDA layout (device memory)."""

    def __init__(self, num_atoms, precision="mixed", device=0, stride=None):
        import torch
        self.num_atoms = num_atoms
        self.precision = precision
        self.stride = stride or ((num_atoms + 31) // 32) * 32
        dev = torch.device("cuda", device)
        pdt = torch.float64 if precision == "double" else torch.float32
        vdt = torch.float32 if precision == "single" else torch.float64
        self.posq = torch.zeros((self.stride, 4), dtype=pdt, device=dev)
        self.corr = torch.zeros((self.stride, 4), dtype=torch.float32, device=dev) if precision == "mixed" else None
        self.velm = torch.zeros((self.stride, 4), dtype=vdt, device=dev)
        self.force = torch.zeros(3 * self.stride, dtype=torch.int64, device=dev)
        # OpenMM's posDelta (mixed4 per slot), for free atoms under constraints
        self.pos_delta = torch.zeros((self.stride, 4), dtype=vdt, device=dev)
        self.location = np.arange(num_atoms, dtype=np.int64)

    def struct(self):
        return _lib.Buffers(self.posq.data_ptr(), self.corr.data_ptr() if self.corr is not None else None,
                            self.velm.data_ptr(), self.force.data_ptr(), self.stride)

    def _loc(self):
        import torch
        return torch.as_tensor(self.location, device=self.posq.device)

    def set_positions(self, x):
        import torch
        x = torch.as_tensor(np.asarray(x, dtype=np.float64), device=self.posq.device)
        loc = self._loc()
        if self.precision == "mixed":
            hi = x.to(torch.float32)
            self.posq[loc, :3] = hi
            self.corr[loc, :3] = (x - hi.to(torch.float64)).to(torch.float32)
        else:
            self.posq[loc, :3] = x.to(self.posq.dtype)

    def set_velocities(self, v, masses):
        import torch
        v = torch.as_tensor(np.asarray(v, dtype=np.float64), device=self.posq.device)
        m = np.asarray(masses, dtype=np.float64)
        inv = torch.as_tensor(np.where(m > 0, 1.0 / np.where(m > 0, m, 1.0), 0.0), device=self.posq.device)
        loc = self._loc()
        self.velm[loc, :3] = v.to(self.velm.dtype)
        self.velm[loc, 3] = inv.to(self.velm.dtype)

    def set_forces(self, f):
        import torch
        f = torch.as_tensor(np.asarray(f, dtype=np.float64), device=self.posq.device)
        fx = torch.round(f * FIXED_POINT_SCALE).to(torch.int64)
        loc = self._loc()
        for c in range(3):
            self.force[loc + c * self.stride] = fx[:, c]

    def get_pos_delta(self):
        return self.pos_delta[self._loc(), :3].to(self.pos_delta.dtype).cpu().double().numpy()

    def set_pos_delta(self, d):
        import torch
        self.pos_delta[self._loc(), :3] = torch.as_tensor(np.asarray(d, dtype=np.float64),
                                                          device=self.posq.device).to(self.pos_delta.dtype)

    def relocate(self, location):
        """Move every atom's slot contents to its new slot, as OpenMM's atom reordering does
        (posq, posqCorrection, velm and the three force components move together)."""
        import torch
        old = self._loc()
        new = torch.as_tensor(np.asarray(location, dtype=np.int64), device=self.posq.device)
        for a in (self.posq, self.corr, self.velm):
            if a is not None:
                a[new] = a[old].clone()
        for c in range(3):
            self.force[new + c * self.stride] = self.force[old + c * self.stride].clone()
        self.location = np.asarray(location, dtype=np.int64)

    def get_positions(self):
        import torch
        loc = self._loc()
        x = self.posq[loc, :3].to(torch.float64)
        if self.corr is not None:
            x = x + self.corr[loc, :3].to(torch.float64)
        return x.cpu().numpy()

    def get_velocities(self):
        import torch
        return self.velm[self._loc(), :3].to(torch.float64).cpu().numpy()


class IntegratorKernel:
    """One rigid-body integrator on one device, driven through the C ABI."""

    def __init__(self, masses, body_indices, rotation_mode=0, precision="mixed", device=0):
        lib = _lib.load()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64)
        self.body_indices = np.ascontiguousarray(body_indices, dtype=np.int32)
        if precision not in _lib.PRECISIONS:
            raise ValueError(f"unknown precision {precision!r}")
        self.precision = precision
        self.num_atoms = len(self.masses)
        h = ctypes.c_void_p()
        _lib.check(lib.rbx_create(ctypes.byref(h), self.num_atoms, _iptr(self.body_indices), _dptr(self.masses),
                                  int(rotation_mode), _lib.PRECISIONS[precision], int(device)))
        self._h = h
        self._lib = lib

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.rbx_destroy(h)
            self._h = None

    # setup ------------------------------------------------------------------------------
    def set_atom_locations(self, location):
        loc = np.ascontiguousarray(location, dtype=np.int32)
        _lib.check(self._lib.rbx_set_atom_locations(self._h, _iptr(loc)))

    def upload_state(self, positions, velocities):
        x = np.ascontiguousarray(positions, dtype=np.float64)
        v = np.ascontiguousarray(velocities, dtype=np.float64)
        _lib.check(self._lib.rbx_upload_state(self._h, _dptr(x), _dptr(v)))

    def upload_state_device(self, buffers, stream=None):
        """Body setup on the device from the positions and velocities in `buffers`."""
        b = buffers.struct()
        _lib.check(self._lib.rbx_upload_state_device(self._h, _stream_handle(stream), ctypes.byref(b)))

    def _get_int(self, fn):
        out = ctypes.c_int()
        _lib.check(fn(self._h, ctypes.byref(out)))
        return out.value

    @property
    def num_dof(self):
        return self._get_int(self._lib.rbx_get_num_dof)

    @property
    def num_dof_reference(self):
        """The reference's own count (one per free atom, unique indices as one-atom bodies)."""
        return self._get_int(self._lib.rbx_get_num_dof_reference)

    @property
    def num_bodies(self):
        return self._get_int(self._lib.rbx_get_num_bodies)

    @property
    def num_free(self):
        return self._get_int(self._lib.rbx_get_num_free)

    @property
    def rotation_mode(self):
        return self._get_int(self._lib.rbx_get_rotation_mode)

    @property
    def tile_threads(self):
        """Block size of the step kernel's tiles (256, or 128 in single/mixed precision when every
        body has at most 32 atoms); results do not depend on it (rbx_set_tile_threads)."""
        return self._get_int(self._lib.rbx_get_tile_threads)

    @tile_threads.setter
    def tile_threads(self, threads):
        _lib.check(self._lib.rbx_set_tile_threads(self._h, int(threads)))

    # device steps -------------------------------------------------------------------------
    def part1(self, buffers, dt, stream=None):
        b = buffers.struct()
        _lib.check(self._lib.rbx_integrate_part1(self._h, _stream_handle(stream), ctypes.byref(b), float(dt)))

    def part2(self, buffers, dt, stream=None):
        b = buffers.struct()
        _lib.check(self._lib.rbx_integrate_part2(self._h, _stream_handle(stream), ctypes.byref(b), float(dt)))

    def fused(self, buffers, dt, stream=None):
        b = buffers.struct()
        _lib.check(self._lib.rbx_integrate_fused(self._h, _stream_handle(stream), ctypes.byref(b), float(dt)))

    # free atoms under constraints (OpenMM's posDelta protocol) ----------------------------------
    def set_constraints(self, pairs):
        p = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        _lib.check(self._lib.rbx_set_constraints(self._h, len(p), _iptr(p) if len(p) else None))

    def free_atoms_delta(self, buffers, dt, stream=None):
        b = buffers.struct()
        _lib.check(self._lib.rbx_free_atoms_delta(self._h, _stream_handle(stream), ctypes.byref(b),
                                                  ctypes.c_void_p(buffers.pos_delta.data_ptr()), float(dt)))

    def part1_delta(self, buffers, dt, stream=None):
        b = buffers.struct()
        _lib.check(self._lib.rbx_integrate_part1_delta(self._h, _stream_handle(stream), ctypes.byref(b),
                                                       ctypes.c_void_p(buffers.pos_delta.data_ptr()), float(dt)))

    def check_state(self, stream=None):
        """(bad bodies, bad free atoms) flagged by the step kernels since the last state change:
        both 0 unless a step left a non-finite state (rbx_check_state)."""
        nb, nf = ctypes.c_int(), ctypes.c_int()
        rc = self._lib.rbx_check_state(self._h, _stream_handle(stream), ctypes.byref(nb), ctypes.byref(nf))
        if rc not in (0, _lib.RBX_ERR_NUMERIC):
            _lib.check(rc)
        return nb.value, nf.value

    def kinetic_energies(self, buffers, stream=None):
        out = np.zeros(2)
        b = buffers.struct()
        _lib.check(self._lib.rbx_kinetic_energies(self._h, _stream_handle(stream), ctypes.byref(b), _dptr(out)))
        return out

    # refined ("shadow") energies --------------------------------------------------------------
    def set_compute_refined_energies(self, compute):
        _lib.check(self._lib.rbx_set_compute_refined_energies(self._h, int(bool(compute))))

    @property
    def compute_refined_energies(self):
        out = ctypes.c_int(0)
        _lib.check(self._lib.rbx_get_compute_refined_energies(self._h, ctypes.byref(out)))
        return bool(out.value)

    def refined_kinetic_energies(self, buffers, stream=None):
        """[KE_t, KE_r] refined (the plain kinetic energies while refined energies are off)."""
        out = np.zeros(2)
        b = buffers.struct() if hasattr(buffers, "struct") else buffers
        _lib.check(self._lib.rbx_refined_kinetic_energies(self._h, _stream_handle(stream), ctypes.byref(b),
                                                          _dptr(out)))
        return out

    def potential_energy_refinement(self, buffers, stream=None):
        out = np.zeros(1)
        b = buffers.struct() if hasattr(buffers, "struct") else buffers
        _lib.check(self._lib.rbx_potential_energy_refinement(self._h, _stream_handle(stream), ctypes.byref(b),
                                                             _dptr(out)))
        return float(out[0])

    def context_refined_kinetic_energies(self, stream=None):
        return self.refined_kinetic_energies(self.context_buffers(), stream)

    def context_potential_energy_refinement(self, stream=None):
        return self.potential_energy_refinement(self.context_buffers(), stream)

    @property
    def last_launch_count(self):
        return self._lib.rbx_last_launch_count(self._h)

    # body state -----------------------------------------------------------------------------
    def body_atoms(self):
        first = np.zeros(self.num_bodies + 1, dtype=np.int32)
        nba = self.num_atoms  # upper bound
        atoms = np.zeros(nba, dtype=np.int32)
        _lib.check(self._lib.rbx_get_body_atoms(self._h, _iptr(first), _iptr(atoms)))
        return first, atoms[:first[-1]]

    def body_state(self):
        out = np.zeros((self.num_bodies, 14))
        _lib.check(self._lib.rbx_get_body_state(self._h, _dptr(out)))
        return out

    def set_body_state(self, state):
        s = np.ascontiguousarray(state, dtype=np.float64)
        _lib.check(self._lib.rbx_set_body_state(self._h, _dptr(s)))

    def body_state_raw(self):
        """The body state's exact device words, 112 bytes per body (rbx_get_body_state_raw)."""
        out = np.zeros((self.num_bodies, 112), dtype=np.uint8)
        _lib.check(self._lib.rbx_get_body_state_raw(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def set_body_state_raw(self, rows):
        r = np.ascontiguousarray(rows, dtype=np.uint8)
        _lib.check(self._lib.rbx_set_body_state_raw(self._h, r.ctypes.data_as(ctypes.c_void_p)))

    def geometry(self):
        first, _ = self.body_atoms()
        I = np.zeros((self.num_bodies, 3))
        d = np.zeros((int(first[-1]), 3))
        _lib.check(self._lib.rbx_get_body_geometry(self._h, _dptr(I), _dptr(d)))
        return I, d

    # owned context (host-buffer API) --------------------------------------------------------
    def context_set_state(self, positions, velocities, stream=None):
        x = np.ascontiguousarray(positions, dtype=np.float64)
        v = np.ascontiguousarray(velocities, dtype=np.float64)
        _lib.check(self._lib.rbx_context_set_state(self._h, _stream_handle(stream), _dptr(x), _dptr(v)))

    def context_load(self, positions, velocities, stream=None):
        """Write positions and velocities into the owned buffers as they are (no body rebuild)."""
        x = np.ascontiguousarray(positions, dtype=np.float64)
        v = np.ascontiguousarray(velocities, dtype=np.float64)
        _lib.check(self._lib.rbx_context_load(self._h, _stream_handle(stream), _dptr(x), _dptr(v)))

    def context_buffers(self):
        b = _lib.Buffers()
        _lib.check(self._lib.rbx_context_buffers(self._h, ctypes.byref(b)))
        return b

    def context_get_state(self, stream=None):
        x = np.zeros((self.num_atoms, 3))
        v = np.zeros((self.num_atoms, 3))
        _lib.check(self._lib.rbx_context_get_state(self._h, _stream_handle(stream), _dptr(x), _dptr(v)))
        return x, v

    def step_host(self, nsteps, dt, forces, positions_out, velocities_out, stream=None):
        """Host-buffer step: arrays must be C-contiguous float64 [num_atoms, 3]."""
        _lib.check(self._lib.rbx_step_host(self._h, _stream_handle(stream), int(nsteps), float(dt), _dptr(forces),
                                           _dptr(positions_out), _dptr(velocities_out)))

    def context_set_forces(self, forces, stream=None):
        f = np.ascontiguousarray(forces, dtype=np.float64)
        _lib.check(self._lib.rbx_context_set_forces(self._h, _stream_handle(stream), _dptr(f)))

    def context_step(self, kind, dt, stream=None):
        """part1, part2 or fused on the owned buffers."""
        fn = {"part1": self._lib.rbx_integrate_part1, "part2": self._lib.rbx_integrate_part2,
              "fused": self._lib.rbx_integrate_fused}[kind]
        b = self.context_buffers()
        _lib.check(fn(self._h, _stream_handle(stream), ctypes.byref(b), float(dt)))

    def step_host_async(self, nsteps, dt, forces, positions_out, velocities_out, stream=None):
        """Pipelined step_host: returns at once; the host arrays (C-contiguous float64, pinned for
        overlap) must stay alive and untouched until step_host_wait()."""
        _lib.check(self._lib.rbx_step_host_async(self._h, _stream_handle(stream), int(nsteps), float(dt),
                                                 _dptr(forces), _dptr(positions_out), _dptr(velocities_out)))

    def step_host_wait(self):
        _lib.check(self._lib.rbx_step_host_wait(self._h))

    def context_kinetic_energies(self, stream=None):
        out = np.zeros(2)
        b = self.context_buffers()
        _lib.check(self._lib.rbx_kinetic_energies(self._h, _stream_handle(stream), ctypes.byref(b), _dptr(out)))
        return out
