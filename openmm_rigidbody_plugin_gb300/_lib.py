"""ctypes binding of librbx.so (the C ABI declared in include/rbx.h).

The library is the only compute path: there is no CPU fallback. ``load()`` raises if the library
has not been built (``python -m openmm_rigidbody_plugin_gb300.build``) or cannot be loaded.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librbx.so")

PRECISIONS = {"single": 0, "mixed": 1, "double": 2}

RBX_OK = 0
STATUS_NAMES = {1: "invalid argument", 2: "CUDA error", 3: "bad call order", 4: "unsupported", 5: "numerical failure"}
RBX_ERR_NUMERIC = 5

# Every exported symbol of include/rbx.h: (name, restype, argtypes)
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)


class Buffers(ctypes.Structure):
    """rbx_buffers: OpenMM-layout device buffers (borrowed)."""
    _fields_ = [("posq", ctypes.c_void_p), ("posq_correction", ctypes.c_void_p), ("velm", ctypes.c_void_p),
                ("force", ctypes.c_void_p), ("stride", ctypes.c_int)]


_bp = ctypes.POINTER(Buffers)

SIGNATURES = [
    ("rbx_last_error", ctypes.c_char_p, []),
    ("rbx_version", ctypes.c_int, []),
    ("rbx_create", ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _ip, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("rbx_destroy", ctypes.c_int, [_vp]),
    ("rbx_set_atom_locations", ctypes.c_int, [_vp, _ip]),
    ("rbx_upload_state", ctypes.c_int, [_vp, _dp, _dp]),
    ("rbx_upload_state_device", ctypes.c_int, [_vp, _vp, _bp]),
    ("rbx_get_num_dof", ctypes.c_int, [_vp, _ip]),
    ("rbx_get_num_dof_reference", ctypes.c_int, [_vp, _ip]),
    ("rbx_check_state", ctypes.c_int, [_vp, _vp, _ip, _ip]),
    ("rbx_set_tile_threads", ctypes.c_int, [_vp, ctypes.c_int]),
    ("rbx_get_tile_threads", ctypes.c_int, [_vp, _ip]),
    ("rbx_get_num_bodies", ctypes.c_int, [_vp, _ip]),
    ("rbx_get_num_free", ctypes.c_int, [_vp, _ip]),
    ("rbx_get_rotation_mode", ctypes.c_int, [_vp, _ip]),
    ("rbx_integrate_part1", ctypes.c_int, [_vp, _vp, _bp, ctypes.c_double]),
    ("rbx_integrate_part2", ctypes.c_int, [_vp, _vp, _bp, ctypes.c_double]),
    ("rbx_integrate_fused", ctypes.c_int, [_vp, _vp, _bp, ctypes.c_double]),
    ("rbx_kinetic_energies", ctypes.c_int, [_vp, _vp, _bp, _dp]),
    ("rbx_set_constraints", ctypes.c_int, [_vp, ctypes.c_int, _ip]),
    ("rbx_free_atoms_delta", ctypes.c_int, [_vp, _vp, _bp, _vp, ctypes.c_double]),
    ("rbx_integrate_part1_delta", ctypes.c_int, [_vp, _vp, _bp, _vp, ctypes.c_double]),
    ("rbx_set_compute_refined_energies", ctypes.c_int, [_vp, ctypes.c_int]),
    ("rbx_get_compute_refined_energies", ctypes.c_int, [_vp, _ip]),
    ("rbx_refined_kinetic_energies", ctypes.c_int, [_vp, _vp, _bp, _dp]),
    ("rbx_potential_energy_refinement", ctypes.c_int, [_vp, _vp, _bp, _dp]),
    ("rbx_get_body_state", ctypes.c_int, [_vp, _dp]),
    ("rbx_set_body_state", ctypes.c_int, [_vp, _dp]),
    ("rbx_get_body_state_raw", ctypes.c_int, [_vp, _vp]),
    ("rbx_set_body_state_raw", ctypes.c_int, [_vp, _vp]),
    ("rbx_get_body_geometry", ctypes.c_int, [_vp, _dp, _dp]),
    ("rbx_get_body_atoms", ctypes.c_int, [_vp, _ip, _ip]),
    ("rbx_context_set_state", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_context_buffers", ctypes.c_int, [_vp, _bp]),
    ("rbx_context_set_forces", ctypes.c_int, [_vp, _vp, _dp]),
    ("rbx_context_get_state", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_context_load", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_context_get_range", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _dp, _dp]),
    ("rbx_context_sync_bodies", ctypes.c_int, [_vp, _vp]),
    ("rbx_step_host", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp]),
    ("rbx_step_host_async", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_double, _dp, _dp, _dp]),
    ("rbx_step_host_wait", ctypes.c_int, [_vp]),
    ("rbx_last_launch_count", ctypes.c_int, [_vp]),
    ("rbx_kinetic_energies_static", ctypes.c_int, [_dp, ctypes.c_int, ctypes.c_int, _dp, _dp, _vp, _ip, ctypes.c_int,
                                                   ctypes.c_int, _vp, _dp]),
    ("rbx_batch_create", ctypes.c_int, [ctypes.POINTER(_vp), ctypes.c_int, _ip, _dp, _dp, _ip, _dp, _dp, _dp, _dp,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    ("rbx_batch_destroy", ctypes.c_int, [_vp]),
    ("rbx_batch_set_state", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_batch_get_state", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_batch_get_body_state", ctypes.c_int, [_vp, _vp]),
    ("rbx_batch_get_system_state", ctypes.c_int, [_vp, _vp, ctypes.c_int, _dp, _dp]),
    ("rbx_batch_restore", ctypes.c_int, [_vp, _vp, _vp, _dp, _dp]),
    ("rbx_batch_step", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_double]),
    ("rbx_batch_relax", ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("rbx_batch_energies", ctypes.c_int, [_vp, _vp, _dp]),
    ("rbx_batch_autotune", ctypes.c_int, [_vp, _vp, ctypes.c_double, ctypes.c_int, _ip]),
    ("rbx_batch_set_tuning", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
    ("rbx_batch_set_tile_threads", ctypes.c_int, [_vp, ctypes.c_int]),
    ("rbx_batch_get_tile_threads", ctypes.c_int, [_vp, _ip]),
    ("rbx_batch_forces", ctypes.c_int, [_vp, _vp, _dp, _dp]),
    ("rbx_batch_get_num_dof", ctypes.c_int, [_vp, _ip]),
    ("rbx_batch_status", ctypes.c_int, [_vp, _vp, _ip, _ip]),
    ("rbx_batch_memory", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_size_t)]),
    ("rbx_batch_list_builds", ctypes.c_int, [_vp, _vp, ctypes.POINTER(ctypes.c_uint)]),
    ("rbx_batch_set_graph_steps", ctypes.c_int, [_vp, ctypes.c_int]),
    ("rbx_batch_set_timing", ctypes.c_int, [_vp, ctypes.c_int]),
    ("rbx_batch_kernel_times", ctypes.c_int, [_vp, _dp, _dp, _ip]),
    ("rbx_batch_last_launch_count", ctypes.c_int, [_vp]),
]

_lib = None


class RbxError(RuntimeError):
    """A librbx call returned a non-zero status."""

    def __init__(self, status, message):
        super().__init__(f"{message} [{STATUS_NAMES.get(status, status)}]")
        self.status = status


def load(path=None):
    """Load librbx.so and declare its signatures; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"librbx.so not found at {path}: build it with "
                          "`python -m openmm_rigidbody_plugin_gb300.build` (nvcc required)")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != RBX_OK:
        raise RbxError(status, load().rbx_last_error().decode())
    return status
