"""librbx.so loads, exports every entry point of include/rbx.h, and validates arguments before
touching a GPU (runs without one)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from openmm_rigidbody_plugin_gb300 import _lib, build
    build.build_library()
    return _lib.load()


def header_functions():
    text = open(os.path.join(ROOT, "include", "rbx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rbx_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = header_functions()
    assert "rbx_create" in names and "rbx_integrate_fused" in names
    assert len(names) >= 20


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from openmm_rigidbody_plugin_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(header_functions()) == bound


def _create(lib, masses, bidx, mode=0, prec=1):
    h = ctypes.c_void_p()
    m = np.ascontiguousarray(masses, dtype=np.float64)
    b = np.ascontiguousarray(bidx, dtype=np.int32)
    rc = lib.rbx_create(ctypes.byref(h), len(m), b.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                        m.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), mode, prec, 0)
    return rc, h


def test_negative_rotation_mode_rejected(lib):
    """RigidBodyIntegrator::setRotationMode throws for mode < 0 (RigidBodyIntegrator.cpp:28-29)."""
    rc, _ = _create(lib, [1.0, 1.0, 1.0], [1, 1, 1], mode=-1)
    assert rc == 1
    assert b"negative" in lib.rbx_last_error()


def test_bad_precision_and_sizes_rejected(lib):
    rc, _ = _create(lib, [1.0, 1.0], [1, 1], prec=7)
    assert rc == 1
    h = ctypes.c_void_p()
    assert lib.rbx_create(ctypes.byref(h), 0, None, None, 0, 1, 0) == 1


def test_massless_body_atom_rejected(lib):
    rc, _ = _create(lib, [1.0, 0.0, 1.0], [1, 1, 1])
    assert rc == 1
    assert b"no mass" in lib.rbx_last_error()


@pytest.mark.parametrize("prec,limit", [(1, 1024), (0, 1024), (2, 512)])
def test_body_larger_than_a_tile_rejected(lib, prec, limit):
    """A body must fit one tile (1024 atoms in single/mixed, 512 in double): RBX_ERR_UNSUPPORTED,
    before any device call."""
    rc, _ = _create(lib, np.ones(limit + 1), np.ones(limit + 1, dtype=np.int32), prec=prec)
    assert rc == 4
    assert b"exceeds" in lib.rbx_last_error()


def test_new_entry_points_reject_a_null_handle(lib):
    """Constraints, refined energies and the posDelta steps validate their handle first."""
    pairs = np.array([0, 1], dtype=np.int32)
    assert lib.rbx_set_constraints(None, 1, pairs.ctypes.data_as(ctypes.POINTER(ctypes.c_int))) == 1
    assert lib.rbx_set_compute_refined_energies(None, 1) == 1
    out = np.zeros(2)
    assert lib.rbx_refined_kinetic_energies(None, None, None, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 1
    assert lib.rbx_free_atoms_delta(None, None, None, None, 0.002) == 1
    assert lib.rbx_integrate_part1_delta(None, None, None, None, 0.002) == 1


def test_null_handle_calls_fail_cleanly(lib):
    out = ctypes.c_int()
    assert lib.rbx_get_num_bodies(None, ctypes.byref(out)) == 1
    assert lib.rbx_destroy(None) == 0
    assert lib.rbx_last_launch_count(None) == 0


def test_header_is_plain_c_and_links_from_c(lib, tmp_path):
    """include/rbx.h compiles as pedantic C99, and a C program links librbx.so and calls it (no GPU
    call): the boundary a cgo, JNI or ctypes binding sees."""
    import shutil
    import subprocess
    from openmm_rigidbody_plugin_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    src = tmp_path / "use_rbx.c"
    src.write_text('#include "rbx.h"\n#include <stdio.h>\n'
                   'int main(void) { rbx_integrator* h = 0;\n'
                   '  int rc = rbx_create(&h, 0, 0, 0, 0, RBX_PRECISION_MIXED, 0);\n'
                   '  printf("%d %d\\n", rbx_version(), rc); return rc == RBX_ERR_INVALID_ARGUMENT ? 0 : 1; }\n')
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = tmp_path / "use_rbx"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lrbx", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert int(r.stdout.split()[0]) == lib.rbx_version()
