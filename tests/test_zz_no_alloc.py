"""rbx_kinetic_energies_static: the kinetic-energy reduction for callers that cannot allocate
device memory (a serving process working inside a device-memory budget it reserved up front, a
host framework whose pool owns every allocation, a loop that cannot take the synchronisation
of cudaMalloc). It reads caller-owned device arrays and keeps its scratch in a fixed static
device array, so it must give the same energies as rbx_kinetic_energies, call after call.

This file is named to be collected last, so a stop-at-first-failure run has already run every
other test when it reaches this one.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ITEMS = 4_194_304  # bodies or free atoms one call accepts (1024 block sums of 4096)


PRECISIONS = {"single": 0, "mixed": 1, "double": 2}
# Agreement with the allocating entry point: both reduce in FP64, in different partitions. In single
# and mixed precision the handle keeps 1/m and 1/I as float-float pairs (about 2^-48 relative),
# while the caller's copies below are FP64.
RTOL = {"single": 1e-10, "mixed": 1e-10, "double": 1e-12}


@pytest.fixture(scope="module", params=list(PRECISIONS))
def setup(request):
    import torch
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    from openmm_rigidbody_plugin_gb300 import _lib, build, kernel
    from openmm_rigidbody_plugin_gb300 import workloads as W
    prec = request.param
    build.build_library()
    lib = _lib.load()
    s = W.mixed_system(n_bodies=5000, n_free=700, fractions=(0.6, 0.25, 0.15), seed=31)
    k = kernel.IntegratorKernel(s.masses, s.body_indices, rotation_mode=0, precision=prec)
    # one padding slot beyond the atoms: velm row of zeros, a massless particle (w = 1/m = 0)
    buf = kernel.DeviceBuffers(s.num_atoms, precision=prec, stride=s.num_atoms + 1)
    buf.set_positions(s.positions)
    buf.set_velocities(s.velocities, s.masses)
    buf.set_forces(W.gaussian_forces(s.num_atoms, seed=5, sd=50.0))
    k.upload_state(s.positions, s.velocities)
    for _ in range(5):
        k.part1(buf, 0.002)
        k.part2(buf, 0.002)
    reference = k.kinetic_energies(buf)

    # Caller-owned device copies of the body arrays in the layout the entry point reads: FP64 body
    # state rows (the handle's state, exactly, in every precision) and the velm array of the
    # handle's precision (float4 in single, double4 in mixed and double).
    nb = k.num_bodies
    state = k.body_state()                       # [nb, 14]
    I, _ = k.geometry()                          # [nb, 3]
    first, atoms = k.body_atoms()
    invm = 1.0 / np.add.reduceat(np.asarray(s.masses)[atoms], first[:-1])
    invI = np.where(I > 0, 1.0 / np.where(I > 0, I, 1.0), 0.0)
    dev = buf.velm.device
    d_state = torch.as_tensor(np.ascontiguousarray(state.T), device=dev)
    d_invm = torch.as_tensor(invm, device=dev)
    d_invI = torch.as_tensor(np.ascontiguousarray(invI.T), device=dev)
    free = np.nonzero(s.body_indices == 0)[0].astype(np.int32)
    d_free = torch.as_tensor(free, device=dev)
    d_free_massless = torch.as_tensor(np.append(free, np.int32(s.num_atoms)), device=dev)
    torch.cuda.synchronize()
    return dict(lib=lib, torch=torch, prec=prec, k=k, buf=buf, nb=nb, nf=len(free), reference=reference,
                state=d_state, invm=d_invm, invI=d_invI, free=d_free, free_massless=d_free_massless)


def _call(S, out, nb=None, nf=None, stride=None, free=None):
    torch = S["torch"]
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    free = S["free"] if free is None else free
    return S["lib"].rbx_kinetic_energies_static(
        ctypes.cast(S["state"].data_ptr(), dp), S["nb"] if nb is None else nb, S["nb"] if stride is None else stride,
        ctypes.cast(S["invm"].data_ptr(), dp), ctypes.cast(S["invI"].data_ptr(), dp),
        ctypes.c_void_p(S["buf"].velm.data_ptr()), ctypes.cast(free.data_ptr(), ip),
        S["nf"] if nf is None else nf, PRECISIONS[S["prec"]], stream, ctypes.cast(out.data_ptr(), dp))


def test_static_scratch_matches_allocating_entry_point_twice(setup):
    S = setup
    torch = S["torch"]
    results = []
    for _ in range(2):  # the second call reuses the scratch left by the first
        out = torch.full((2,), float("nan"), dtype=torch.float64, device=S["buf"].velm.device)
        assert _call(S, out) == 0, S["lib"].rbx_last_error()
        torch.cuda.synchronize()
        results.append(out.cpu().numpy())
        np.testing.assert_allclose(results[-1], S["reference"], rtol=RTOL[S["prec"]])
    assert np.array_equal(results[0], results[1])


def test_massless_free_slot_contributes_nothing(setup):
    S = setup
    torch = S["torch"]
    out = torch.full((2,), float("nan"), dtype=torch.float64, device=S["buf"].velm.device)
    assert _call(S, out, nf=S["nf"] + 1, free=S["free_massless"]) == 0, S["lib"].rbx_last_error()
    torch.cuda.synchronize()
    np.testing.assert_allclose(out.cpu().numpy(), S["reference"], rtol=RTOL[S["prec"]])


def test_sizes_beyond_the_static_scratch_are_rejected(setup):
    S = setup
    torch = S["torch"]
    out = torch.zeros(2, dtype=torch.float64, device=S["buf"].velm.device)
    # Rejected on the host before anything is read: the counts exceed the documented maximum.
    assert _call(S, out, nb=MAX_ITEMS + 1) == 4
    assert b"at most" in S["lib"].rbx_last_error()
    assert _call(S, out, nf=MAX_ITEMS + 1) == 4
    # a body stride whose 14 rows overflow 32-bit indexing
    assert _call(S, out, stride=(2 ** 31 - 1) // 14 + 1) == 4
    assert b"32-bit" in S["lib"].rbx_last_error()
