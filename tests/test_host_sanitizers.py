"""The host side of rbx_create under AddressSanitizer and UndefinedBehaviorSanitizer, on the CPU.

rbx_create compacts body ids, orders bodies and free atoms, and packs tiles before its first CUDA
call (cleanBodyIndices and the atom lists of RigidBodySystem.cpp:28-105). Without a GPU that call
fails cleanly. rbx_host.cpp and rbx_batch.cpp are rebuilt with the sanitizers and linked with the
library's other objects. A driver then feeds rbx_create adversarial inputs: few large bodies,
mostly singletons, waters, negative ids, one body of every atom, sparse huge ids, and massless
free atoms. Every call must return a status with no sanitizer report: RBX_OK, a validation error,
or RBX_ERR_CUDA at the device call.
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

DRIVER = r"""
#include <cstdio>
#include <random>
#include <vector>
#include "rbx.h"
int main() {
    std::mt19937 rng(7);
    int counts[8] = {0};
    for (int trial = 0; trial < 240; trial++) {
        const int n = 1 + (int)(rng() % (trial < 200 ? 3000 : 60000));
        std::vector<int> b(n);
        std::vector<double> m(n, 1.0);
        const int kind = trial % 6;
        for (int i = 0; i < n; i++) {
            switch (kind) {
                case 0: b[i] = (int)(rng() % 50); break;
                case 1: b[i] = (int)(rng() % (n + 1)); break;
                case 2: b[i] = i / 3 + 1; break;
                case 3: b[i] = (rng() % 4) ? (int)(rng() % 1500) : -(int)(rng() % 5); break;
                case 4: b[i] = 1; break;
                default: b[i] = (int)(rng() % 7) * 1000000; break;
            }
            if (rng() % 17 == 0 && b[i] <= 0) m[i] = 0.0;
        }
        for (int prec = 0; prec < 3; prec++) {
            rbx_integrator* h = nullptr;
            const int rc = rbx_create(&h, n, b.data(), m.data(), (int)(rng() % 12), prec, 0);
            if (rc < 0 || rc > 7) return 2;
            counts[rc]++;
            if (rc == RBX_OK) rbx_destroy(h);
            else if (h != nullptr) return 3;
        }
    }
    for (int k = 0; k < 8; k++) printf("%d ", counts[k]);
    printf("\n");
    return 0;
}
"""


def test_rbx_create_host_planning_under_sanitizers(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    from openmm_rigidbody_plugin_gb300 import build
    build.build_library()
    objs = [os.path.join(build.BUILD, os.path.splitext(s)[0] + ".o") for s in build.SOURCES
            if s.endswith(".cu")]
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(build.nvcc())))
    flags = ["-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
             "-fno-sanitize-recover=undefined", "-I", os.path.join(cuda, "include"), "-I", os.path.join(ROOT, "include")]
    san = []
    for src in ("rbx_host.cpp", "rbx_batch.cpp"):
        o = str(tmp_path / (src + ".o"))
        r = subprocess.run([gxx, *flags, "-c", os.path.join(build.CSRC, src), "-o", o], capture_output=True, text=True)
        if r.returncode != 0 and "sanitize" in r.stderr:
            pytest.skip("sanitizer runtime not available")
        assert r.returncode == 0, r.stderr[-2000:]
        san.append(o)
    drv = tmp_path / "drive.cpp"
    drv.write_text(DRIVER)
    exe = str(tmp_path / "drive")
    r = subprocess.run([gxx, *flags, str(drv), *san, *objs, "-L", os.path.join(cuda, "lib64"), "-lcudart",
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr, r.stderr[-4000:]
    counts = [int(c) for c in r.stdout.split()]
    assert sum(counts) == 240 * 3
