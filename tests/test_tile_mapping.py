"""The step kernel's block -> tile map (csrc/rbx_tiles.h), compiled for the host and checked on the CPU.

Every grid block must map to exactly one body tile or one free-atom tile, and every tile must get
exactly one block: a block without a tile, or two blocks on one tile, would skip or double-step
atoms. Free-atom tile j must also run right after the body tiles that cover the same span of slots,
which is what the placement is for.
"""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "rbx_tiles.h"
int main(int argc, char** argv) {
    for (int a = 1; a + 1 < argc; a += 2) {
        const int nb = atoi(argv[a]), nf = atoi(argv[a + 1]);
        printf("%d %d:", nb, nf);
        for (int i = 0; i < nb + nf; i++) printf(" %d", rbx::tile_of_block(i, nb, nf));
        printf("\n");
    }
    return 0;
}
"""

SIZES = [(0, 1), (1, 0), (1, 1), (2, 7), (7, 2), (3, 3), (10, 1), (1, 10), (4200, 391), (4224, 196),
         (31, 5), (100000, 1), (5, 100000), (1000, 999), (0, 0)]


@pytest.fixture(scope="module")
def tiles(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    d = tmp_path_factory.mktemp("tiles")
    src, exe = d / "tiles.cpp", d / "tiles"
    src.write_text(DRIVER)
    csrc = os.path.join(ROOT, "openmm_rigidbody_plugin_gb300", "csrc")
    subprocess.run([gxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", csrc, str(src), "-o", str(exe)], check=True)
    args = [str(v) for nb_nf in SIZES for v in nb_nf]
    out = subprocess.run([str(exe)] + args, check=True, capture_output=True, text=True).stdout
    maps = {}
    for line in out.splitlines():
        head, _, rest = line.partition(":")
        nb, nf = (int(v) for v in head.split())
        maps[(nb, nf)] = [int(v) for v in rest.split()]
    return maps


@pytest.mark.parametrize("nb,nf", SIZES)
def test_every_tile_gets_exactly_one_block(tiles, nb, nf):
    m = tiles[(nb, nf)]
    assert len(m) == nb + nf
    assert sorted(t for t in m if t >= 0) == list(range(nb))
    assert sorted(-1 - t for t in m if t < 0) == list(range(nf))


@pytest.mark.parametrize("nb,nf", [s for s in SIZES if s[0] and s[1]])
def test_free_tile_follows_the_body_tiles_of_its_slot_span(tiles, nb, nf):
    """Free-atom tile j holds the free atoms of the j-th of nf equal spans of slots, which the body
    tiles up to (j + 1) nb / nf cover: it runs right after the first ceil((j + 1) nb / nf) body
    tiles (the last of them reaching into the span's end), and free-atom tiles run in order."""
    m = tiles[(nb, nf)]
    bodies_before, j_prev = 0, -1
    for t in m:
        if t >= 0:
            bodies_before += 1
            continue
        j = -1 - t
        assert j == j_prev + 1
        j_prev = j
        assert bodies_before == -(-(j + 1) * nb // nf)
