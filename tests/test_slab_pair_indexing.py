"""Host-side check (no GPU) of the slab-pair launch arithmetic: tests/slab_pair_check.cu replays,
item by item, the item order, tile offsets and tile copies of the pair kernel
(hv_pass_device.cuh: pair_body) on the library's own plans and passes, and checks that each pass of
a pair writes every state exactly once, that pass B only reads states pass A wrote in the same slab,
that every tile of A(s) precedes every tile of B(s) in the item order (the waits can always end),
and that every address lies inside the vector."""
import os
import subprocess

import pytest

from conftest import REPO

esc = pytest.importorskip("energyspincurrents_gb300")

PKG = os.path.join(REPO, "energyspincurrents_gb300")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    from energyspincurrents_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("slab") / "slab_pair_check")
    nvcc = build._nvcc()
    lib = os.path.join(PKG, "_build")
    cmd = [nvcc, *build.ARCH, "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"), "-I", lib, "-I",
           os.path.join(REPO, "include"), os.path.join(REPO, "tests", "slab_pair_check.cu"), "-o", out, "-L", lib,
           "-lesc", "-Xlinker", "-rpath", "-Xlinker", lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


# (Lx, Ly, tile bits, log2 threads per tile): 24 sites with 2048-, 4096- and 8192-state tiles
# (4 and 3 passes), 28 sites with 8192-state tiles and 1024 threads
@pytest.mark.parametrize("shape", [(3, 8, 11, 9), (3, 8, 12, 9), (3, 8, 13, 9), (3, 8, 12, 8), (7, 4, 13, 10)])
def test_slab_pair_index_arithmetic(checker, shape):
    r = subprocess.run([checker, *map(str, shape)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("pair ")]
    assert lines and all(": OK" in l for l in lines), r.stdout
