"""Host-side checks that need no GPU: the C-ABI library loads and exports every entry point
declared in include/esc.h, the parameter-file parser follows the reference's rules, the
neighbour tables match the oracle, and device entry points fail loudly without a device."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN, REPO, golden_names, parse_param_text

esc = pytest.importorskip("energyspincurrents_gb300")


@pytest.fixture(scope="module", autouse=True)
def built():
    from energyspincurrents_gb300 import build
    build.build()


def header_symbols():
    text = open(os.path.join(REPO, "include", "esc.h")).read()
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(esc_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol():
    syms = header_symbols()
    assert len(syms) >= 17
    L = ctypes.CDLL(esc.lib_path())
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(esc.EXPORTS) == syms


def write(tmp_path, text, name="p.inp"):
    f = tmp_path / name
    f.write_text(text)
    return str(f)


def test_parser_reference_file():
    p = esc.ConstVariables(os.path.join(REPO, "tests", "golden", "midinput.inp"))
    assert (p.Lx, p.Ly, p.seed, p.model, p.solver, p.lanctype) == (3, 4, 3, "Kitaev", "none", "All")
    assert (p.Kxx, p.Bzz, p.lanczos_steps, p.threads, p.energy_curr_dyn, p.local_skw) == (1.0, 0.3, 100, 8, 1, 0)
    # reference constants as defaults of the added keys
    assert (p.omega_steps, p.domega, p.eta, p.jheis, p.dyn_mode, p.reortho) == (1000, 0.002, 0.005, 0.0, 0, 1)


BASE = """NumberofSitesLx=3
NumberofSitesLy=4
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=3
Model=Kitaev
Solver=none
Temperature=1
LanczosEps=0
Threads=8
LancType=All
Kxx=1.0
Kyy=1.0
Kzz=1.0
Bxx=0.3
Byy=0.3
Bzz=0.3
"""


def test_parser_semantics(tmp_path):
    # first parseable match wins; "Key =" (space) is not the key; comments are other keys
    t = BASE.replace("Kxx=1.0", "#Kxx=7\nKxx =5\nKxx=abc\nKxx=-0.5\nKxx=9")
    p = esc.ConstVariables(write(tmp_path, t))
    assert p.Kxx == -0.5
    assert p.lanczos_steps == 200                  # default (src/ParametersEngine.h:85-90)
    p = esc.ConstVariables(write(tmp_path, BASE + "LanczosSteps=57.9\nRandomSeed=99\n"))
    assert p.lanczos_steps == 57 and p.seed == 3   # int() truncation; first RandomSeed wins
    p = esc.ConstVariables(write(tmp_path, BASE + "Jheis=0.1\nDynMode=CF\nOmegaSteps=1999\nOmegaMax=6\nEta=0.05\n"))
    assert p.jheis == 0.1 and p.dyn_mode == 1 and p.omega_steps == 1999 and abs(p.domega - 6 / 1999) < 1e-15


@pytest.mark.parametrize("drop,msg", [("Kzz=1.0\n", "Kzz= argument is missing in the input file!"),
                                      ("Model=Kitaev\n", "Model= argument is missing in the input file!")])
def test_parser_missing_key(tmp_path, drop, msg):
    with pytest.raises(ValueError, match=msg):
        esc.ConstVariables(write(tmp_path, BASE.replace(drop, "")))


def test_parser_dynamics_needs_all(tmp_path):
    with pytest.raises(ValueError, match="LancType=All"):
        esc.ConstVariables(write(tmp_path, BASE.replace("LancType=All", "LancType=GS") + "EnergyCurrDynamics=1\n"))


def test_parser_missing_file():
    with pytest.raises(ValueError, match="cannot open"):
        esc.ConstVariables("/nonexistent/params.inp")


@pytest.mark.parametrize("shape", [(2, 4), (3, 4), (2, 6), (4, 4), (3, 6), (3, 8), (4, 6), (7, 4), (4, 8)])
@pytest.mark.parametrize("pbc", [(1, 1), (0, 1), (1, 0)])
def test_lattice_matches_oracle(shape, pbc):
    Lx, Ly = shape
    nb = esc.lattice(dict(Lx=Lx, Ly=Ly, pbcx=pbc[0], pbcy=pbc[1]))
    ref = O.lattice("Kitaev", Lx, Ly, *pbc)
    assert (nb == ref).all()
    if pbc == (1, 1):
        # full 3-coordination, symmetric, N/2 bonds per type
        for c in range(3):
            assert (nb[nb[:, c], c] == np.arange(Lx * Ly)).all()


def test_lattice_goldens():
    for name in golden_names():
        g = np.load(f"{GOLDEN}/{name}.npz")
        p = parse_param_text(g["params"])
        nb = esc.lattice(dict(Lx=int(p["NumberofSitesLx"]), Ly=int(p["NumberofSitesLy"]),
                              pbcx=int(p["IsPeriodicX"]), pbcy=int(p["IsPeriodicY"])))
        assert (nb == g["neigh"]).all(), name


def test_chain_lattice():
    nb = esc.lattice(dict(Lx=6, Ly=1, model="HeisenbergChain", pbcx=1))
    assert nb[:, 0].tolist() == [1, 2, 3, 4, 5, 0] and nb[:, 1].tolist() == [5, 0, 1, 2, 3, 4]


def test_bad_model():
    with pytest.raises(esc.EscError, match="Unknown Model"):
        esc.lattice(dict(model="Ising"))


def test_device_entry_points_fail_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(esc.EscError, match="no CUDA device"):
        esc.Handle(dict(Lx=2, Ly=4))


@pytest.mark.parametrize("shape,J", [((3, 4), 0.0), ((4, 4), 0.1), ((3, 6), 0.1), ((3, 8), 0.1), ((7, 4), 0.05),
                                     ((4, 8), 0.05), ((5, 6), 0.05)])
@pytest.mark.parametrize("tile", [(13, 3), (10, 3), (14, 4), (12, 1)])
def test_planner_covers_every_term(shape, J, tile):
    """esc_plan builds the pass list (make_passes throws if any bond fits no tile) and a bijective
    site -> bit relabelling; pass counts stay small."""
    Lx, Ly = shape
    b = -0.02 / 3 ** 0.5
    perm, npass = esc.plan(dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, jheis=J), *tile)
    assert sorted(perm.tolist()) == list(range(Lx * Ly))
    N = Lx * Ly
    T = tile[0]
    assert npass == 1 if N <= T else 2 <= npass <= 2 + 2 * (N - T)


@pytest.mark.parametrize("shape,tile,most", [((3, 8), 12, 3), ((4, 8), 13, 4), ((4, 8), 12, 5), ((7, 4), 13, 3)])
def test_planner_annealed_pass_counts(shape, tile, most):
    """Pass counts of the annealed covering (Kitaev-Heisenberg, every bond off-diagonal): 3 passes
    of 4096-state tiles at 24 sites and 4 of 8192-state tiles at 32, one fewer than the greedy
    covering alone (ESC_PLAN_GREEDY)."""
    Lx, Ly = shape
    b = -0.02 / 3 ** 0.5
    p = dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, jheis=0.05)
    perm, npass = esc.plan(p, tile, 3)
    assert sorted(perm.tolist()) == list(range(Lx * Ly))
    assert npass <= most
    if tile == 13 and Lx * Ly == 32 or tile == 12 and Lx * Ly == 24:
        os.environ["ESC_PLAN_GREEDY"] = "1"
        try:
            assert esc.plan(p, tile, 3)[1] == npass + 1
        finally:
            del os.environ["ESC_PLAN_GREEDY"]


def test_default_plan_takes_8192_state_tiles_above_26_sites_when_fewer_passes():
    """Without ESC_TILE_BITS the plan uses 4096-state tiles, or 8192-state tiles above 26 sites when
    they need fewer passes (N=32: 4 instead of 5; N=28: 3 instead of 4); esc_plan reports the same
    default as esc_create."""
    b = -0.02 / 3 ** 0.5
    for (Lx, Ly), want, t12 in [((3, 8), 3, 3), ((7, 4), 3, 4), ((4, 8), 4, 5)]:
        p = dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, jheis=0.05)
        assert esc.plan(p)[1] == want
        assert esc.plan(p, 12, 3)[1] == t12
