"""The CPU oracle against golden vectors produced by the reference's own code.

Fixtures in tests/golden/*.npz come from tests/golden/make_golden.py, which runs the reference's
unmodified classes (src/Lattice.h, src/Hamiltonian.h, src/DynLanczosSolver.h,
src/Observables.h, src/dynamics.h) compiled by oracle/ref/build_ref.py.
"""
import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN, golden_names, parse_param_text

OPS = ["Sx", "Sy", "Sz", "Sp", "Sm", "Spe3", "Sme3", "Jsx", "Jsy", "Jsz", "Jex", "Jey", "JexJeyJez", "JsxJsyJsz"]
TOTALS = ["JsxTotal", "JsyTotal", "JszTotal", "JexTotal", "JeyTotal"]


def load(name):
    g = np.load(f"{GOLDEN}/{name}.npz")
    p = parse_param_text(g["params"])
    m = O.Model(p["Model"], int(p["NumberofSitesLx"]), int(p["NumberofSitesLy"]), int(p["IsPeriodicX"]),
                int(p["IsPeriodicY"]), *[float(p[k]) for k in ["Kxx", "Kyy", "Kzz", "Bxx", "Byy", "Bzz"]], 0.0,
                int(p["Threads"]))
    return g, p, m


@pytest.mark.parametrize("name", golden_names())
def test_lattice_and_hamiltonian(name):
    g, p, m = load(name)
    nb = O.lattice(p["Model"], int(p["NumberofSitesLx"]), int(p["NumberofSitesLy"]), int(p["IsPeriodicX"]),
                   int(p["IsPeriodicY"]))
    assert (nb == g["neigh"][:, : nb.shape[1]]).all()
    assert np.array_equal(m.hdiag(), g["hdiag"])
    x = O.random_start(int(g["testvec_seed"]), m.D, normalize=False)
    hx = m.hv(x)
    # same operation order as the reference's COO scatter: bit-identical
    assert np.array_equal(hx[: g["hx"].size], g["hx"])


@pytest.mark.parametrize("name", golden_names())
def test_lanczos(name):
    g, p, m = load(name)
    v0 = O.random_start(int(p["RandomSeed"]), m.D)
    r = m.lanczos(v0, int(p["LanczosSteps"]), float(p["LanczosEps"]), p["LancType"])
    # alpha/beta were printed by the reference with 16 significant digits
    np.testing.assert_allclose(r["alpha"], g["alpha"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(r["beta"][: g["beta"].size], g["beta"], rtol=0, atol=1e-14)
    # Ritz values: reference uses LAPACK zheev, the oracle its own QL; both are backward stable
    np.testing.assert_allclose(r["ritz"], g["ritz"], rtol=0, atol=1e-13)
    assert abs(r["ritz"][0] - g["ritz"][0]) / abs(g["ritz"][0]) < 1e-14
    if "psi" in g.files:
        assert abs(abs(np.vdot(g["psi"], m.psi())) - 1.0) < 1e-12


@pytest.mark.parametrize("name", [n for n in golden_names() if "JeJe" in np.load(f"{GOLDEN}/{n}.npz").files])
def test_dynamics(name):
    g, p, m = load(name)
    v0 = O.random_start(int(p["RandomSeed"]), m.D)
    m.lanczos(v0, int(p["LanczosSteps"]), float(p["LanczosEps"]), p["LancType"])
    for key, which in (("JeJe", "Energy Current"), ("JsJs", "Spin Current"), ("SSLocal", "LocalSzSz")):
        s = m.dynamics(which)
        ref = g[key]
        assert s.shape == ref.shape
        err = np.abs(s - ref).max()
        assert err <= 1e-10 * max(1.0, np.abs(ref).max()), (key, err)


@pytest.mark.parametrize("name", [n for n in golden_names() if "proj_Jex" in np.load(f"{GOLDEN}/{n}.npz").files])
def test_operators(name):
    g, p, m = load(name)
    x = O.random_start(int(g["testvec_seed"]), m.D, normalize=False)
    y1, y2 = [O.random_start(int(s), m.D, normalize=False) for s in g["probe_seeds"]]

    def proj(o):
        return np.array([np.vdot(y1, o), np.vdot(y2, o), np.vdot(o, o)])

    for op in OPS:
        for s in range(m.N):
            o = m.apply(op, s, x)
            np.testing.assert_allclose(proj(o), g["proj_" + op][s], rtol=1e-13, atol=1e-12)
            if "full_" + op in g.files:
                assert np.array_equal(o, g["full_" + op][s]), (op, s)
    for op in TOTALS:
        o = m.apply(op, 0, x)
        np.testing.assert_allclose(proj(o), g["proj_" + op], rtol=1e-13, atol=1e-12)
        if "full_" + op in g.files:
            assert np.array_equal(o, g["full_" + op])


CORR_PAIRS = [("Sz", "Sz"), ("Sx", "Sy"), ("Sp", "Sm"), ("Jsx", "Jsy"), ("Jex", "Jey")]


@pytest.mark.parametrize("name", [n for n in golden_names() if "corr_Sz_Sz" in np.load(f"{GOLDEN}/{n}.npz").files])
def test_two_point_corr(name):
    """Observables::TwoPointCorr (src/Observables.h:131-158) on the reference's own ground state."""
    g, p, m = load(name)
    for a, b in CORR_PAIRS:
        c = m.two_point(a, b, g["psi"])
        np.testing.assert_allclose(c, g[f"corr_{a}_{b}"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", [n for n in golden_names() if "localJe" in np.load(f"{GOLDEN}/{n}.npz").files])
def test_measure_local_je(name):
    """Observables::measureLocalJe (src/Observables.h:88-104): <gs|Je_x,i|gs>, <gs|Je_y,i|gs> per site,
    evaluated by the oracle's operators on the reference's own ground state (printed by the reference
    at 17 digits)."""
    g, p, m = load(name)
    if "psi" not in g.files:
        pytest.skip("ground state not stored for this case")
    psi = g["psi"]
    je = np.array([[np.vdot(psi, m.apply(op, s, psi)) for op in ("Jex", "Jey")] for s in range(m.N)])
    np.testing.assert_allclose(je, g["localJe"], rtol=0, atol=1e-15)
