"""The oracle against independent dense diagonalisation (numpy), including the extensions the
reference does not have (Heisenberg J, continued-fraction spectra, HeisenbergChain)."""
import numpy as np
import pytest

import oracle as O

S3 = 3 ** 0.5


def kit(J=0.0, h=0.05, Lx=3, Ly=4, coo=True):
    b = -h / S3
    return O.Model("Kitaev", Lx, Ly, 1, 1, -1.0, -1.0, -1.0, b, b, b, J, 4, coo)


def test_tridiag_vs_numpy():
    rng = np.random.default_rng(0)
    for n in (1, 2, 7, 60):
        d = rng.standard_normal(n); e = rng.standard_normal(n)
        w, z = O.tridiag_eig(d, e)
        T = np.diag(d) + np.diag(e[: n - 1], 1) + np.diag(e[: n - 1], -1)
        np.testing.assert_allclose(w, np.linalg.eigvalsh(T), atol=1e-13)
        np.testing.assert_allclose(T @ z, z * w, atol=1e-12)


@pytest.mark.parametrize("J", [0.0, 0.1])
def test_spectrum_vs_dense(J):
    m = kit(J)
    H = m.dense()
    assert np.abs(H - H.conj().T).max() == 0.0
    w = np.linalg.eigvalsh(H)
    # lowest four eigenvalues of the 12-site [111]-field model, h=0.05
    expect = {0.0: [-2.50608306, -2.49340255, -2.49164122, -2.49164122],
              0.1: [-2.26756097, -2.24927338, -2.24839706, -2.24839706]}[J]
    np.testing.assert_allclose(w[:4], expect, atol=5e-8)


def test_matrix_free_matches_coo():
    rng = np.random.default_rng(1)
    for J in (0.0, 0.1):
        a, b = kit(J), kit(J, coo=False)
        x = rng.standard_normal(a.D) + 1j * rng.standard_normal(a.D)
        np.testing.assert_allclose(b.hv(x), a.hv(x), atol=1e-13)
        np.testing.assert_allclose(b.hv_rows(x, 100, 900), a.hv(x)[100:900], atol=1e-13)


def test_heisenberg_j_term_is_si_dot_sj():
    """J alone on the honeycomb equals sum over nn bonds of S_i.S_j built from Pauli matrices."""
    m = O.Model("Kitaev", 2, 4, 1, 1, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.7, 2, True)
    H = m.dense()
    sx = np.array([[0, 1], [1, 0]]) / 2; sy = np.array([[0, -1j], [1j, 0]]) / 2; sz = np.array([[1, 0], [0, -1]]) / 2
    N = m.N

    def op(o, s):
        # bit s of the basis index = site s; bit 0 = up
        out = np.array([[1.0]])
        for t in reversed(range(N)):
            out = np.kron(out, o if t == s else np.eye(2))
        return out

    nb = O.lattice("Kitaev", 2, 4)
    Href = np.zeros_like(H)
    for i in range(N):
        for j in set(nb[i]):
            if i < j:
                for o in (sx, sy, sz):
                    Href += 0.7 * op(o, i) @ op(o, j)
    np.testing.assert_allclose(H, Href, atol=1e-14)


def test_cf_matches_exact_lehmann():
    # 8 sites: the Krylov space of A|gs> is exhausted, so the continued fraction is exact
    m = kit(0.1, Lx=2, Ly=4)
    H = m.dense()
    w, V = np.linalg.eigh(H)
    gs = V[:, 0]
    phi = m.apply("JexTotal", 0, gs)
    a, b = m.cf_lanczos(phi, 300, reortho=True)
    om = np.linspace(0, 6, 200)
    eta = 0.05
    g = O.cf_eval(a, b, w[0], om, eta)
    ov = V.conj().T @ phi
    exact = (np.abs(ov)[None, :] ** 2 / (om[:, None] - (w[None, :] - w[0]) - 1j * eta)).sum(1)
    np.testing.assert_allclose(g, exact, atol=1e-9)


def test_chain_vs_dense():
    m = O.Model("HeisenbergChain", 8, 1, 1, 0, 1.0, 0.9, 1.1, 0.1, 0.0, 0.05, 0.0, 2, True)
    H = m.dense()
    sx = np.array([[0, 1], [1, 0]]) / 2; sy = np.array([[0, -1j], [1j, 0]]) / 2; sz = np.array([[1, 0], [0, -1]]) / 2
    N = 8

    def op(o, s):
        out = np.array([[1.0]])
        for t in reversed(range(N)):
            out = np.kron(out, o if t == s else np.eye(2))
        return out

    Href = np.zeros_like(H)
    for i in range(N):
        j = (i + 1) % N
        Href += 1.0 * op(sx, i) @ op(sx, j) + 0.9 * op(sy, i) @ op(sy, j) + 1.1 * op(sz, i) @ op(sz, j)
        Href += 0.1 * op(sx, i) + 0.05 * op(sz, i)
    np.testing.assert_allclose(H, Href, atol=1e-14)
