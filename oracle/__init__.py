"""CPU oracle for the Lanczos exact-diagonalisation path (TEST INFRASTRUCTURE ONLY).

A ctypes front-end over oracle/esc_oracle.cpp, a C++ restatement of the reference
fengshi96/EnergySpinCurrents (src/Lattice.h, src/Hamiltonian.h, src/DynLanczosSolver.h,
src/Observables.h, src/dynamics.h).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline may import this package; the product library never does.

Parity status: pinned.  The restatement is checked against golden vectors produced by the
reference's own unmodified sources (tests/golden/, generated by tests/golden/make_golden.py
from a build made by oracle/ref/build_ref.py) and against dense numpy diagonalisation.
"""
import ctypes
import os

import numpy as np

from .build_oracle import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        so = _build()
        L = ctypes.CDLL(so)
        c_int, c_double, c_char_p, c_void_p, c_int64 = (ctypes.c_int, ctypes.c_double, ctypes.c_char_p,
                                                         ctypes.c_void_p, ctypes.c_int64)
        P = ctypes.POINTER
        L.or_last_error.restype = c_char_p
        L.or_lattice.argtypes = [c_char_p, c_int, c_int, c_int, c_int, P(c_int), P(c_int)]
        L.or_model_create.restype = c_void_p
        L.or_model_create.argtypes = [c_char_p, c_int, c_int, c_int, c_int] + [c_double] * 7 + [c_int, c_int]
        L.or_model_destroy.argtypes = [c_void_p]
        L.or_model_info.argtypes = [c_void_p, P(c_int), P(c_int64), P(c_int), P(c_int), P(c_int), P(c_int)]
        L.or_hdiag.argtypes = [c_void_p, c_void_p]
        L.or_hv.argtypes = [c_void_p, c_void_p, c_void_p]
        L.or_hv_rows.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_int]
        L.or_hv_rows_c64.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_int64, c_int]
        L.or_random_start.argtypes = [c_int64, c_int64, c_void_p, c_int]
        L.or_tridiag.argtypes = [c_int, c_void_p, c_void_p, c_void_p, c_void_p]
        L.or_lanczos.argtypes = [c_void_p, c_void_p, c_int, c_double, c_char_p, c_void_p, c_void_p, c_void_p, P(c_int)]
        L.or_get_psi.argtypes = [c_void_p, c_void_p]
        L.or_lanczos3.argtypes = [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p]
        L.or_set_ritz.argtypes = [c_void_p, c_int, c_void_p, c_void_p]
        L.or_apply.argtypes = [c_void_p, c_char_p, c_int, c_void_p, c_void_p]
        L.or_dynamics.argtypes = [c_void_p, c_char_p, c_int, c_double, c_double, c_void_p]
        L.or_cf_lanczos.argtypes = [c_void_p, c_void_p, c_int, c_int, c_void_p, c_void_p, P(c_int)]
        L.or_cf_eval.argtypes = [c_void_p, c_void_p, c_int, c_double, c_int, c_void_p, c_double, c_void_p]
        L.or_dot.argtypes = [c_int64, c_void_p, c_void_p, c_void_p]
        L.or_two_point.argtypes = [c_void_p, c_char_p, c_char_p, c_void_p, c_void_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def lattice(model, Lx, Ly, pbcx=1, pbcy=1):
    """Neighbour table N x ncol (honeycomb columns 0=z, 1=y, 2=x; src/Lattice.h:497-522)."""
    N = Lx * Ly
    out = np.full(N * 3, -1, dtype=np.int32)
    nc = ctypes.c_int()
    lib().or_lattice(model.encode(), Lx, Ly, pbcx, pbcy, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                     ctypes.byref(nc))
    return out[: N * nc.value].reshape(N, nc.value)


def random_start(seed, D, normalize=True):
    """Reference start vector (src/DynLanczosSolver.h:465-474), complex128."""
    v = np.empty(D, dtype=np.complex128)
    lib().or_random_start(int(seed), int(D), _p(v), 1 if normalize else 0)
    return v


def tridiag_eig(d, e, vectors=True):
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = d.size
    ee = np.zeros(n)
    ee[: n - 1] = e[: n - 1]
    w = np.empty(n)
    z = np.empty((n, n), order="F") if vectors else None
    rc = lib().or_tridiag(n, _p(d), _p(ee), _p(w), _p(z) if vectors else None)
    if rc != 0:
        raise RuntimeError("tridiagonal eigensolver did not converge")
    return (w, z) if vectors else w


def cf_eval(a, b, E0, omega, eta):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    omega = np.ascontiguousarray(omega, dtype=np.float64)
    out = np.empty(omega.size * 2)
    lib().or_cf_eval(_p(a), _p(b), a.size, float(E0), omega.size, _p(omega), float(eta), _p(out))
    return out[0::2] + 1j * out[1::2]


class Model:
    """Hamiltonian + Lanczos + observables restated on the CPU (one instance per parameter set)."""

    def __init__(self, model="Kitaev", Lx=3, Ly=4, pbcx=1, pbcy=1, Kxx=1.0, Kyy=1.0, Kzz=1.0,
                 Bxx=0.0, Byy=0.0, Bzz=0.0, J=0.0, threads=8, coo=True):
        L = lib()
        self.h = L.or_model_create(model.encode(), Lx, Ly, pbcx, pbcy, Kxx, Kyy, Kzz, Bxx, Byy, Bzz, J,
                                   threads, 1 if coo else 0)
        if not self.h:
            raise ValueError(L.or_last_error().decode())
        N = ctypes.c_int(); D = ctypes.c_int64(); nx = ctypes.c_int(); ny = ctypes.c_int(); nz = ctypes.c_int()
        L.or_model_info(self.h, ctypes.byref(N), ctypes.byref(D), ctypes.byref(nx), ctypes.byref(ny),
                        ctypes.byref(nz), None)
        self.N, self.D = N.value, D.value
        self.nbonds = (nx.value, ny.value, nz.value)
        self.params = dict(model=model, Lx=Lx, Ly=Ly, Kxx=Kxx, Kyy=Kyy, Kzz=Kzz, Bxx=Bxx, Byy=Byy, Bzz=Bzz, J=J)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_model_destroy(self.h)
            self.h = None

    def bonds(self):
        n = sum(self.nbonds)
        b = np.zeros(2 * max(n, 1), dtype=np.int32)
        z = ctypes.c_int()
        lib().or_model_info(self.h, ctypes.byref(z), ctypes.byref(ctypes.c_int64()), ctypes.byref(z),
                            ctypes.byref(z), ctypes.byref(z), b.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
        b = b[: 2 * n].reshape(n, 2)
        nx, ny, nz = self.nbonds
        return b[:nx], b[nx:nx + ny], b[nx + ny:]

    def hdiag(self):
        out = np.empty(self.D, dtype=np.complex128)
        lib().or_hdiag(self.h, _p(out))
        return out

    def hv(self, v):
        v = np.ascontiguousarray(v, dtype=np.complex128)
        out = np.empty_like(v)
        lib().or_hv(self.h, _p(v), _p(out))
        return out

    def hv_rows(self, v, r0, r1, threads=8, c64=False):
        if c64:
            v = np.ascontiguousarray(v, dtype=np.complex64)
            out = np.empty(r1 - r0, dtype=np.complex64)
            lib().or_hv_rows_c64(self.h, _p(v), _p(out), r0, r1, threads)
        else:
            v = np.ascontiguousarray(v, dtype=np.complex128)
            out = np.empty(r1 - r0, dtype=np.complex128)
            lib().or_hv_rows(self.h, _p(v), _p(out), r0, r1, threads)
        return out

    def dense(self):
        """Dense H built column by column from hv (small N only)."""
        H = np.empty((self.D, self.D), dtype=np.complex128)
        e = np.zeros(self.D, dtype=np.complex128)
        for j in range(self.D):
            e[j] = 1.0
            H[:, j] = self.hv(e)
            e[j] = 0.0
        return H

    def lanczos(self, start, M, eps=0.0, lanctype="All"):
        start = np.ascontiguousarray(start, dtype=np.complex128)
        a = np.zeros(M); b = np.zeros(M + 1); r = np.zeros(M)
        n = ctypes.c_int()
        rc = lib().or_lanczos(self.h, _p(start), M, eps, lanctype.encode(), _p(a), _p(b), _p(r), ctypes.byref(n))
        if rc:
            raise RuntimeError(lib().or_last_error().decode())
        n = n.value
        return dict(alpha=a[:n], beta=b[: n + 1], ritz=r[:n], steps=n)

    def lanczos3(self, start, M, want_gs=True):
        """Three-vector FP64 Lanczos without reorthogonalisation on the matrix-free H.v (bases whose
        COO lists or M+1 vectors do not fit); |gs> rebuilt in a second sweep and normalised."""
        start = np.ascontiguousarray(start, dtype=np.complex128)
        a = np.zeros(M); b = np.zeros(M + 1); r = np.zeros(M)
        gs = np.empty(self.D, dtype=np.complex128) if want_gs else None
        if lib().or_lanczos3(self.h, _p(start), M, _p(a), _p(b), _p(r), _p(gs) if want_gs else None):
            raise RuntimeError(lib().or_last_error().decode())
        return dict(alpha=a, beta=b, ritz=r, E0=r[0], gs=gs)

    def psi(self):
        out = np.empty(self.D, dtype=np.complex128)
        lib().or_get_psi(self.h, _p(out))
        return out

    def set_eigenpairs(self, evals, evecs_cols):
        """Solver=ED path: evecs_cols is D x n (columns are eigenvectors)."""
        n = evals.size
        ps = np.ascontiguousarray(evecs_cols.T, dtype=np.complex128)
        lib().or_set_ritz(self.h, n, _p(np.ascontiguousarray(evals, dtype=np.float64)), _p(ps))

    def apply(self, op, site, v):
        v = np.ascontiguousarray(v, dtype=np.complex128)
        out = np.empty_like(v)
        if lib().or_apply(self.h, op.encode(), int(site), _p(v), _p(out)):
            raise ValueError(lib().or_last_error().decode())
        return out

    def dynamics(self, which, omegasteps=1000, domega=0.002, eta=0.005):
        ncol = {"Energy Current": 6, "Spin Current": 15, "LocalSzSz": 9}[which]
        out = np.empty((omegasteps + 1) * ncol)
        if lib().or_dynamics(self.h, which.encode(), omegasteps, domega, eta, _p(out)):
            raise ValueError(lib().or_last_error().decode())
        return out.reshape(omegasteps + 1, ncol)

    def two_point(self, opA, opB, psi=None):
        """Observables::TwoPointCorr: N x N matrix <gs| A_si B_sj |gs> (si >= sj, mirrored)."""
        out = np.empty(self.N * self.N * 2)
        p = None if psi is None else np.ascontiguousarray(psi, dtype=np.complex128)
        if lib().or_two_point(self.h, opA.encode(), opB.encode(), None if p is None else _p(p), _p(out)):
            raise ValueError(lib().or_last_error().decode())
        return (out[0::2] + 1j * out[1::2]).reshape(self.N, self.N)

    def cf_lanczos(self, phi, steps, reortho=False):
        phi = np.ascontiguousarray(phi, dtype=np.complex128)
        a = np.zeros(steps); b = np.zeros(steps)
        n = ctypes.c_int()
        lib().or_cf_lanczos(self.h, _p(phi), steps, 1 if reortho else 0, _p(a), _p(b), ctypes.byref(n))
        return a[: n.value], b[: n.value]
