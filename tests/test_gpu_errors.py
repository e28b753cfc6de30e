"""Error paths of the ground-state Lanczos (checks after the recurrence, mirroring the reference's
runtime_error on LAPACK failure, src/DynLanczosSolver.h:398-411), reached with ordinary inputs:
nothing is planted in the device code and no kernel faults or waits.

  * beta = 0: a Hamiltonian that is diagonal in the basis (no transverse couplings, no transverse
    field) maps a basis vector onto itself, so w = H v - alpha v is exactly zero after the first
    step and the Krylov space is exhausted.
  * NaN: a NaN coupling makes every H.v NaN, so alpha is not finite.
Both must come back as ESC_ERR_NUMERIC with a message, and the handle must stay usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
esc = pytest.importorskip("energyspincurrents_gb300")

S3 = 3 ** 0.5


def test_beta_zero_breakdown_is_reported():
    h = esc.Handle(dict(Lx=2, Ly=4, Kxx=0.0, Kyy=0.0, Kzz=-1.0, Bxx=0.0, Byy=0.0, Bzz=0.1, seed=0))
    e0 = np.zeros(h.D, dtype=np.complex128)
    e0[5] = 1.0
    for dt in (np.complex128, np.complex64):
        with pytest.raises(esc.EscError, match="beta=0") as ei:
            h.lanczos_gs(steps=6, start=e0.astype(dt), lanctype="GS", reortho=0, dtype=dt)
        assert ei.value.status == esc.ESC_ERR_NUMERIC
    # the handle still works: a start vector with weight on two diagonal entries has a
    # 2-dimensional Krylov space, and two steps give the lower diagonal entry exactly
    v = np.zeros(h.D, dtype=np.complex128)
    v[3] = v[12] = 2 ** -0.5
    r = h.lanczos_gs(steps=2, start=v, lanctype="GS", reortho=0)
    d = np.real(np.array([h.hv(np.eye(1, h.D, k, dtype=np.complex128)[0])[k] for k in (3, 12)]))
    assert abs(r["E0"] - d.min()) < 1e-12


def test_nan_coefficients_are_reported():
    b = -0.05 / S3
    h = esc.Handle(dict(Lx=2, Ly=4, Kxx=float("nan"), Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, seed=0))
    for dt in (np.complex128, np.complex64):
        with pytest.raises(esc.EscError, match="NaN/Inf in Lanczos coefficients") as ei:
            h.lanczos_gs(steps=8, lanctype="GS", reortho=0, dtype=dt)
        assert ei.value.status == esc.ESC_ERR_NUMERIC
        with pytest.raises(esc.EscError, match="NaN/Inf"):
            h.lanczos_gs(steps=8, lanctype="All", reortho=1, dtype=dt)


def test_bad_dtype_is_refused():
    h = esc.Handle(dict(Lx=2, Ly=4, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0))
    x = np.zeros(h.D, dtype=np.complex128)
    lib = esc.lib()
    st = lib.esc_hv(h.h, esc._ptr(x), esc._ptr(np.empty_like(x)), 5, 0)
    assert st == esc.ESC_ERR_PARAM and b"dt must be" in lib.esc_last_error(h.h)
