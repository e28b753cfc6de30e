"""esc_rayleigh_noalloc: the allocation-free variant of esc_rayleigh.

It exists for callers that cannot allocate device memory (code inside another framework's memory
pool, processes under a fixed device-memory budget): it takes the model parameters and a device
vector, keeps its scratch in a static device array, and must agree with the handle-based
esc_rayleigh.  Collected last (file name) so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
esc = pytest.importorskip("energyspincurrents_gb300")
torch = pytest.importorskip("torch")

S3 = 3 ** 0.5


def params(Lx, Ly, J=0.1, h=0.05):
    b = -h / S3
    return dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-0.9, Kzz=-1.1, Bxx=b, Byy=b, Bzz=b, jheis=J)


def noalloc(P, v_dev, dt, stream):
    E = ctypes.c_double()
    st = esc.lib().esc_rayleigh_noalloc(ctypes.byref(P.p), ctypes.c_void_p(v_dev.data_ptr()), dt,
                                         ctypes.c_void_p(stream), ctypes.byref(E))
    if st != esc.ESC_OK:
        raise esc.EscError(st, esc.lib().esc_last_error(None).decode())
    return E.value


@pytest.mark.parametrize("shape", [(2, 4), (3, 6), (3, 8)])
@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_noalloc_matches_handle_twice(shape, dtype):
    P = esc.ConstVariables(**params(*shape))
    h = esc.Handle(P)
    x = O.random_start(21, h.D).astype(dtype)
    expect = h.rayleigh(x)                                  # existing entry point (handle scratch)
    dev = torch.from_numpy(x).to("cuda")
    stream = torch.cuda.current_stream().cuda_stream
    dt = esc.C64 if dtype == np.complex64 else esc.C128
    tol = 1e-12 * max(abs(expect), 1.0)                    # energies are O(1); a random vector sits near 0
    for _ in range(2):                                      # the second call reuses the same static scratch
        got = noalloc(P, dev, dt, stream)
        assert abs(got - expect) <= tol, (got, expect)


def test_noalloc_rejects_too_many_sites():
    P = esc.ConstVariables(**params(13, 2))                 # 26 sites: beyond the static scratch
    dummy = torch.zeros(2, dtype=torch.complex128, device="cuda")
    with pytest.raises(esc.EscError, match="at most 25 sites"):
        noalloc(P, dummy, esc.C128, torch.cuda.current_stream().cuda_stream)


def test_noalloc_rejects_bad_dtype():
    """A dtype value other than complex128 / complex64 is refused before any kernel reads the vector."""
    P = esc.ConstVariables(**params(2, 4))
    dummy = torch.zeros(256, dtype=torch.complex64, device="cuda")
    with pytest.raises(esc.EscError, match="dt must be"):
        noalloc(P, dummy, 7, torch.cuda.current_stream().cuda_stream)
