"""Slab-pair H.v launches: two passes of the tiled H.v in one cooperative launch, slab by slab, so
that the second pass finds the slab's input and the first pass's partial result in the L2 cache
(hv_pass_device.cuh: pair_body).  From 27 sites on the library pairs passes by itself; here
ESC_SLAB_PAIRS=1 pairs them at 24 sites and ESC_SLAB_PAIRS=0 runs the same passes, in the same
order, one launch each.  The pair kernel performs each state's operations in the same order as the
single-pass kernel, so the two H.v agree bit for bit."""
import time

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
esc = pytest.importorskip("energyspincurrents_gb300")

S3 = 3 ** 0.5


def kitaev(Lx=3, Ly=8, J=0.1, h=0.05, **kw):
    b = -h / S3
    return dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, jheis=J, **kw)


def relerr(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


# 24 sites: T=11 gives 4 passes (two pairs, the last pair carries the alpha epilogue; specialised
# kernels only), T=12 and T=13 give 3 passes (one pair and one pass alone; ahead-of-time and
# specialised pair kernels)
CONFIGS = [("11", "require"), ("12", "0"), ("12", "require"), ("13", "0"), ("13", "require")]


def handles(monkeypatch, tile_bits, jit, p):
    monkeypatch.setenv("ESC_TILE_BITS", tile_bits)
    monkeypatch.setenv("ESC_JIT", jit)
    monkeypatch.setenv("ESC_SLAB_PAIRS", "0")
    h0 = esc.Handle(p)
    monkeypatch.setenv("ESC_SLAB_PAIRS", "1")
    h1 = esc.Handle(p)
    return h0, h1


@pytest.mark.parametrize("tile_bits,jit", CONFIGS)
def test_slab_pairs_bitwise_equal(tile_bits, jit, monkeypatch):
    """Paired and unpaired launches of the same passes give bit-identical complex64 H.v, which agrees
    with the oracle's matrix-free H.v to complex64 rounding."""
    p = kitaev()
    h0, h1 = handles(monkeypatch, tile_bits, jit, p)
    x = O.random_start(21, h0.D, normalize=False).astype(np.complex64)
    y0, y1 = h0.hv(x), h1.hv(x)
    assert np.array_equal(y0, y1)
    m = O.Model("Kitaev", 3, 8, 1, 1, -1.0, -1.0, -1.0, p["Bxx"], p["Byy"], p["Bzz"], 0.1, 4, False)
    assert relerr(y1.astype(np.complex128), m.hv(x.astype(np.complex128))) < 2e-6
    # a second call (counters zeroed again before the launch) gives the same vector
    assert np.array_equal(h1.hv(x), y1)


@pytest.mark.parametrize("tile_bits,jit", [("11", "require"), ("13", "0")])
def test_slab_pairs_lanczos(tile_bits, jit, monkeypatch):
    """The complex64 Lanczos without reorthogonalisation (CUDA-graph recurrence, alpha from the
    epilogue of the last launch) with paired passes: deterministic, and alpha / beta / E0 as with
    unpaired passes to complex64 rounding (the alpha partials come from a different grid)."""
    p = kitaev(seed=0)
    h0, h1 = handles(monkeypatch, tile_bits, jit, p)
    x = O.random_start(0, h0.D)
    kw = dict(steps=40, lanctype="OnlyEgs", reortho=0, start=x, dtype=np.complex64, want_gs=False)
    r0, r1 = h0.lanczos_gs(**kw), h1.lanczos_gs(**kw)
    r1b = esc.Handle(p).lanczos_gs(**kw)   # ESC_SLAB_PAIRS=1 still set: paired again
    assert np.array_equal(r1["alpha"], r1b["alpha"]) and np.array_equal(r1["beta"], r1b["beta"])
    assert np.abs(r1["alpha"][:20] - r0["alpha"][:20]).max() < 1e-5
    assert np.abs(r1["beta"][:20] - r0["beta"][:20]).max() < 1e-5
    assert abs(r1["E0"] - r0["E0"]) < 1e-5 * abs(r0["E0"])


@pytest.mark.parametrize("tile_bits,jit", CONFIGS)
def test_slab_pair_wait_gives_up(tile_bits, jit, monkeypatch):
    """The waits of a pair launch are bounded: with a per-slab count that is never reached
    (ESC_TEST_SLAB_STALL=1), the first wait gives up after about a second, every later wait of the
    launch returns at once, the launch ends, and the call reports ESC_ERR_TIMEOUT.  The handle is
    usable afterwards and computes the same H.v as before.  (That the call stalls at all also shows
    that this configuration runs the pair kernel.)"""
    p = kitaev()
    monkeypatch.setenv("ESC_TILE_BITS", tile_bits)
    monkeypatch.setenv("ESC_JIT", jit)
    monkeypatch.setenv("ESC_SLAB_PAIRS", "1")
    h = esc.Handle(p)
    x = O.random_start(5, h.D, normalize=False).astype(np.complex64)
    good = h.hv(x)
    monkeypatch.setenv("ESC_TEST_SLAB_STALL", "1")
    t0 = time.perf_counter()
    with pytest.raises(esc.EscError) as ei:
        h.hv(x)
    el = time.perf_counter() - t0
    assert ei.value.status == esc.ESC_ERR_TIMEOUT, str(ei.value)
    assert 0.5 < el < 30.0, el
    monkeypatch.delenv("ESC_TEST_SLAB_STALL")
    assert np.array_equal(h.hv(x), good)
