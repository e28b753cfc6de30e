"""Oracle fixtures for the FP64 configuration tests at sizes where the oracle needs CPU-hours
(test infrastructure; the tests only read the .npz files this writes).

C2 (tests/golden/c2_n24.npz): 24-site honeycomb (3x4 unit cells, Lx=3, Ly=8, PBC), K=-1, J=0.1,
h=0.05 along [111], reference start vector from RandomSeed=0.  300 ground-state Lanczos steps
without reorthogonalisation (three vectors, ground state rebuilt in a second sweep), then the
continued-fraction spectra of the energy current (JeJe) and the spin current (JsJs) with 500 CF
steps per resolvent on 2000 omega in [0, 6], eta = 0.05.
C2 local (tests/golden/c2_n18_local.npz): the LocalSzSz spectrum in the same form on the 18-site
cluster (3x3 unit cells): 18 sites x 11 resolvents per site, too many for the CPU at 24 sites.

Everything runs in the CPU oracle (oracle/esc_oracle.cpp: matrix-free H.v, the three-vector
Lanczos, the CF recurrence, the reference's operators); the spectra are assembled below from
the resolvents with the reference's column order and elastic subtractions (src/dynamics.h:345-460
JeJe, :222-341 JsJs, :64-217 LocalSzSz), off-diagonal correlations by the polarisation identity.

    python tests/golden/make_config_fixtures.py [c2|local|all] [--threads T]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402

S3 = 3 ** 0.5
K, J, HF, SEED = -1.0, 0.1, 0.05, 0
GS_STEPS, CF_STEPS = 300, 500
NW, WMAX, ETA = 2000, 6.0, 0.05


def model(Lx, Ly, threads):
    b = -HF / S3
    return O.Model("Kitaev", Lx, Ly, 1, 1, K, K, K, b, b, b, J, threads, False)


def resolvents(m, E0, phis, log):
    """G(omega) = <phi|(omega + E0 - i eta - H)^-1|phi> from the CF coefficients of each phi."""
    om = WMAX / (NW - 1) * np.arange(NW)
    G, A, B = [], [], []
    for i, phi in enumerate(phis):
        t = time.time()
        a, b = m.cf_lanczos(phi, CF_STEPS)
        G.append(O.cf_eval(a, b, E0, om, ETA))
        A.append(a)
        B.append(b)
        log(f"  resolvent {i + 1}/{len(phis)}: {a.size} steps, {time.time() - t:.0f} s")
    return om, G, A, B


def pol(Gab, Gaa, Gbb, Giab):
    """S_ab and S_ba from G(a+b), G(a+ib) and the diagonal resolvents."""
    X = Gab - Gaa - Gbb
    Y = Giab - Gaa - Gbb
    return 0.5 * (X - 1j * Y), 0.5 * (X + 1j * Y)


def current_spectra(m, gs, E0, je, log):
    ops = ["JexTotal", "JeyTotal"] if je else ["JsxTotal", "JsyTotal", "JszTotal"]
    ch = [m.apply(o, 0, gs) for o in ops]
    ch.append(sum(ch))                                   # t = x + y (+ z)
    el = [np.vdot(gs, c) for c in ch]
    pairs = [(0, 1)] if je else [(0, 1), (0, 2), (1, 2)]
    runs = list(ch)
    at = []
    for a, b in pairs:
        ip = len(ch) - 1 if je else len(runs)
        if not je:
            runs.append(ch[a] + ch[b])
        at.append((ip, len(runs)))
        runs.append(ch[a] + 1j * ch[b])
    om, G, A, B = resolvents(m, E0, runs, log)
    nc = len(ch)
    S = {(c, c): G[c] for c in range(nc)}
    for q, (a, b) in enumerate(pairs):
        S[(a, b)], S[(b, a)] = pol(G[at[q][0]], G[a], G[b], G[at[q][1]])
    dn = om - 1j * ETA
    t = nc - 1
    if je:
        cols = [om, (S[0, 0] - np.conj(el[0]) * el[0] / dn).imag, (S[1, 1] - np.conj(el[1]) * el[1] / dn).imag,
                (S[0, 1] - np.conj(el[0]) * el[1] / dn).imag, S[1, 0].imag,    # yx: the reference's unset Jez[0] = 0
                (S[t, t] - np.conj(el[t]) * el[t] / dn).imag]
    else:
        cols = [om]
        for a, b in ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)):
            v = S[a, b] - np.conj(el[a]) * el[b] / dn
            cols += [v.real, v.imag]
        v = S[t, t] - np.conj(el[t]) * el[t] / dn
        cols += [v.real, v.imag]
    return np.stack(cols, 1), A, B, np.array(el)


def local_spectrum(m, gs, E0, log):
    nw = NW
    acc = np.zeros((nw, 8), dtype=np.complex128)
    om = WMAX / (NW - 1) * np.arange(NW)
    dn = om - 1j * ETA
    for si in range(m.N):
        log(f" site {si}")
        v = [m.apply(o, si, gs) for o in ("Sx", "Sy", "Sz", "Spe3", "Sme3")]   # x y z p m
        el = [np.vdot(gs, c) for c in v]
        pp = [(0, 1), (0, 2), (1, 2)]
        runs = list(v) + [r for a, b in pp for r in (v[a] + v[b], v[a] + 1j * v[b])]
        _, G, _, _ = resolvents(m, E0, runs, log)
        R = [G[0], G[1], G[2]]
        for q, (a, b) in enumerate(pp):
            R.append(pol(G[5 + 2 * q], G[a], G[b], G[6 + 2 * q])[0])
        # xx yy zz xy xz yz, then S^-e3 S^+e3 and S^+e3 S^-e3 (dynamics.h:189-196)
        acc[:, :6] += np.stack(R, 1)
        acc[:, 6] += G[3]
        acc[:, 7] += G[4]
        acc[:, 0] -= np.conj(el[0]) * el[0] / dn
        acc[:, 3] -= np.conj(el[0]) * el[1] / dn
        acc[:, 4] -= np.conj(el[0]) * el[2] / dn
        acc[:, 1] -= np.conj(el[1]) * el[1] / dn
        acc[:, 5] -= np.conj(el[1]) * el[2] / dn
        acc[:, 2] -= np.conj(el[2]) * el[2] / dn
        acc[:, 6] -= el[4] * el[3] / dn                 # Sm*Sp without conjugation, as written (:185-186)
        acc[:, 7] -= el[3] * el[4] / dn
    return np.concatenate([om[:, None], acc.imag], 1)


def ground_state(m, log):
    t = time.time()
    v0 = O.random_start(SEED, m.D)
    r = m.lanczos3(v0, GS_STEPS)
    log(f" ground state: E0 = {r['E0']:.15f} ({time.time() - t:.0f} s)")
    return r


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="?", default="all", choices=["c2", "local", "all"])
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    args = ap.parse_args()

    def log(s):
        print(time.strftime("%H:%M:%S"), s, flush=True)

    if args.which in ("c2", "all"):
        m = model(3, 8, args.threads)
        r = ground_state(m, log)
        out = dict(params=np.array([3, 8, K, J, HF, SEED, GS_STEPS, CF_STEPS, NW, WMAX, ETA]), E0=r["E0"],
                   alpha=r["alpha"], beta=r["beta"], ritz=r["ritz"][:8])
        for key, je in (("JeJe", True), ("JsJs", False)):
            log(key)
            S, A, B, el = current_spectra(m, r["gs"], r["E0"], je, log)
            out[key] = S
            out[key + "_elastic"] = el
            out[key + "_cf_a"] = np.stack([a[:120] for a in A])
            out[key + "_cf_b"] = np.stack([b[:121] for b in B])
            np.savez_compressed(os.path.join(HERE, "c2_n24.npz"), **out)
        log("c2 done")
    if args.which in ("local", "all"):
        m = model(3, 6, args.threads)
        r = ground_state(m, log)
        S = local_spectrum(m, r["gs"], r["E0"], log)
        np.savez_compressed(os.path.join(HERE, "c2_n18_local.npz"),
                            params=np.array([3, 6, K, J, HF, SEED, GS_STEPS, CF_STEPS, NW, WMAX, ETA]), E0=r["E0"],
                            SSLocal=S)
        log("local done")


if __name__ == "__main__":
    main()
