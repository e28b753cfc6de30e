"""Generate the golden fixtures in tests/golden/*.npz from the reference's own code.

Runs oracle/_ref/golden_driver (the reference's unmodified classes, compiled by
oracle/ref/build_ref.py from the reference source tree) on the parameter sets below and stores
its outputs.  Needs the reference tree, so it runs in the build container only; the fixtures it
writes are committed and are all that the tests read.

    python tests/golden/make_golden.py
"""
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

import oracle  # noqa: E402
from oracle.ref import build_ref  # noqa: E402

S3 = 3 ** 0.5

# name -> (parameter file text, full operator vectors?)
# (No HeisenbergChain case: the reference's Chain() prints N1neigh_(i,2) on a two-column table,
#  src/Lattice.h:187, which fails the Matrix bounds assert in its shipped Debug build.)
CASES = {
    # the reference's shipped example input (2-fold degenerate ground state: spectra not pinned)
    "midinput": ("""NumberofSitesLx=3
NumberofSitesLy=4
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=3
Model=Kitaev
Solver=none
Reortho=1
Temperature=1
LanczosEps=0
LanczosSteps=100
Threads=8
LancType=All
LocalSkw=1
SpinCurrDynamics=0
EnergyCurrDynamics=1
Kxx=1.0
Kyy=1.0
Kzz=1.0
Bxx=0.3
Byy=0.3
Bzz=0.3
""", False),
    # 12-site Kitaev model in a [111] field, K=-1, h=0.05 (non-degenerate ground state)
    "kitaev12": (f"""NumberofSitesLx=3
NumberofSitesLy=4
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=0
Model=Kitaev
Solver=none
Temperature=0
LanczosEps=0
LanczosSteps=200
Threads=8
LancType=All
LocalSkw=1
EnergyCurrDynamics=1
Kxx=-1.0
Kyy=-1.0
Kzz=-1.0
Bxx={-0.05 / S3!r}
Byy={-0.05 / S3!r}
Bzz={-0.05 / S3!r}
""", False),
    # same model, 60 steps: short of the step (~66) where the reference's own Lanczos sequence
    # starts to depend on its summation order, so every output is reproducible to ~1e-12
    "kitaev12m60": (f"""NumberofSitesLx=3
NumberofSitesLy=4
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=0
Model=Kitaev
Solver=none
Temperature=0
LanczosEps=0
LanczosSteps=60
Threads=8
LancType=All
LocalSkw=1
EnergyCurrDynamics=1
Kxx=-1.0
Kyy=-1.0
Kzz=-1.0
Bxx={-0.05 / S3!r}
Byy={-0.05 / S3!r}
Bzz={-0.05 / S3!r}
""", False),
    # anisotropic couplings and an off-axis field on the (2,6) cluster: catches x/y/z mix-ups
    "aniso12": ("""NumberofSitesLx=2
NumberofSitesLy=6
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=5
Model=Kitaev
Solver=none
Temperature=0
LanczosEps=0
LanczosSteps=150
Threads=4
LancType=All
LocalSkw=1
EnergyCurrDynamics=1
Kxx=-1.0
Kyy=-0.8
Kzz=-1.2
Bxx=0.02
Byy=-0.05
Bzz=0.03
""", False),
    # 8 sites: small enough to store every operator vector in full
    "kitaev8": ("""NumberofSitesLx=2
NumberofSitesLy=4
IsPeriodicX=1
IsPeriodicY=1
RandomSeed=1
Model=Kitaev
Solver=none
Temperature=0
LanczosEps=0
LanczosSteps=60
Threads=2
LancType=All
LocalSkw=1
EnergyCurrDynamics=1
Kxx=-1.0
Kyy=-1.0
Kzz=-1.0
Bxx=-0.1
Byy=-0.07
Bzz=-0.04
""", True),
    # 16 sites, open boundaries along x (exercises the non-periodic neighbour table)
    "kitaev16obc": ("""NumberofSitesLx=4
NumberofSitesLy=4
IsPeriodicX=0
IsPeriodicY=1
RandomSeed=7
Model=Kitaev
Solver=none
Temperature=0
LanczosEps=0
LanczosSteps=80
Threads=8
LancType=All
LocalSkw=0
EnergyCurrDynamics=0
Kxx=-1.0
Kyy=-1.0
Kzz=-1.0
Bxx=-0.03
Byy=-0.03
Bzz=-0.03
""", False),
}

OPS = ["Sx", "Sy", "Sz", "Sp", "Sm", "Spe3", "Sme3", "Jsx", "Jsy", "Jsz", "Jex", "Jey", "JexJeyJez", "JsxJsyJsz"]
TOTALS = ["JsxTotal", "JsyTotal", "JszTotal", "JexTotal", "JeyTotal"]
TESTVEC_SEED = 12345
PROBE_SEEDS = (777, 778)


def parse_params(text):
    d = {}
    for line in text.splitlines():
        if "=" in line:
            k, v = line.split("=", 1)
            d[k] = v.strip()
    return d


def probes(D):
    return [oracle.random_start(s, D, normalize=False) for s in PROBE_SEEDS]


def project(vecs, D):
    """vecs: (..., D) -> (..., 3) complex: <y1|v>, <y2|v>, |v|^2."""
    y1, y2 = probes(D)
    v = vecs.reshape(-1, D)
    out = np.stack([v @ y1.conj(), v @ y2.conj(), (np.abs(v) ** 2).sum(1) + 0j], axis=1)
    return out.reshape(vecs.shape[:-1] + (3,))


# Observables::TwoPointCorr pairs dumped by golden_driver.cpp
CORR_PAIRS = [("Sz", "Sz"), ("Sx", "Sy"), ("Sp", "Sm"), ("Jsx", "Jsy"), ("Jex", "Jey")]


def parse_local_je(log, N):
    """<Je_x,i>, <Je_y,i> per site from the lines the reference's measureLocalJe prints
    (src/Observables.h:88-104: 'site \\t (re,im) \\t (re,im) \\t  \\t (re,im)'), N x 2 complex."""
    seg = log.split("@@LOCALJE_BEGIN")[1].split("@@LOCALJE_END")[0]
    rows = {}
    for line in seg.splitlines():
        vals = re.findall(r"\(([-+0-9.eE]+),([-+0-9.eE]+)\)", line)
        head = line.strip().split()
        if len(vals) == 3 and head and head[0].isdigit():
            rows[int(head[0])] = [complex(float(a), float(b)) for a, b in vals[:2]]
    if sorted(rows) != list(range(N)):
        raise RuntimeError("measureLocalJe output incomplete")
    return np.array([rows[s] for s in range(N)], dtype=np.complex128)


def run_case(name, text, full_ops, exe):
    p = parse_params(text)
    N = int(p["NumberofSitesLx"]) * int(p["NumberofSitesLy"])
    D = 2 ** N
    work = tempfile.mkdtemp(prefix="golden_")
    try:
        pf = os.path.join(work, "params.inp")
        with open(pf, "w") as f:
            f.write(text)
        x = oracle.random_start(TESTVEC_SEED, D, normalize=False)
        tv = os.path.join(work, "testvec.bin")
        x.tofile(tv)
        out = os.path.join(work, "out")
        os.makedirs(out)
        r = subprocess.run([exe, pf, out, tv], capture_output=True, text=True, check=True)
        log = r.stdout
        seg = log.split("@@LANCZOS_BEGIN")[1].split("@@LANCZOS_END")[0]
        m = re.search(r"Alpha and beta of Tridiag Matrix :(.*)", seg)
        pairs = re.findall(r"\(([-+0-9.eE]+),([-+0-9.eE]+)\)", m.group(1))
        alpha = np.array([float(a) for a, _ in pairs])
        beta = np.array([float(b) for _, b in pairs])
        rd = lambda fn, dt: np.fromfile(os.path.join(out, fn), dtype=dt)
        res = dict(params=np.array(text), N=N, testvec_seed=TESTVEC_SEED, probe_seeds=np.array(PROBE_SEEDS),
                   neigh=rd("neigh.bin", np.int32).reshape(N, 3), hdiag=rd("hdiag.bin", np.complex128),
                   alpha=alpha, beta=beta, ritz=rd("ritz.bin", np.float64))
        hx = rd("hx.bin", np.complex128)
        res["hx"] = hx if N <= 12 else hx[:4096]
        res["hx_proj"] = project(hx, D)
        psi = rd("psi.bin", np.complex128)
        if N <= 12:
            res["psi"] = psi
        complete = p["Model"] == "Kitaev" and bool((res["neigh"] >= 0).all())
        if complete:
            opv = {}
            for op in OPS:
                v = rd(f"op_{op}.bin", np.complex128).reshape(N, D)
                res[f"proj_{op}"] = project(v, D)
                if full_ops:
                    opv[op] = v
            for op in TOTALS:
                v = rd(f"op_{op}.bin", np.complex128)
                res[f"proj_{op}"] = project(v, D)
                if full_ops:
                    opv[op] = v
            for k, v in opv.items():
                res[f"full_{k}"] = v
            if p.get("LancType") == "All":
                res["localS"] = rd("localS.bin", np.complex128).reshape(N, 3)
                res["localJe"] = parse_local_je(log, N)
                for a, b in CORR_PAIRS:
                    res[f"corr_{a}_{b}"] = rd(f"corr_{a}_{b}.bin", np.complex128).reshape(N, N)
                for fn, key in (("JeJe_outSpectrum.real", "JeJe"), ("JsJs_outSpectrum.real", "JsJs"),
                                ("2SSLocal_outSpectrum.real", "SSLocal")):
                    res[key] = np.loadtxt(os.path.join(out, fn))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
        return res
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main():
    out = build_ref.build()
    exe = os.path.join(out, "golden_driver")
    for name, (text, full) in CASES.items():
        res = run_case(name, text, full, exe)
        print(name, "N=%d" % res["N"], "E0=%.15f" % res["ritz"][0], "steps=%d" % res["alpha"].size)


if __name__ == "__main__" and "--refout" not in sys.argv:
    main()


def make_reference_outputs(name="kitaev12m60"):
    """Run the reference's unmodified main (oracle/_ref/LanczosCond) and keep its output files
    (format fixtures for the drop-in executable: default stream precision, ' \\t ' separators)."""
    out = build_ref.build()
    text = CASES[name][0]
    work = tempfile.mkdtemp(prefix="refout_")
    try:
        with open(os.path.join(work, "params.inp"), "w") as f:
            f.write(text)
        subprocess.run([os.path.join(out, "LanczosCond"), "params.inp"], cwd=work, capture_output=True, check=True)
        for fn in ("JeJe_outSpectrum.real", "JsJs_outSpectrum.real"):
            shutil.copy(os.path.join(work, fn), os.path.join(HERE, f"refout_{name}_{fn}"))
        with open(os.path.join(HERE, f"refout_{name}.inp"), "w") as f:
            f.write(text)
    finally:
        shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__" and "--refout" in sys.argv:
    make_reference_outputs()
