"""The drop-in executable against the reference's own executable.

tests/golden/refout_* were written by the reference's unmodified main (compiled from its sources by
oracle/ref/build_ref.py, generated by tests/golden/make_golden.py --refout) for the parameter file
tests/golden/refout_kitaev12m60.inp (60 Lanczos steps: short of the step where the reference's own
output starts to depend on its summation order).  Our LanczosCond must write the same files: same
rows, same separators, values equal to the 6 significant digits the reference's stream writes."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO

pytestmark = pytest.mark.gpu
esc = pytest.importorskip("energyspincurrents_gb300")


def test_lanczoscond_writes_reference_files(tmp_path):
    from energyspincurrents_gb300 import build
    build.build()
    exe = os.path.join(REPO, "energyspincurrents_gb300", "_build", "LanczosCond")
    shutil.copy(os.path.join(GOLDEN, "refout_kitaev12m60.inp"), tmp_path / "params.inp")
    r = subprocess.run([exe, "params.inp"], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "measuring: site, <sx>, <sy>, <sz>" in r.stdout and "Alpha and beta of Tridiag Matrix" in r.stdout
    for fn in ("JeJe_outSpectrum.real", "JsJs_outSpectrum.real"):
        ours = open(tmp_path / fn).read()
        ref = open(os.path.join(GOLDEN, f"refout_kitaev12m60_{fn}")).read()
        # layout: identical row count, separators and leading blanks
        lo, lr = ours.split(" \n "), ref.split(" \n ")
        assert len(lo) == len(lr)
        assert [len(x.split(" \t ")) for x in lo] == [len(x.split(" \t ")) for x in lr]
        a = np.array([[float(t) for t in row.split()] for row in lo if row.strip()])
        b = np.array([[float(t) for t in row.split()] for row in lr if row.strip()])
        # 6 significant digits in both files: rounding of the last printed digit
        assert np.all(np.abs(a - b) <= 1e-5 * np.maximum(np.abs(b), 1e-3) + 1e-12), fn


def test_lanczoscond_usage_error():
    exe = os.path.join(REPO, "energyspincurrents_gb300", "_build", "LanczosCond")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode != 0
