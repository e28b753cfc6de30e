"""Recipe: compile the reference's own sources into oracle/_ref/ (test infrastructure only).

The reference (fengshi96/EnergySpinCurrents) builds with CMake against Eigen3 and macOS
Accelerate, none of which exist here.  This recipe does not run that build system.  It compiles
the reference's unmodified files where they lie (main.cpp and src/*.h under the reference tree)
with g++, substituting
  * oracle/ref/shim/          -- this project's own minimal Eigen-API header, and
  * oracle/ref/lapack_bridge.cpp -- zheev_/dstev_ forwarded to the LP64 OpenBLAS bundled in scipy.
Outputs (git-ignored): oracle/_ref/LanczosCond (the reference main, unmodified) and
oracle/_ref/golden_driver (our driver around the reference's classes, for full-precision dumps).
"""
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(REPO, "oracle", "_ref")
# The reference source tree: ESC_REFERENCE_DIR, else the read-only mount of the build container
# (absent on GPU hosts, which use the prebuilt outputs and never call this recipe).
DEFAULT_REFERENCE_DIR = "/root/reference"


def reference_dir():
    """Directory holding the reference's main.cpp and src/, or None when it is not present."""
    d = os.environ.get("ESC_REFERENCE_DIR") or DEFAULT_REFERENCE_DIR
    return d if os.path.isdir(os.path.join(d, "src")) else None


def _openblas():
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs", "libscipy_openblas-*.so"))
    if not libs:
        raise RuntimeError("scipy's bundled OpenBLAS (LP64) not found")
    return libs[0]


def build(force=False):
    REF = reference_dir()
    if REF is None:
        raise RuntimeError("reference source tree not present: set ESC_REFERENCE_DIR to the directory holding "
                           "the reference's main.cpp and src/")
    os.makedirs(OUT, exist_ok=True)
    blas = _openblas()
    common = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-w", "-I", os.path.join(HERE, "shim"),
              "-I", os.path.join(REF, "src")]
    link = [os.path.join(HERE, "lapack_bridge.cpp"), blas, "-Wl,-rpath," + os.path.dirname(blas)]
    targets = {
        "LanczosCond": os.path.join(REF, "main.cpp"),
        "golden_driver": os.path.join(HERE, "golden_driver.cpp"),
    }
    deps = glob.glob(os.path.join(HERE, "shim", "**", "*"), recursive=True) + [os.path.join(HERE, "lapack_bridge.cpp"),
                                                                              os.path.abspath(__file__)]
    for name, src in targets.items():
        exe = os.path.join(OUT, name)
        if os.path.exists(exe) and not force and all(
                os.path.getmtime(exe) >= os.path.getmtime(d) for d in [src] + deps if os.path.isfile(d)):
            continue
        subprocess.run(common + ["-o", exe, src] + link, check=True)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
