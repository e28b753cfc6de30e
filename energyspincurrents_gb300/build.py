"""Build the GB300 library and the drop-in executable in-tree.

    python -m energyspincurrents_gb300.build            # libesc.so + LanczosCond

Outputs (git-ignored) in energyspincurrents_gb300/_build/:
    libesc.so      C-ABI library (include/esc.h), sm_103a kernels
    LanczosCond    drop-in replacement of the reference executable (reads the same input file)

Only nvcc and the host g++ are used (no cmake); translation units compile in parallel.  Flags
are portable across the x86_64 build container and the aarch64 GPU hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libesc.so")
EXE = os.path.join(OUT, "LanczosCond")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["kernels.cu", "hv_tiled.cu", "batched.cu", "hv_jit.cu", "permute.cu", "alu_bench.cu"]
CPP_SOURCES = ["esc_abi.cpp", "lanczos.cpp", "spectra.cpp", "grad.cpp", "tune.cpp", "params.cpp", "model.cpp", "numerics.cpp",
               "planner.cpp", "exactdiag.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _cuda_home(nvcc):
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(REPO, "include", "esc.h")]


def _embed_device_source():
    """_build/hv_pass_device.inc: hv_pass_device.cuh as a C++ raw string (the source that the
    run-time specialisation hands to NVRTC)."""
    src = os.path.join(CSRC, "hv_pass_device.cuh")
    dst = os.path.join(OUT, "hv_pass_device.inc")
    with open(src) as f:
        body = f.read()
    if ')ESCSRC"' in body:
        raise RuntimeError("hv_pass_device.cuh contains the raw-string delimiter")
    text = 'R"ESCSRC(' + body + ')ESCSRC"\n'
    if not os.path.exists(dst) or open(dst).read() != text:
        with open(dst, "w") as f:
            f.write(text)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    cuda = _cuda_home(nvcc)
    _embed_device_source()
    inc = ["-I", CSRC, "-I", OUT, "-I", os.path.join(REPO, "include"), "-I", os.path.join(cuda, "include")]
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES + CPP_SOURCES:
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        if not force and not _newer(obj, [path] + hdrs):
            continue
        if src.endswith(".cu"):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                   *inc, "-c", path, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-fopenmp", *inc, "-c", path, "-o", obj]
        jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)
        return cmd

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or not os.path.exists(LIB):
        run([nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-Xcompiler", "-fopenmp", "-lgomp",
             "-L", os.path.join(cuda, "lib64"), "-lnvrtc", "-ldl", "-Xlinker", "-rpath", "-Xlinker", os.path.join(cuda, "lib64")])
        os.replace(LIB + ".tmp", LIB)
    exe_src = os.path.join(CSRC, "LanczosCond.cpp")
    if os.path.exists(exe_src) and (force or _newer(EXE, [exe_src, LIB] + hdrs)):
        run(["g++", "-O2", "-std=c++17", *inc, "-o", EXE, exe_src, "-L", OUT, "-lesc",
             "-Wl,-rpath,$ORIGIN", "-L", os.path.join(cuda, "lib64"), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
