"""Benchmark: H.v throughput (GB/s of algorithmic bytes) on the N=32 Kitaev-Heisenberg honeycomb.

Workload (the configuration the headline metric is quoted on): 4x4 unit cells (Lx=4, Ly=8),
N=32 sites, 2^32 states, K=-1, J=0.05, h=0.02 along [111], complex64 vectors (mixed precision:
FP32 arithmetic on complex64 storage, FP64 reductions).  One step = one H.v over the full 2^32
basis (34.4 GB in, 34.4 GB out) with the inputs resident in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--sites 32]

Prints ONE JSON line (rank 0).  Fields beyond the contract: roofline (dominant kernel vs the
measured HBM copy peak), cpu_baseline (the CPU oracle's matrix-free H.v on a bounded row-slab of
the same operator, all host threads), e2e (the same step through esc_hv with host buffers:
host->device copy, H.v, device->host copy inside the timed region), clocks.
"""
import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

S3 = 3 ** 0.5
METRIC = "H·v GB/s and time-to-S(ω) at N=32: batched mixed vs FP64 GPU at ≤1e-6 error"


def workload(sites):
    shapes = {32: (4, 8), 30: (5, 6), 28: (7, 4), 24: (3, 8), 20: (5, 4), 18: (3, 6), 16: (4, 4), 12: (3, 4)}
    Lx, Ly = shapes[sites]
    hf, J = 0.02, 0.05
    b = -hf / S3
    return dict(Lx=Lx, Ly=Ly, Kxx=-1.0, Kyy=-1.0, Kzz=-1.0, Bxx=b, Byy=b, Bzz=b, jheis=J, seed=1)


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile():
    """DRAM bytes per H.v launch from the committed ncu summary, or None."""
    p = os.path.join(REPO, "profiles", "hv_traffic.json")
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


class Clocks:
    """Samples nvidia-smi during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 9 for i in range(4) if s[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(params, sites, target_s=12.0, kind="port"):
    """The oracle's matrix-free H.v (OpenMP, all host threads) on rows [0, R) of the same operator.

    The input vector is a lazily-zeroed 2^N complex64 array in which only the index ranges that
    rows [0, R) read (k ^ mask for every term mask) are filled with data."""
    import numpy as np
    import oracle as O
    m = O.Model("Kitaev", params["Lx"], params["Ly"], 1, 1, params["Kxx"], params["Kyy"], params["Kzz"],
                params["Bxx"], params["Byy"], params["Bzz"], params["jheis"], os.cpu_count(), False)
    D = m.D
    rbits = min(sites, 24)
    R = 1 << rbits
    v = np.zeros(D, dtype=np.complex64)
    masks = {0}
    nb = O.lattice("Kitaev", params["Lx"], params["Ly"])
    for i in range(m.N):
        masks.add(1 << i)
        for j in nb[i]:
            masks.add((1 << i) | (1 << int(j)))
    rng = np.random.default_rng(0)
    fill = (rng.standard_normal(R) + 1j * rng.standard_normal(R)).astype(np.complex64)
    for hi in sorted({mk & ~(R - 1) for mk in masks}):
        v[hi:hi + R] = fill
    threads = os.cpu_count()
    m.hv_rows(v, 0, R, threads, c64=True)         # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        m.hv_rows(v, 0, R, threads, c64=True)
        reps += 1
        el = time.perf_counter() - t0
        if el > target_s or reps >= 200:
            break
    gbs = reps * R * 16 / el / 1e9
    return {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": kind,
            "sample": f"rows [0, 2^{rbits}) of the N={sites} H.v, {reps} passes in {el:.1f} s, complex64, "
                      f"oracle matrix-free gather (oracle/esc_oracle.cpp hv_matfree)"}


def workload_config(sites, world, dtype="c64"):
    """The `config` both arms report for the --sites workload."""
    params = workload(sites)
    D = 1 << sites
    cname = "complex128" if dtype == "c128" else "complex64"
    return {"workload": f"Kitaev-Heisenberg honeycomb N={sites} ({params['Lx']}x{params['Ly']//2} "
                        f"unit cells, PBC), K=-1 J=0.05 h=0.02[111], one H.v per step ({cname})",
            "states": D, "l2": "inputs larger than L2 (no flush needed)" if D * 8 > 129e6 else "inputs smaller than L2",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def run_reference(args, rank):
    if rank != 0:
        return
    params = workload(args.sites)
    cb = cpu_baseline(params, args.sites, target_s=max(3.0, 2.0 * args.steps))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": workload_config(args.sites, args.gpus),
            "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_to_spectrum(esc, sites=24, gs_steps=300, cf_steps=1000):
    """time-to-S(omega) on the JeJe channels (CF mode, 2000 omega in [0,6], eta=0.05), from one FP64
    ground state: mixed batched (complex64 CF vectors after the default complex128 head of 24 steps, the
    channels as columns of one batched CUDA-graph recurrence) against plain FP64 (complex128, same
    path).  1000 CF steps: the continued fraction is converged there (two FP64 runs that differ
    only in rounding agree to ~1e-11), so the mixed-vs-FP64 difference measures precision, not the
    rounding sensitivity of a half-converged fraction.  The ground state is computed first and is
    not timed."""
    import numpy as np
    params = workload(sites)
    P = esc.ConstVariables(**params, omega_steps=1999, domega=6.0 / 1999, eta=0.05)
    out = {"sites": sites, "kind": "JeJe, continued fraction", "gs_steps": gs_steps, "cf_steps": cf_steps,
           "omega": "2000 points in [0,6]", "eta": 0.05, "fp64_head": 24}
    h = esc.Handle(P)
    h.autotune()      # complex64 passes for this Hamiltonian (untimed; before the ground state by design)
    h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, want_gs=False)
    res = {}
    for name, dt in (("mixed", np.complex64), ("fp64", np.complex128)):
        torch_sync()
        t0 = time.perf_counter()
        S = h.spectrum("Energy Current", "CF", cf_steps=cf_steps, dtype=dt)
        res[name] = (time.perf_counter() - t0, S)
    h.close()
    out["mixed_batched_s"] = round(res["mixed"][0], 3)
    out["fp64_s"] = round(res["fp64"][0], 3)
    out["speedup"] = round(res["fp64"][0] / res["mixed"][0], 2)
    out["max_abs_dS"] = float(np.abs(res["mixed"][1][:, 1:] - res["fp64"][1][:, 1:]).max())
    out["max_abs_S"] = float(np.abs(res["fp64"][1][:, 1:]).max())
    return out


def ground_state_report(esc, sites, steps=200):
    """Mixed-precision ground state of the workload: Lanczos on complex64 vectors without stored basis
    (three vectors; the ground state is rebuilt in a second sweep from the recorded alpha/beta), then
    the FP64 Rayleigh quotient of the complex64 ground state."""
    import numpy as np
    h = esc.Handle(workload(sites))
    t0 = time.perf_counter()
    tune = h.autotune().strip().splitlines()[-1]
    t1 = time.perf_counter()
    r = h.lanczos_gs(steps=steps, lanctype="GS", reortho=0, dtype=np.complex64, want_gs=False)
    t2 = time.perf_counter()
    e_ray = h.rayleigh()
    t3 = time.perf_counter()
    h.close()
    return {"sites": sites, "states": 2 ** sites, "lanczos_steps": r["steps"], "E0_lanczos": r["E0"],
            "E0_rayleigh_fp64": e_ray, "E0_per_site": e_ray / sites, "beta_last": float(r["beta"][-1]),
            "lanczos_s": round(t2 - t1, 2), "rayleigh_s": round(t3 - t2, 2), "autotune_s": round(t1 - t0, 1),
            "tuning": tune, "vectors": "complex64, 3 resident + ground state"}


def lanczos_step_report(esc, sites, steps=48, autotune=True):
    """Cost of one ground-state Lanczos step (complex64, no reorthogonalisation: the H.v passes with
    alpha from the last pass's epilogue, then one update sweep fused with |u|^2) against one H.v,
    both on the self-tuned passes (autotune=False: the configuration esc_create applied, e.g. from
    ESC_TUNE_FILE).  The run is LancType=OnlyEgs, so nothing else is timed."""
    import numpy as np
    import torch
    h = esc.Handle(workload(sites))
    tune = h.autotune().strip().splitlines()[-1] if autotune else os.environ.get("ESC_TUNE_FILE")
    D = h.D
    v = torch.empty(D, dtype=torch.complex64, device="cuda")
    out = torch.empty_like(v)
    flags = esc.DEVICE_PTR | esc.ASYNC | esc.INTERNAL_ORDER
    esc.lib().esc_start_vector(h.h, 1, 1, esc.ctypes.c_void_p(v.data_ptr()), esc.C64, flags)
    stream = torch.cuda.ExternalStream(h.stream())
    for _ in range(2):
        h.hv_device(v.data_ptr(), out.data_ptr(), esc.C64, flags)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(5):
        h.hv_device(v.data_ptr(), out.data_ptr(), esc.C64, flags)
    ev1.record(stream)
    torch.cuda.synchronize()
    hv_ms = ev0.elapsed_time(ev1) / 5
    del v, out
    torch.cuda.empty_cache()
    # warm-up run: allocates the recurrence vectors and the scalars once
    short = steps // 3
    h.lanczos_gs(steps=short, lanctype="OnlyEgs", reortho=0, dtype=np.complex64, want_gs=False)
    t = []
    for n in (short, steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h.lanczos_gs(steps=n, lanctype="OnlyEgs", reortho=0, dtype=np.complex64, want_gs=False)
        t.append(time.perf_counter() - t0)
    step_ms = (t[1] - t[0]) / (steps - short) * 1e3     # set-up and start vector cancel
    h.close()
    return {"sites": sites, "hv_ms": round(hv_ms, 3), "lanczos_step_ms": round(step_ms, 3),
            "step_over_hv": round(step_ms / hv_ms, 3), "tuning": tune}


def refine_report(esc, sites, gs_steps=300, refine_steps=20):
    """FP64 residual refinement of a complex64 ground state: |H psi - E psi| (FP64) before and after
    refinement steps, the energies, and the times."""
    import numpy as np
    h = esc.Handle(workload(sites))
    h.autotune()
    t0 = time.perf_counter()
    r = h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, dtype=np.complex64, want_gs=False)
    t1 = time.perf_counter()
    e_ray = h.rayleigh()
    t2 = time.perf_counter()
    E, rn = h.refine_gs(refine_steps)
    t3 = time.perf_counter()
    h.close()
    return {"sites": sites, "gs_steps": gs_steps, "E0_lanczos_c64": r["E0"], "E0_rayleigh_fp64": e_ray,
            "E0_refined": E, "refine_steps": refine_steps, "residual": [float(x) for x in rn],
            "lanczos_s": round(t1 - t0, 2), "rayleigh_s": round(t2 - t1, 2), "refine_s": round(t3 - t2, 2)}


def c3_report(esc, gs_steps=300, cf_steps=1000, refine28=40, refine32=10):
    """Mixed precision against FP64 for the 32-site workload (K=-1, J=0.05, h=0.02 [111], seed 1):
    on the 28-site cluster (7x2 unit cells) both run -- FP64 ground state and FP64 continued
    fractions against the complex64 ground state (FP64 Rayleigh value, FP64 refinement) and complex64
    continued fractions -- and the E0 and S(omega) differences are reported; on the 32-site cluster
    FP64 does not fit (a complex128 vector is 68.7 GB), and the mixed E0, the FP64 residual of the
    refined ground state and the spectrum are reported.  JeJe spectra, 2000 omega in [0, 6],
    eta = 0.05."""
    import numpy as np
    out = {"cf_steps": cf_steps, "gs_steps": gs_steps, "omega": "2000 points in [0,6]", "eta": 0.05,
           "refine_steps": {"n28": refine28, "n32": refine32}}
    kw = dict(omega_steps=1999, domega=6.0 / 1999, eta=0.05)
    # 28 sites, FP64
    h = esc.Handle(esc.ConstVariables(**workload(28), **kw))
    h.autotune()
    t0 = time.perf_counter()
    r64 = h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, want_gs=False)
    t1 = time.perf_counter()
    S64 = h.spectrum("Energy Current", "CF", cf_steps=cf_steps)
    t2 = time.perf_counter()
    h.close()
    # 28 sites, mixed
    h = esc.Handle(esc.ConstVariables(**workload(28), **kw))
    h.autotune()
    t3 = time.perf_counter()
    r32 = h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, dtype=np.complex64, want_gs=False)
    e_ray = h.rayleigh()
    E_ref, rn = h.refine_gs(refine28)
    t4 = time.perf_counter()
    S32 = h.spectrum("Energy Current", "CF", cf_steps=cf_steps, dtype=np.complex64)
    t5 = time.perf_counter()
    h.close()
    e64 = r64["E0"]
    out["n28"] = {"E0_fp64": e64, "E0_c64_lanczos": r32["E0"], "E0_c64_rayleigh_fp64": e_ray, "E0_refined": E_ref,
                  "relerr_E0_c64_lanczos": abs(r32["E0"] - e64) / abs(e64),
                  "relerr_E0_rayleigh": abs(e_ray - e64) / abs(e64), "relerr_E0_refined": abs(E_ref - e64) / abs(e64),
                  "refine_residual": [float(rn[0]), float(rn[-1])],
                  "max_abs_dS": float(np.abs(S32[:, 1:] - S64[:, 1:]).max()), "max_abs_S": float(np.abs(S64[:, 1:]).max()),
                  "fp64_gs_s": round(t1 - t0, 1), "fp64_S_s": round(t2 - t1, 1), "mixed_gs_s": round(t4 - t3, 1),
                  "mixed_S_s": round(t5 - t4, 1)}
    # 32 sites, mixed only
    h = esc.Handle(esc.ConstVariables(**workload(32), **kw))
    h.autotune()
    t6 = time.perf_counter()
    r = h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, dtype=np.complex64, want_gs=False)
    e_ray = h.rayleigh()
    E_ref, rn = h.refine_gs(refine32)
    t7 = time.perf_counter()
    S = h.spectrum("Energy Current", "CF", cf_steps=cf_steps // 2, dtype=np.complex64)
    t8 = time.perf_counter()
    h.close()
    out["n32"] = {"E0_c64_lanczos": r["E0"], "E0_c64_rayleigh_fp64": e_ray, "E0_refined": E_ref,
                  "E0_per_site": E_ref / 32, "refine_residual": [float(rn[0]), float(rn[-1])],
                  "cf_steps": cf_steps // 2, "max_abs_S": float(np.abs(S[:, 1:]).max()),
                  "omega_at_max_tt": float(S[np.abs(S[:, 5]).argmax(), 0]),
                  "gs_and_refine_s": round(t7 - t6, 1), "time_to_S_s": round(t8 - t7, 1)}
    return out


def e2e_report(esc, sites=32, reps=3):
    """The legs of the pipelined host-buffer H.v (esc_hv_batched, 2 complex64 columns in reference
    order) timed alone: host->device copy of one vector, device->host copy, both at once on two
    streams, the device work of one column (basis permutation in, H.v, permutation out), and the
    whole pipelined call.  Pinned host buffers; wall-clock after a warm-up, best of `reps`."""
    import numpy as np
    import torch
    h = esc.Handle(workload(sites))
    tune = h.autotune().strip().splitlines()[-1]
    D = h.D
    hin = torch.empty((2, D), dtype=torch.complex64, pin_memory=True)
    hout = torch.empty((2, D), dtype=torch.complex64, pin_memory=True)
    hin.zero_()
    out = {"sites": sites, "vector_GB": D * 8 / 1e9, "tuning": tune}

    def best(f):
        f()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            f()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts) * 1e3

    d0 = torch.empty(D, dtype=torch.complex64, device="cuda")
    d1 = torch.empty(D, dtype=torch.complex64, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    out["h2d_ms"] = best(lambda: d0.copy_(hin[0], non_blocking=True))
    out["d2h_ms"] = best(lambda: hout[0].copy_(d0, non_blocking=True))

    def both():
        with torch.cuda.stream(s1):
            d0.copy_(hin[0], non_blocking=True)
        with torch.cuda.stream(s2):
            hout[1].copy_(d1, non_blocking=True)
    out["h2d_and_d2h_ms"] = best(both)
    out["device_column_ms"] = best(lambda: h.hv_device(d0.data_ptr(), d1.data_ptr(), esc.C64, esc.DEVICE_PTR))
    del d0, d1
    torch.cuda.empty_cache()
    out["pipelined_2col_ms"] = best(lambda: h.hv_batched(hin.numpy(), out=hout.numpy()))
    vb = D * 8 / 1e9
    out["link_bound_2col_ms"] = round(max(2 * out["h2d_ms"], 2 * out["d2h_ms"], out["h2d_and_d2h_ms"] + out["h2d_ms"]), 1)
    out["e2e_GBs"] = round(2 * 2 * vb / (out["pipelined_2col_ms"] * 1e-3), 1)
    h.close()
    return {k: (round(v, 2) if isinstance(v, float) else v) for k, v in out.items()}


def reduce_max(x, dist, device):
    """Max over the ranks of a per-rank time (the slowest replica sets the job's time)."""
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_gbs(bytes_per_replica, world, ms):
    """Whole-job throughput of `world` independent replicas that each move bytes_per_replica in
    (at most) ms milliseconds: replicas only, no exchange between them."""
    return world * bytes_per_replica / (ms * 1e-3) / 1e9


def mixed_spectrum_report(esc, sites, gs_steps=200, cf_steps=500):
    """JeJe CF spectrum (2000 omega in [0,6], eta=0.05) of the workload entirely in complex64: the
    ground state of a complex64 Lanczos run (three vectors) and complex64 continued fractions (the
    complex128 head is skipped when its vectors do not fit, as at 32 sites)."""
    import numpy as np
    P = esc.ConstVariables(**workload(sites), omega_steps=1999, domega=6.0 / 1999, eta=0.05)
    h = esc.Handle(P)
    tune = h.autotune().strip().splitlines()[-1]
    t0 = time.perf_counter()
    r = h.lanczos_gs(steps=gs_steps, lanctype="GS", reortho=0, dtype=np.complex64, want_gs=False)
    t1 = time.perf_counter()
    S = h.spectrum("Energy Current", "CF", cf_steps=cf_steps)
    t2 = time.perf_counter()
    h.close()
    return {"sites": sites, "kind": "JeJe, continued fraction, complex64", "gs_steps": gs_steps, "cf_steps": cf_steps,
            "E0": r["E0"], "gs_s": round(t1 - t0, 2), "time_to_S_s": round(t2 - t1, 2),
            "max_abs_S": float(np.abs(S[:, 1:]).max()), "omega_at_max_tt": float(S[np.abs(S[:, 5]).argmax(), 0]),
            "tuning": tune}


def torch_sync():
    import torch
    torch.cuda.synchronize()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sites", type=int, default=32)
    ap.add_argument("--dtype", default="c64", choices=["c64", "c128"],
                    help="c128: the step is the plain FP64 H.v (complex128 vectors; no self-tuner, e2e or spectrum legs)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-spectrum", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="skip the self-tuner (library default plan)")
    ap.add_argument("--tts-report", action="store_true",
                    help="time-to-S(omega) of the --sites cluster in mixed precision only (complex64 ground state and "
                         "continued fractions; for clusters whose FP64 vectors do not fit) and print one JSON line")
    ap.add_argument("--gs-report", action="store_true",
                    help="time a mixed-precision ground state of the --sites cluster (Lanczos on complex64 vectors, "
                         "FP64 Rayleigh refinement) and print one JSON line, then exit")
    ap.add_argument("--alu-report", action="store_true",
                    help="measure the FP32 / packed FP32 / FP64 FMA ceilings of the GPU (clocks sampled) and print one JSON line")
    ap.add_argument("--refine-report", action="store_true",
                    help="FP64 residual refinement of a complex64 ground state of --sites; print one JSON line")
    ap.add_argument("--c3-report", action="store_true",
                    help="mixed precision against FP64 at 28 sites and the mixed 32-site run; print one JSON line")
    ap.add_argument("--e2e-report", action="store_true",
                    help="time the legs of the pipelined host-buffer H.v of --sites alone; print one JSON line")
    ap.add_argument("--step-report", action="store_true",
                    help="time one complex64 Lanczos step of the --sites cluster against one H.v and print one JSON line")
    ap.add_argument("--autotune-report", action="store_true",
                    help="print the self-tuner's timing of every H.v variant for --sites and exit (no JSON line)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch
    import energyspincurrents_gb300 as esc
    from energyspincurrents_gb300 import build
    build.build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.autotune_report:
        print(esc.Handle(workload(args.sites)).autotune(), end="")
        return
    if args.gs_report:
        print(json.dumps(ground_state_report(esc, args.sites)), flush=True)
        return
    if args.alu_report:
        with Clocks(local) as clk:
            r = esc.alu_peaks()
        r["clocks"] = clk.summary()
        mhz = r["clocks"].get("sm_mhz")
        if mhz:   # per SM and clock: flops / (SMs x cycles)
            sms = torch.cuda.get_device_properties(local).multi_processor_count
            for k in ("ffma", "ffma2", "dfma"):
                r[k + "_flops_per_sm_clock"] = round(r[k + "_tflops"] * 1e12 / (sms * mhz * 1e6), 2)
        print(json.dumps(r), flush=True)
        return
    if args.step_report:
        print(json.dumps(lanczos_step_report(esc, args.sites, autotune=not args.no_autotune)), flush=True)
        return
    if args.e2e_report:
        print(json.dumps(e2e_report(esc, args.sites)), flush=True)
        return
    if args.refine_report:
        print(json.dumps(refine_report(esc, args.sites)), flush=True)
        return
    if args.c3_report:
        print(json.dumps(c3_report(esc)), flush=True)
        return
    if args.tts_report:
        print(json.dumps(mixed_spectrum_report(esc, args.sites)), flush=True)
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    params = workload(args.sites)
    h = esc.Handle(params)
    D = h.D
    c128 = args.dtype == "c128"
    if c128:
        args.no_autotune = args.no_e2e = args.no_spectrum = True
    tuning = None
    if not args.no_autotune:
        # the library's self-tuner: per-pass choice of kernel variant for this Hamiltonian (untimed)
        tuning = h.autotune().strip().splitlines()[-1]
    stream = torch.cuda.ExternalStream(h.stream())
    edt = esc.C128 if c128 else esc.C64
    v = torch.empty(D, dtype=torch.complex128 if c128 else torch.complex64, device="cuda")
    out = torch.empty_like(v)
    # vectors stay resident in the library's internal basis order (a fixed relabelling of the sites;
    # inner products and spectra do not depend on it), so a step is exactly the H.v kernels
    flags = esc.DEVICE_PTR | esc.ASYNC | esc.INTERNAL_ORDER
    st = esc.lib().esc_start_vector(h.h, 1, 1, esc.ctypes.c_void_p(v.data_ptr()), edt, flags)
    assert st == 0, esc.lib().esc_last_error(h.h)
    npasses = esc.plan(esc.ConstVariables(**params))[1]
    npairs = 0
    if tuning:
        chosen = tuning.split("passes:")[1]
        npasses = len(re.findall(r"\b(?:jit|aot)/\d+/\d+", chosen))
        m = re.search(r"slab pairs (\d+)", chosen)
        npairs = int(m.group(1)) if m else 0
    torch.cuda.synchronize()

    def step():
        h.hv_device(v.data_ptr(), out.data_ptr(), edt, flags)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist:
        ms = reduce_max(ms, dist, "cuda")
    algo_bytes = D * (32 if c128 else 16)            # read v + write out
    gbs_total = replicas_gbs(algo_bytes, world, ms)
    kernel_gbs = algo_bytes / (ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    prof = traffic_from_profile() or {}
    traffic, tsrc = None, None
    meas = prof.get("measured_bytes_per_hv", {})
    if c128:
        pass   # the committed traffic figures are for the complex64 passes
    elif str(args.sites) in meas:
        traffic, tsrc = int(meas[str(args.sites)]), prof.get("source")
    elif prof.get("first_pass_bytes_per_state"):
        # per-pass DRAM bytes per state measured on a smaller cluster, scaled by the states and
        # passes of this one (pass 1 reads v and the bond diagonal, later passes v and the partial)
        traffic = int(D * (prof["first_pass_bytes_per_state"] + (npasses - 1) * prof["later_pass_bytes_per_state"]))
        tsrc = prof.get("source") + f", scaled to 2^{args.sites} states and {npasses} passes"
    roof = {"bound": "hbm", "achieved": round(kernel_gbs, 1), "peak": peak, "unit": "GB/s",
            "frac": round(kernel_gbs / peak, 4), "peak_source": peak_kind, "traffic": traffic,
            "kernel": ("complex128 tiled H.v passes (k_hv_pass_fast<double>)" if c128 else
                       "complex64 tiled H.v passes (esc_jit_pass*, k_hv_pass_f32g; per-pass choice of the self-tuner)"),
            "passes": npasses,
            "algorithmic_bytes_per_launch": algo_bytes, "traffic_source": tsrc}
    del v, out
    torch.cuda.empty_cache()

    # end to end through the C ABI: host buffers (pinned) in the reference basis order; the host->
    # device copy, the basis permutations, H.v and the device->host copy are inside the timed region
    # A step is a batch of 2 vectors through esc_hv_batched when the host has room for 4 pinned
    # vectors: the library then overlaps one vector's copy in, the other's H.v and copy out (the
    # host link is full duplex); otherwise 1 vector through esc_hv.
    e2e = None
    if not args.no_e2e:
        try:
            # every rank pins its own host buffers: size them so that all ranks fit in host memory
            avail = os.sysconf("SC_AVPHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
            ncols = 2 if avail > world * 4 * D * 8 + (24 << 30) else 1
            if avail < world * 2 * D * 8 + (24 << 30):
                raise MemoryError(f"host memory for {world} replicas' pinned vectors: {avail >> 30} GiB available")
            hin = torch.empty((ncols, D), dtype=torch.complex64, pin_memory=True)
            hout = torch.empty((ncols, D), dtype=torch.complex64, pin_memory=True)
            hin.zero_()
            if ncols == 1:
                call = lambda: h.hv(hin[0].numpy(), out=hout[0].numpy())
            else:
                call = lambda: h.hv_batched(hin.numpy(), out=hout.numpy())
            call()   # warm-up (allocates the staging buffers)
            reps = max(1, min(args.steps, 3))
            t0 = time.perf_counter()
            for _ in range(reps):
                call()
            el = (time.perf_counter() - t0) / reps
            e2e = {"value": round(world * ncols * algo_bytes / el / 1e9, 3), "unit": "GB/s",
                   "h2d_bytes_per_step": ncols * D * 8, "d2h_bytes_per_step": ncols * D * 8,
                   "ms_per_step": round(el * 1e3, 3), "vectors_per_step": ncols,
                   "path": ("esc_hv_batched (2 columns, copies overlapped with H.v)" if ncols == 2 else "esc_hv") +
                           ", host pointers, reference basis order"}
            del hin, hout
        except Exception as ex:
            e2e = {"value": None, "unit": "GB/s", "error": str(ex)[:200]}
    h.close()
    torch.cuda.empty_cache()
    tts = None
    if rank == 0 and not args.no_spectrum:
        try:
            tts = time_to_spectrum(esc)
        except Exception as ex:
            tts = {"error": str(ex)[:200]}
    cb = None
    if rank == 0 and not args.no_cpu:
        cb = cpu_baseline(params, args.sites)
    if rank == 0:
        line = {"metric": METRIC, "value": round(gbs_total, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": args.dtype, "data": "synthetic",
                "config": dict(workload_config(args.sites, world, args.dtype), tuning=tuning),
                "roofline": roof, "cpu_baseline": cb, "e2e": e2e, "time_to_S": tts, "clocks": clk.summary(),
                "gpu_launches": args.steps * (npasses - npairs)}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
