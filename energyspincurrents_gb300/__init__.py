"""GB300-native Lanczos exact diagonalisation of the Kitaev(-Heisenberg) honeycomb model.

Python front-end over the C ABI in include/esc.h (libesc.so, hand-written sm_103a kernels).  It
mirrors the reference's C++ classes (fengshi96/EnergySpinCurrents) by name:

    ConstVariables      src/ParametersEngine.h   parameter file -> parameters
    Hamiltonian         src/Hamiltonian.h        MatrixVectorMult(v)
    DynLanczosSolver    src/DynLanczosSolver.h   Lanczos_Nirav(PsiOrAll) -> |gs>, TriDeval
    Observables         src/Observables.h        ApplyOp / ApplySx ... / ApplyJexTotal ...
    StartDynamics       src/dynamics.h           "Energy Current" / "Spin Current" / "LocalSzSz"

Vectors are numpy complex128 (or complex64) arrays in the reference's basis order.  There is no
CPU implementation: without the CUDA library or a CUDA device every call raises.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "_build", "libesc.so")

ESC_OK, ESC_ERR_PARAM, ESC_ERR_MEMORY, ESC_ERR_CUDA, ESC_ERR_NUMERIC, ESC_ERR_STATE, ESC_ERR_TIMEOUT = range(7)
C128, C64 = 0, 1
DEVICE_PTR, ASYNC, INTERNAL_ORDER = 1, 2, 4

OPS = ["I", "Sx", "Sy", "Sz", "Sp", "Sm", "Spe3", "Sme3", "SxSySz", "Jsx", "Jsy", "Jsz", "Jex", "Jey", "JexJeyJez",
       "JsxJsyJsz", "JsxTotal", "JsyTotal", "JszTotal", "JexTotal", "JeyTotal", "JsTotal", "JeTotal"]
OP_ID = {n: i for i, n in enumerate(OPS)}
DYN_KIND = {"Energy Current": 0, "Spin Current": 1, "LocalSzSz": 2}
DYN_FILE = {"Energy Current": "JeJe_outSpectrum.real", "Spin Current": "JsJs_outSpectrum.real",
            "LocalSzSz": "2SSLocal_outSpectrum.real"}


class EscError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [("Lx", ctypes.c_int), ("Ly", ctypes.c_int), ("pbcx", ctypes.c_int), ("pbcy", ctypes.c_int),
                ("seed", ctypes.c_int), ("model", ctypes.c_char * 32), ("solver", ctypes.c_char * 16),
                ("lanctype", ctypes.c_char * 16),
                ("Kxx", ctypes.c_double), ("Kyy", ctypes.c_double), ("Kzz", ctypes.c_double),
                ("Bxx", ctypes.c_double), ("Byy", ctypes.c_double), ("Bzz", ctypes.c_double),
                ("temperature", ctypes.c_double), ("lanczos_eps", ctypes.c_double),
                ("lanczos_steps", ctypes.c_int), ("threads", ctypes.c_int), ("local_skw", ctypes.c_int),
                ("spin_curr_dyn", ctypes.c_int), ("energy_curr_dyn", ctypes.c_int),
                ("jheis", ctypes.c_double), ("omega_steps", ctypes.c_int), ("domega", ctypes.c_double),
                ("eta", ctypes.c_double), ("dyn_mode", ctypes.c_int), ("dyn_lanczos_steps", ctypes.c_int),
                ("precision", ctypes.c_int), ("start_vector", ctypes.c_int), ("local_szsz_dyn", ctypes.c_int),
                ("reortho", ctypes.c_int)]


class LanczosCfg(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("eps", ctypes.c_double), ("lanctype", ctypes.c_int),
                ("reortho", ctypes.c_int), ("dtype", ctypes.c_int)]


class CFBatchCfg(ctypes.Structure):
    _fields_ = [("ncols", ctypes.c_int), ("max_steps", ctypes.c_int), ("steps", ctypes.c_void_p),
                ("fields", ctypes.c_void_p), ("tol", ctypes.c_double), ("dtype", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("fp64_head", ctypes.c_int)]


class DynCfg(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("mode", ctypes.c_int), ("omega_steps", ctypes.c_int),
                ("domega", ctypes.c_double), ("eta", ctypes.c_double), ("cf_steps", ctypes.c_int),
                ("dtype", ctypes.c_int), ("fp64_head", ctypes.c_int)]


_lib = None

# every symbol declared in include/esc.h
EXPORTS = ["esc_params_default", "esc_params_from_file", "esc_lattice", "esc_plan", "esc_create", "esc_destroy", "esc_last_error",
           "esc_num_sites", "esc_dim", "esc_neighbors", "esc_basis_permutation", "esc_stream", "esc_hv", "esc_hv_batched", "esc_apply_op",
           "esc_start_vector", "esc_rayleigh", "esc_rayleigh_noalloc", "esc_refine_gs", "esc_lanczos_gs", "esc_cf_batched", "esc_spectrum", "esc_measure_local", "esc_grad", "esc_autotune", "esc_two_point", "esc_alu_peaks", "esc_exact_diag"]


def lib_path():
    return _LIB_PATH


def lib():
    """Load libesc.so (built by energyspincurrents_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise EscError(ESC_ERR_CUDA, f"CUDA library not built: {_LIB_PATH} missing (run energyspincurrents_gb300.build)")
    L = ctypes.CDLL(_LIB_PATH)
    P, vp, ci, cd, i64 = ctypes.POINTER, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_int64
    L.esc_params_default.argtypes = [P(Params)]
    L.esc_params_from_file.argtypes = [ctypes.c_char_p, P(Params), ctypes.c_char_p, ctypes.c_size_t]
    L.esc_lattice.argtypes = [P(Params), P(ci), P(ci)]
    L.esc_plan.argtypes = [P(Params), ci, ci, P(ci), P(ci)]
    L.esc_create.argtypes = [P(Params), P(vp)]
    L.esc_destroy.argtypes = [vp]
    L.esc_last_error.argtypes = [vp]
    L.esc_last_error.restype = ctypes.c_char_p
    L.esc_num_sites.argtypes = [vp]
    L.esc_dim.argtypes = [vp]
    L.esc_dim.restype = i64
    L.esc_neighbors.argtypes = [vp, P(ci)]
    L.esc_basis_permutation.argtypes = [vp, P(ci)]
    L.esc_stream.argtypes = [vp]
    L.esc_stream.restype = vp
    L.esc_hv.argtypes = [vp, vp, vp, ci, ci]
    L.esc_hv_batched.argtypes = [vp, vp, vp, ci, i64, vp, ci, ci]
    L.esc_apply_op.argtypes = [vp, ci, ci, vp, vp, ci, ci]
    L.esc_start_vector.argtypes = [vp, ci, ci, vp, ci, ci]
    L.esc_rayleigh.argtypes = [vp, vp, ci, ci, P(cd)]
    L.esc_rayleigh_noalloc.argtypes = [P(Params), vp, ci, vp, P(cd)]
    L.esc_refine_gs.argtypes = [vp, ci, P(cd), vp]
    L.esc_lanczos_gs.argtypes = [vp, P(LanczosCfg), vp, ci, P(cd), vp, vp, vp, P(ci), vp]
    L.esc_spectrum.argtypes = [vp, P(DynCfg), vp, P(ci), P(ci)]
    L.esc_cf_batched.argtypes = [vp, P(CFBatchCfg), vp, i64, ci, vp, vp, vp]
    L.esc_measure_local.argtypes = [vp, vp, vp]
    L.esc_grad.argtypes = [vp, P(DynCfg), vp, vp]
    L.esc_autotune.argtypes = [vp, ctypes.c_char_p, ctypes.c_size_t]
    L.esc_two_point.argtypes = [vp, ci, ci, vp]
    L.esc_alu_peaks.argtypes = [vp]
    L.esc_exact_diag.argtypes = [vp, vp, vp, ci]
    _lib = L
    return L


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _dt(a):
    if a.dtype == np.complex64:
        return C64
    if a.dtype == np.complex128:
        return C128
    raise TypeError("vectors must be complex128 or complex64")


# ------------------------------------------------------------------------------------------------
# Parameters (ConstVariables, src/ParametersEngine.h)
# ------------------------------------------------------------------------------------------------
class ConstVariables:
    """Parameters read like the reference's ConstVariables, plus keyword construction."""

    def __init__(self, inputfile=None, **kw):
        self.p = Params()
        L = lib()
        L.esc_params_default(ctypes.byref(self.p))
        if inputfile is not None:
            err = ctypes.create_string_buffer(512)
            st = L.esc_params_from_file(str(inputfile).encode(), ctypes.byref(self.p), err, 512)
            if st != ESC_OK:
                raise ValueError(err.value.decode())
        for k, v in kw.items():
            if k in ("model", "solver", "lanctype"):
                setattr(self.p, k, v.encode())
            else:
                setattr(self.p, k, v)

    def __getattr__(self, k):
        if k == "p":
            raise AttributeError(k)
        v = getattr(self.p, k)
        return v.decode() if isinstance(v, bytes) else v

    @property
    def NumberofSites(self):
        return self.p.Lx * self.p.Ly


def lattice(params):
    """Neighbour table (N x 3, columns z, y, x) computed on the host (no device needed)."""
    if not isinstance(params, ConstVariables):
        params = ConstVariables(**params)
    N = params.p.Lx * params.p.Ly
    out = np.full(max(N, 1) * 3, -1, dtype=np.int32)
    n = ctypes.c_int()
    st = lib().esc_lattice(ctypes.byref(params.p), out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.byref(n))
    if st != ESC_OK:
        raise EscError(st, lib().esc_last_error(None).decode())
    return out[: 3 * n.value].reshape(n.value, 3)


def plan(params, tile_bits=0, low_bits=0):
    """(bit_of_site, npasses) of the tiled H.v plan, computed on the host."""
    if not isinstance(params, ConstVariables):
        params = ConstVariables(**params)
    N = params.p.Lx * params.p.Ly
    perm = np.empty(N, dtype=np.int32)
    n = ctypes.c_int()
    st = lib().esc_plan(ctypes.byref(params.p), tile_bits, low_bits, perm.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                        ctypes.byref(n))
    if st != ESC_OK:
        raise EscError(st, lib().esc_last_error(None).decode())
    return perm, n.value


def _check(h, st):
    if st != ESC_OK:
        raise EscError(st, lib().esc_last_error(h).decode())


class Handle:
    """One esc_handle: model tables, device buffers, its CUDA stream."""

    def __init__(self, params):
        if not isinstance(params, ConstVariables):
            params = ConstVariables(**params)
        self.params = params
        h = ctypes.c_void_p()
        st = lib().esc_create(ctypes.byref(params.p), ctypes.byref(h))
        if st != ESC_OK:
            raise EscError(st, lib().esc_last_error(None).decode())
        self.h = h
        self.N = lib().esc_num_sites(h)
        self.D = lib().esc_dim(h)

    def close(self):
        if getattr(self, "h", None):
            lib().esc_destroy(self.h)
            self.h = None

    __del__ = close

    def stream(self):
        return lib().esc_stream(self.h)

    def neighbors(self):
        out = np.empty(self.N * 3, dtype=np.int32)
        _check(self.h, lib().esc_neighbors(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out.reshape(self.N, 3)

    def basis_permutation(self):
        """bit_of_site[s]: position of site s's bit in the internal basis index."""
        out = np.empty(self.N, dtype=np.int32)
        _check(self.h, lib().esc_basis_permutation(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return out

    def to_internal(self, v):
        """Reference-order vector -> internal order (host-side permutation, for tests)."""
        perm = self.basis_permutation()
        k = np.arange(self.D, dtype=np.int64)
        j = np.zeros_like(k)
        for s in range(self.N):
            j |= ((k >> s) & 1) << int(perm[s])
        out = np.empty_like(v)
        out[j] = v
        return out

    # -- operators ------------------------------------------------------------------------------
    def hv(self, v, out=None, flags=0):
        v = np.ascontiguousarray(v)
        out = np.empty_like(v) if out is None else out
        _check(self.h, lib().esc_hv(self.h, _ptr(v), _ptr(out), _dt(v), flags))
        return out

    def hv_device(self, in_ptr, out_ptr, dtype=C128, flags=DEVICE_PTR):
        _check(self.h, lib().esc_hv(self.h, ctypes.c_void_p(in_ptr), ctypes.c_void_p(out_ptr), dtype, flags))

    def hv_batched(self, V, fields=None, out=None):
        """V: (ncols, D) array; fields: (ncols, 3) Bxx, Byy, Bzz per column."""
        V = np.ascontiguousarray(V)
        out = np.empty_like(V) if out is None else out
        f = None if fields is None else np.ascontiguousarray(fields, dtype=np.float64)
        _check(self.h, lib().esc_hv_batched(self.h, _ptr(V), _ptr(out), V.shape[0], V.shape[1], _ptr(f), _dt(V), 0))
        return out

    def apply(self, op, site, v, out=None):
        v = np.ascontiguousarray(v)
        out = np.empty_like(v) if out is None else out
        oid = OP_ID[op] if isinstance(op, str) else int(op)
        _check(self.h, lib().esc_apply_op(self.h, oid, int(site), _ptr(v), _ptr(out), _dt(v), 0))
        return out

    def start_vector(self, kind="RefUniform", seed=None, dtype=np.complex128):
        out = np.empty(self.D, dtype=dtype)
        k = {"RefUniform": 0, "Normal": 1}[kind]
        seed = self.params.p.seed if seed is None else seed
        _check(self.h, lib().esc_start_vector(self.h, k, int(seed), _ptr(out), _dt(out), 0))
        return out

    # -- solvers --------------------------------------------------------------------------------
    def lanczos_gs(self, steps=None, eps=None, lanctype=None, reortho=None, start=None, dtype=np.complex128,
                   want_gs=True):
        p = self.params.p
        steps = p.lanczos_steps if steps is None else steps
        lt = (lanctype or p.lanctype.decode())
        cfg = LanczosCfg(steps, p.lanczos_eps if eps is None else eps, {"OnlyEgs": 0, "GS": 1, "All": 2}[lt],
                         (p.reortho if reortho is None else int(reortho)), C64 if dtype == np.complex64 else C128)
        a = np.zeros(steps); b = np.zeros(steps + 1); r = np.zeros(steps)
        n = ctypes.c_int(); E0 = ctypes.c_double()
        gs = np.empty(self.D, dtype=dtype) if want_gs else None
        st = None
        if start is not None:
            st = np.ascontiguousarray(start, dtype=dtype)
        _check(self.h, lib().esc_lanczos_gs(self.h, ctypes.byref(cfg), _ptr(st) if st is not None else None, 0,
                                            ctypes.byref(E0), _ptr(a), _ptr(b), _ptr(r), ctypes.byref(n), _ptr(gs)))
        n = n.value
        return dict(E0=E0.value, alpha=a[:n], beta=b[: n + 1], ritz=r[:n], steps=n, gs=gs)

    def rayleigh(self, v=None, flags=0):
        """<v|H|v>/<v|v> in FP64 arithmetic (v complex128 or complex64; None: the handle's ground
        state, in place)."""
        E = ctypes.c_double()
        if v is None:
            _check(self.h, lib().esc_rayleigh(self.h, None, C128, 0, ctypes.byref(E)))
            return E.value
        v = np.ascontiguousarray(v)
        _check(self.h, lib().esc_rayleigh(self.h, _ptr(v), _dt(v), flags, ctypes.byref(E)))
        return E.value

    def exact_diag(self):
        """Solver=ED: all eigenvalues (ascending) and the ground state; the eigenpairs replace the
        Ritz pairs for the Ritz-mode spectra."""
        ev = np.empty(self.D)
        gs = np.empty(self.D, dtype=np.complex128)
        _check(self.h, lib().esc_exact_diag(self.h, _ptr(ev), _ptr(gs), 0))
        return ev, gs

    def refine_gs(self, steps=4):
        """FP64 residual refinement of the ground state; returns (E, |H psi - E psi| before each
        step and after the last)."""
        E = ctypes.c_double()
        rn = np.zeros(steps + 1)
        _check(self.h, lib().esc_refine_gs(self.h, int(steps), ctypes.byref(E), _ptr(rn)))
        return E.value, rn

    def cf_batched(self, starts, max_steps, steps=None, fields=None, tol=1e-10, use_graph=True, flags=0, fp64_head=0):
        """Batched continued-fraction Lanczos; starts (ncols, D).  Returns [(a, b)] per column.
        fp64_head (complex64 starts only): leading steps run on complex128 copies of the columns."""
        V = np.ascontiguousarray(starts)
        nc = V.shape[0]
        st = None if steps is None else np.ascontiguousarray(steps, dtype=np.int32)
        fl = None if fields is None else np.ascontiguousarray(fields, dtype=np.float64)
        cfg = CFBatchCfg(nc, max_steps, _ptr(st).value if st is not None else None,
                         _ptr(fl).value if fl is not None else None, tol, _dt(V), 1 if use_graph else 0, int(fp64_head))
        a = np.zeros((nc, max_steps)); b = np.zeros((nc, max_steps + 1)); lens = np.zeros(nc, dtype=np.int32)
        _check(self.h, lib().esc_cf_batched(self.h, ctypes.byref(cfg), _ptr(V), V.shape[1], flags, _ptr(a), _ptr(b),
                                            _ptr(lens)))
        return [(a[c, : lens[c]], b[c, : lens[c] + 1]) for c in range(nc)]

    def two_point(self, opA, opB):
        """Observables::TwoPointCorr: N x N matrix <gs| A_si B_sj |gs> (si >= sj, mirrored)."""
        out = np.empty((self.N, self.N), dtype=np.complex128)
        _check(self.h, lib().esc_two_point(self.h, OP_ID[opA], OP_ID[opB], _ptr(out)))
        return out

    def autotune(self):
        """Times the complex64 H.v variants for this Hamiltonian and keeps the fastest; returns the
        report (one line per candidate, then the choice)."""
        buf = ctypes.create_string_buffer(32768)
        _check(self.h, lib().esc_autotune(self.h, buf, len(buf)))
        return buf.value.decode()

    def spectrum(self, kind, mode="Ritz", omega_steps=None, domega=None, eta=None, cf_steps=0, dtype=None,
                 fp64_head=0):
        """Rows of the reference's output file.  CF mode runs in complex64 when the ground state is
        complex64 or dtype is np.complex64; fp64_head: leading CF steps of a complex64 run done in
        complex128 (0: library default, < 0: none)."""
        p = self.params.p
        dt = C64 if dtype is not None and np.dtype(dtype) == np.complex64 else C128
        cfg = DynCfg(DYN_KIND[kind], {"Ritz": 0, "CF": 1}[mode], p.omega_steps if omega_steps is None else omega_steps,
                     p.domega if domega is None else domega, p.eta if eta is None else eta, cf_steps, dt, fp64_head)
        nr = ctypes.c_int(); nc = ctypes.c_int()
        _check(self.h, lib().esc_spectrum(self.h, ctypes.byref(cfg), None, ctypes.byref(nr), ctypes.byref(nc)))
        out = np.empty(nr.value * nc.value)
        _check(self.h, lib().esc_spectrum(self.h, ctypes.byref(cfg), _ptr(out), ctypes.byref(nr), ctypes.byref(nc)))
        return out.reshape(nr.value, nc.value)

    def measure_local(self):
        s = np.empty((self.N, 3), dtype=np.complex128)
        je = np.empty((self.N, 2), dtype=np.complex128)
        _check(self.h, lib().esc_measure_local(self.h, _ptr(s), _ptr(je)))
        return s, je

    def grad_E0(self):
        d = np.zeros(3)
        _check(self.h, lib().esc_grad(self.h, None, _ptr(d), None))
        return d

    def grad(self, kind="Energy Current", cf_steps=200, omega_steps=499, domega=0.01, eta=0.05):
        """(dE0/d{K,J,h}, dImS_tt(omega)/d{K,J,h}) of the CF-mode total-current spectrum (FP64)."""
        cfg = DynCfg(DYN_KIND[kind], 1, omega_steps, domega, eta, cf_steps, C128)
        d = np.zeros(3)
        dS = np.zeros((omega_steps + 1, 3))
        _check(self.h, lib().esc_grad(self.h, ctypes.byref(cfg), _ptr(d), _ptr(dS)))
        return d, dS


def alu_peaks():
    """FP32 FMA, packed f32x2 FMA and FP64 FMA throughput of the current device (TFLOP/s) and the
    timed kernels' durations (ms)."""
    out = np.zeros(6)
    st = lib().esc_alu_peaks(_ptr(out))
    if st != ESC_OK:
        raise EscError(st, lib().esc_last_error(None).decode())
    return dict(ffma_tflops=out[0], ffma2_tflops=out[1], dfma_tflops=out[2], ms=out[3:].tolist())


# ------------------------------------------------------------------------------------------------
# Reference-named mirror
# ------------------------------------------------------------------------------------------------
class Hamiltonian:
    """Hamiltonian::MatrixVectorMult (src/Hamiltonian.h:480-557) on the GPU."""

    def __init__(self, variables, handle=None):
        self.variables = variables
        self.handle = handle or Handle(variables)

    def MatrixVectorMult(self, Vin):
        if Vin.size != self.handle.D:
            raise ValueError("LanczosSolver.h::Dot-Product size mismatch!")
        return self.handle.hv(Vin)


class DynLanczosSolver:
    """DynLanczosSolver::Lanczos_Nirav (src/DynLanczosSolver.h:38-239) on the GPU."""

    def __init__(self, variables, hamiltonian):
        self.variables = variables
        self.handle = hamiltonian.handle
        self.TriDeval = None

    def Lanczos_Nirav(self, PsiOrAll, start=None):
        if PsiOrAll not in ("OnlyEgs", "GS", "All"):
            raise RuntimeError("DynLanczosSolver: Use PsiOrAll==GS or All")
        r = self.handle.lanczos_gs(lanctype=PsiOrAll, start=start)
        self.TriDeval = r["ritz"]
        self.alpha, self.beta = r["alpha"], r["beta"]
        return r["gs"]


class Observables:
    """Observables::Apply* (src/Observables.h) on the GPU."""

    def __init__(self, variables, hamiltonian):
        self.handle = hamiltonian.handle

    def ApplyOp(self, inV, OpA, site):
        if OpA not in OP_ID:
            raise ValueError("Unknown Operator label")
        return self.handle.apply(OpA, site, inV)

    def __getattr__(self, name):
        if name.startswith("Apply") and name[5:] in OP_ID:
            op = name[5:]
            if op.endswith("Total"):
                return lambda GS_: self.handle.apply(op, 0, GS_)
            return lambda GS_, i: self.handle.apply(op, i, GS_)
        raise AttributeError(name)

    def measureLocalS(self, GS_):
        return self.handle.measure_local()[0]

    def measureLocalJe(self, GS_):
        return self.handle.measure_local()[1]

    def TwoPointCorr(self, OpA, OpB, GS_=None):
        """src/Observables.h:131-158, on the handle's ground state."""
        if OpA not in OP_ID or OpB not in OP_ID:
            raise ValueError("Unknown Operator label")
        return self.handle.two_point(OpA, OpB)


def StartDynamics(dynstr, variables, lanczos, mode=None):
    """src/dynamics.h:43-60: returns the spectrum rows of the dynamics kind `dynstr`."""
    if dynstr not in DYN_KIND:
        raise ValueError("Unknown dynstr parameter")
    p = variables.p
    return lanczos.handle.spectrum(dynstr, mode or ("Ritz" if p.dyn_mode == 0 else "CF"),
                                   cf_steps=p.dyn_lanczos_steps or p.lanczos_steps)
