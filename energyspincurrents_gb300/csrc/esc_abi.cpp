// esc_abi.cpp -- the C ABI (include/esc.h): handle, operators, GPU Lanczos, spectra.
//
// Host C++ drives hand-written sm_103a kernels (kernels.cu).  No CPU fallback exists: every
// vector operation runs on the device; the host only does O(M^2)-O(M^3) work on the tridiagonal
// matrix and the O(Omega x M) Lehmann / continued-fraction sums.
#include <algorithm>
#include <map>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <type_traits>

#include "esc_internal.h"

using esc::cplx;

struct esc_handle {
    esc_params p{};
    esc::Lattice L;
    std::vector<esc::Bond> bonds;
    esc::DevModel dm{};                 // model on relabelled sites (internal basis order)
    esc::Plan plan;                     // site relabelling + pass plan of the tiled H.v
    std::vector<esc::DevPass> passes;
    esc::DevPerm to_int{}, to_ref{};    // basis permutations reference <-> internal
    int N = 0;
    int64_t D = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    // copy streams and per-slot events of the pipelined host-buffer batches (created on first use)
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[2] = {nullptr, nullptr}, ev_afree[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr},
                ev_outfree[2] = {nullptr, nullptr};
    std::string err;
    // device memory owned by the handle
    double* d_part = nullptr; size_t part_bytes = 0;   // reduction partials
    double* d_sc = nullptr; size_t sc_bytes = 0;       // scalars (alpha, |w|^2, projections, ...)
    void* d_L = nullptr; size_t L_bytes = 0;           // Krylov basis
    void* d_work = nullptr; size_t work_bytes = 0;     // work vectors
    void* d_gs = nullptr; size_t gs_bytes = 0;         // ground state
    void* d_io = nullptr; size_t io_bytes = 0;         // staging for host-pointer calls
    void* d_cfb = nullptr; size_t cfb_bytes = 0;       // batched CF vectors (3 x ncols x D)
    double* d_cfs = nullptr; size_t cfs_bytes = 0;     // batched CF scalars
    int* d_cfi = nullptr; size_t cfi_bytes = 0;        // batched CF flags / counters
    void* d_diag[2] = {nullptr, nullptr};              // diagonal of the bond terms per dtype
    size_t diag_bytes[2] = {0, 0};
    // ground-state Lanczos results
    int nsteps = 0;
    bool have_gs = false, have_basis = false;
    esc_dtype basis_dt = ESC_C128;
    int64_t L_ld = 0;
    std::vector<double> alpha, beta, ritz, Z;
};

namespace {

thread_local std::string g_err;

struct Fail : std::runtime_error {
    esc_status st;
    Fail(esc_status s, const std::string& m) : std::runtime_error(m), st(s) {}
};

}  // namespace

void esc::set_last_error(const std::string& msg) { g_err = msg; }

namespace {

esc_status finish(esc_handle* h, esc_status st, const std::string& msg) {
    g_err = msg;
    if (h) h->err = msg;
    return st;
}

template <typename F>
esc_status guarded(esc_handle* h, F&& f) {
    try {
        f();
        if (h) h->err.clear();
        return ESC_OK;
    } catch (Fail& e) {
        return finish(h, e.st, e.what());
    } catch (esc::CudaError& e) {
        return finish(h, ESC_ERR_CUDA, e.what());
    } catch (std::invalid_argument& e) {
        return finish(h, ESC_ERR_PARAM, e.what());
    } catch (std::bad_alloc&) {
        return finish(h, ESC_ERR_MEMORY, "host allocation failed");
    } catch (std::exception& e) {
        return finish(h, ESC_ERR_NUMERIC, e.what());
    }
}

size_t esize(esc_dtype dt) { return dt == ESC_C64 ? 8 : 16; }

void ensure(void*& p, size_t& cap, size_t need) {
    if (need <= cap && p) return;
    if (p) { cudaFree(p); p = nullptr; cap = 0; }
    if (need == 0) return;
    cudaError_t e = cudaMalloc(&p, need);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        p = nullptr;
        throw Fail(ESC_ERR_MEMORY, "device allocation of " + std::to_string(need >> 20) + " MiB failed (" +
                                       cudaGetErrorString(e) + ")");
    }
    cap = need;
}
template <typename T>
void ensure_t(T*& p, size_t& cap, size_t need) {
    void* q = p;
    ensure(q, cap, need);
    p = (T*)q;
}

void sync(esc_handle* h) { ESC_CUDA(cudaStreamSynchronize(h->stream)); }

// Precomputed bond diagonal (the analogue of the reference's HDiag without the field term),
// 4 B/state for complex64, 8 B/state for complex128; computed on first use.  If it cannot be
// allocated the tiled kernel computes the diagonal itself (slower, same result).
const void* diag_for(esc_handle* h, esc_dtype dt) {
    const int i = dt == ESC_C64 ? 1 : 0;
    if (h->d_diag[i]) return h->d_diag[i];
    const size_t need = (size_t)h->D * (dt == ESC_C64 ? 4 : 8);
    if (cudaMalloc(&h->d_diag[i], need) != cudaSuccess) {
        (void)cudaGetLastError();
        h->d_diag[i] = nullptr;
        return nullptr;
    }
    h->diag_bytes[i] = need;
    if (dt == ESC_C64) esc::launch_diag<float>(h->dm, h->d_diag[i], h->D, h->stream);
    else esc::launch_diag<double>(h->dm, h->d_diag[i], h->D, h->stream);
    return h->d_diag[i];
}

void ensure_partials(esc_handle* h, int rows) {
    const size_t need = (size_t)std::max(rows, 4) * esc::RED_MAX_BLOCKS * 2 * sizeof(double);
    ensure_t(h->d_part, h->part_bytes, need);
}
int64_t part_cap_doubles(esc_handle* h) { return (int64_t)(h->part_bytes / sizeof(double)); }

void permute(esc_handle* h, const esc::DevPerm& p, const void* in, void* out, int64_t n, esc_dtype dt) {
    if (dt == ESC_C64) esc::launch_permute<float>(p, in, out, n, h->stream);
    else esc::launch_permute<double>(p, in, out, n, h->stream);
}

// Staged input/output.  The kernels work in the internal basis order; unless the caller says
// ESC_INTERNAL_ORDER, inputs are permuted in and outputs permuted out (through d_io), and host
// pointers are copied.  One call handles `cols` vectors of `n` elements with stride `ld`.
struct Staged {
    const void* in;
    void* out;
    int64_t ld;
};
Staged stage(esc_handle* h, const void* in, void* out, int cols, int64_t ld, esc_dtype dt, int flags) {
    const size_t es = esize(dt);
    const int64_t n = h->D;
    const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
    if (dev && internal) return {in, out, ld};
    const size_t vb = (size_t)n * es;
    ensure(h->d_io, h->io_bytes, 2 * (size_t)cols * vb);
    char* A = (char*)h->d_io;              // internal-order input
    char* B = A + (size_t)cols * vb;       // internal-order output / reference-order staging
    for (int c = 0; c < cols; c++) {
        if (!in) break;
        const char* src = (const char*)in + (size_t)c * ld * es;
        if (internal) {
            ESC_CUDA(cudaMemcpyAsync(A + c * vb, src, vb, cudaMemcpyHostToDevice, h->stream));
        } else if (dev) {
            permute(h, h->to_int, src, A + c * vb, n, dt);
        } else {
            ESC_CUDA(cudaMemcpyAsync(B + c * vb, src, vb, cudaMemcpyHostToDevice, h->stream));
            permute(h, h->to_int, B + c * vb, A + c * vb, n, dt);
        }
    }
    return {in ? A : nullptr, B, n};
}
void unstage(esc_handle* h, const Staged& s, void* out, int cols, int64_t ld, esc_dtype dt, int flags) {
    const size_t es = esize(dt);
    const int64_t n = h->D;
    const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
    if (!(dev && internal) && out) {
        const size_t vb = (size_t)n * es;
        // staging for the reference-order / host copy (already there when stage() made it; a
        // result that lives elsewhere, e.g. the ground state, may need it allocated here)
        if (!internal && !dev) ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, (size_t)cols * vb));
        char* A = (char*)h->d_io;
        for (int c = 0; c < cols; c++) {
            char* dst = (char*)out + (size_t)c * ld * es;
            const char* res = (const char*)s.out + (size_t)c * vb;
            if (internal) {
                ESC_CUDA(cudaMemcpyAsync(dst, res, vb, cudaMemcpyDeviceToHost, h->stream));
            } else if (dev) {
                permute(h, h->to_ref, res, dst, n, dt);
            } else {
                permute(h, h->to_ref, res, A + c * vb, n, dt);
                ESC_CUDA(cudaMemcpyAsync(dst, A + c * vb, vb, cudaMemcpyDeviceToHost, h->stream));
            }
        }
    }
    if (!(flags & ESC_ASYNC) || !dev) sync(h);
}

// ---------------------------------------------------------------------------------------------
// Templated device pipelines
// ---------------------------------------------------------------------------------------------
template <typename R>
struct Pipe {
    esc_handle* h;
    static constexpr size_t ES = 2 * sizeof(R);
    int64_t D;
    explicit Pipe(esc_handle* hh) : h(hh), D(hh->D) {}
    void hv(const void* in, void* out) {
        esc::launch_hv_tiled<R>(h->dm, h->passes, in, out, D, diag_for(h, sizeof(R) == 4 ? ESC_C64 : ESC_C128),
                                h->stream);
    }
    void apply(const esc::DevOp& op, const void* in, void* out) { esc::launch_apply<R>(op, in, out, D, h->stream); }
    void dot(const void* a, const void* b, double* dst) { esc::launch_dot<R>(a, b, D, h->d_part, dst, h->stream); }
    void nrm2(const void* a, double* dst) { esc::launch_nrm2<R>(a, D, h->d_part, dst, h->stream); }
    void scale(const void* in, void* out, const double* d_nrm2) { esc::launch_scale_rsqrt<R>(in, out, d_nrm2, D, h->stream); }
};

// Ground-state Lanczos, DynLanczosSolver::Lanczos_Nirav (src/DynLanczosSolver.h:38-239).
template <typename R>
void lanczos_gs(esc_handle* h, const esc_lanczos_cfg& cfg, const void* d_start) {
    Pipe<R> P(h);
    const int64_t D = h->D;
    const size_t ES = Pipe<R>::ES;
    const int M = cfg.steps;
    // GS without reorthogonalisation keeps three vectors and rebuilds |gs> in a second pass
    // (the Lanczos vectors are recomputed from the recorded alpha/beta, not stored): the mode for
    // bases too large to hold M+1 vectors (N = 28..32).
    const bool recompute = cfg.lanctype == 1 && !cfg.reortho;
    const bool store = cfg.lanctype != 0 && !recompute;  // OnlyEgs keeps no basis (returns a zero vector)
    const bool reo = store && cfg.reortho;
    const int nvec = store ? M + 1 : 3;
    h->have_gs = h->have_basis = false;
    ensure(h->d_L, h->L_bytes, (size_t)nvec * D * ES);
    ensure(h->d_work, h->work_bytes, (size_t)D * ES);
    // scalars: alpha[2M] | b2[M+2] | tmp[8] | r[2(M+2)] | z[M+2]
    const size_t n_sc = 2 * (size_t)M + (M + 2) + 8 + 2 * (size_t)(M + 2) + (M + 2);
    ensure_t(h->d_sc, h->sc_bytes, n_sc * sizeof(double));
    double* d_alpha = h->d_sc;
    double* d_b2 = d_alpha + 2 * M;
    double* d_tmp = d_b2 + (M + 2);
    double* d_r = d_tmp + 8;
    double* d_z = d_r + 2 * (M + 2);
    ensure_partials(h, reo ? M + 2 : 4);
    ESC_CUDA(cudaMemsetAsync(h->d_sc, 0, n_sc * sizeof(double), h->stream));
    auto Lv = [&](int i) -> char* { return (char*)h->d_L + (size_t)(store ? i : i % 3) * D * ES; };
    void* w = h->d_work;

    // Vorig.normalize(); V0 = Vorig (:58-66)
    P.nrm2(d_start, d_tmp);
    P.scale(d_start, Lv(0), d_tmp);
    // iteration 0 (:75-83): V1 = H V0; alpha0 = <V0|V1>; V1 -= alpha0 V0; beta1 = |V1|; normalise
    P.hv(Lv(0), w);
    P.dot(Lv(0), w, d_alpha);
    esc::launch_lanczos_update<R>(w, Lv(0), nullptr, d_alpha, nullptr, D, h->d_part, d_b2 + 1, h->stream);
    P.scale(w, Lv(1), d_b2 + 1);
    int exit_iter = M - 1;
    double E0 = 1.0;
    for (int iter = 1; iter <= M - 1; iter++) {             // :91-163
        P.hv(Lv(iter), w);
        P.dot(Lv(iter), w, d_alpha + 2 * iter);
        esc::launch_lanczos_update<R>(w, Lv(iter), Lv(iter - 1), d_alpha + 2 * iter, d_b2 + iter, D, h->d_part,
                                      d_b2 + iter + 1, h->stream);
        P.scale(w, Lv(iter + 1), d_b2 + iter + 1);
        if (reo) {
            // Full reorthogonalisation against L_0..L_iter (:105-119).  The reference does one
            // modified Gram-Schmidt sweep; here two classical sweeps (CGS2) as two GEMV pairs,
            // which orthogonalise to the same working precision.
            for (int pass = 0; pass < 2; pass++) {
                esc::launch_gemv_h<R>(h->d_L, D, iter + 1, Lv(iter + 1), D, h->d_part, part_cap_doubles(h), d_r,
                                      h->stream);
                esc::launch_gemv_sub<R>(h->d_L, D, iter + 1, d_r, Lv(iter + 1), D, h->stream);
            }
            P.nrm2(Lv(iter + 1), d_tmp + 1);
            P.scale(Lv(iter + 1), Lv(iter + 1), d_tmp + 1);
        }
        if (cfg.eps > 0.0) {                                 // :125-151 (convergence test)
            std::vector<double> a(2 * (iter + 1)), b2(iter + 2);
            ESC_CUDA(cudaMemcpyAsync(a.data(), d_alpha, a.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            ESC_CUDA(cudaMemcpyAsync(b2.data(), d_b2, b2.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            sync(h);
            std::vector<double> d(iter + 1), e(iter + 1, 0.0);
            for (int i = 0; i <= iter; i++) d[i] = a[2 * i];
            for (int i = 0; i < iter; i++) e[i] = std::sqrt(b2[i + 1]);
            if (!esc::tridiag_eig(iter + 1, d, e, nullptr)) throw Fail(ESC_ERR_NUMERIC, "diag: tridiagonal eigensolver failed");
            const double diff = std::fabs(E0 - d[0]);
            E0 = d[0];
            if (diff < cfg.eps) { exit_iter = iter; break; }
        }
    }
    const int n = exit_iter + 1;                             // EXITiter (:164)
    std::vector<double> a(2 * (size_t)M), b2(M + 2);
    ESC_CUDA(cudaMemcpyAsync(a.data(), d_alpha, a.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ESC_CUDA(cudaMemcpyAsync(b2.data(), d_b2, b2.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    sync(h);
    h->alpha.assign(n, 0.0);
    h->beta.assign(n + 1, 0.0);
    for (int i = 0; i < n; i++) h->alpha[i] = a[2 * i];
    for (int i = 1; i <= n; i++) h->beta[i] = std::sqrt(b2[i]);
    for (int i = 0; i < n; i++)
        if (!std::isfinite(h->alpha[i]) || !std::isfinite(h->beta[i + 1]))
            throw Fail(ESC_ERR_NUMERIC, "NaN/Inf in Lanczos coefficients at step " + std::to_string(i));
    for (int i = 1; i < n; i++)
        if (h->beta[i] == 0.0)
            throw Fail(ESC_ERR_NUMERIC, "Lanczos breakdown: beta=0 at step " + std::to_string(i) +
                                            " (Krylov space exhausted; use fewer LanczosSteps)");
    std::vector<double> d(h->alpha), e(n, 0.0);
    for (int i = 0; i < n - 1; i++) e[i] = h->beta[i + 1];
    h->Z.clear();
    if (!esc::tridiag_eig(n, d, e, (store || recompute) ? &h->Z : nullptr)) throw Fail(ESC_ERR_NUMERIC, "diag: tridiagonal eigensolver failed");
    h->ritz = d;
    h->nsteps = n;
    ensure(h->d_gs, h->gs_bytes, (size_t)D * ES);
    if (recompute) {
        // second pass: identical kernels on identical inputs regenerate L_0..L_{n-1} bit for bit
        ESC_CUDA(cudaMemcpyAsync(d_z, h->Z.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        ESC_CUDA(cudaMemsetAsync(h->d_gs, 0, (size_t)D * ES, h->stream));
        P.nrm2(d_start, d_tmp);
        P.scale(d_start, Lv(0), d_tmp);
        esc::launch_axpy_dev<R>(Lv(0), h->d_gs, d_z, D, h->stream);
        for (int it = 0; it + 1 < n; it++) {
            P.hv(Lv(it), w);
            esc::launch_lanczos_update<R>(w, Lv(it), it ? Lv(it - 1) : nullptr, d_alpha + 2 * it, it ? d_b2 + it : nullptr,
                                          D, h->d_part, d_tmp + 2, h->stream);
            P.scale(w, Lv(it + 1), d_b2 + it + 1);
            esc::launch_axpy_dev<R>(Lv(it + 1), h->d_gs, d_z + it + 1, D, h->stream);
        }
    } else if (store) {
        // PsiAll[0] = sum_m L_m Z(m,0) (:208-234), without forming the other Ritz vectors
        ESC_CUDA(cudaMemcpyAsync(d_z, h->Z.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        esc::launch_lincomb<R>(h->d_L, D, n, d_z, h->d_gs, D, h->stream);
        h->have_basis = cfg.lanctype == 2;
    } else {
        ESC_CUDA(cudaMemsetAsync(h->d_gs, 0, (size_t)D * ES, h->stream));   // OnlyEgs returns zeros (:178-180)
    }
    if ((recompute || store) && !reo) {
        // Without reorthogonalisation the Lanczos vectors lose orthogonality once the ground state
        // has converged, and sum_m Z(m,0) L_m is then not a unit vector: normalise it.  (With full
        // reorthogonalisation, the reference's mode, the sum is kept exactly as the reference forms it.)
        P.nrm2(h->d_gs, d_tmp + 3);
        P.scale(h->d_gs, h->d_gs, d_tmp + 3);
    }
    if (!store && h->d_L) {   // the three recurrence vectors are not needed any more: free them for the dynamics
        cudaFree(h->d_L);
        h->d_L = nullptr;
        h->L_bytes = 0;
    }
    h->basis_dt = sizeof(R) == 8 ? ESC_C128 : ESC_C64;
    h->L_ld = D;
    h->have_gs = true;
    sync(h);
}

// ---------------------------------------------------------------------------------------------
// Batched continued-fraction Lanczos (batched.cu)
// ---------------------------------------------------------------------------------------------
int cf_batch_width(esc_handle* h, size_t es, int want) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); fr = 0; }
    const size_t per = 3 * (size_t)h->D * es;
    const size_t have = fr + h->cfb_bytes;
    int w = (int)std::min<size_t>((size_t)want, have > (size_t)1 << 30 ? (have - ((size_t)1 << 30)) / per : 0);
    return std::max(1, std::min(w, esc::MAX_COLS));
}

// Start vectors must already be in column slots of set 1 of d_cfb.  Returns a (Re alpha),
// b (b[0] = |phi|) and the number of steps per column.
//
// head > 0 (complex64 columns only): the first `head` iterations run on complex128 copies of the
// columns; the last two vectors are then rounded to complex64 and the recurrence continues in
// complex64 from iteration `head`.  The leading iterations fix the converged, low-lying poles of
// the continued fraction, so their rounding in FP32 is what costs accuracy; the tail only adds
// resolution.  The head needs 3 x ncols complex128 vectors for its duration; without that much
// free device memory the run is all complex64.
template <typename R>
void cf_batch_run(esc_handle* h, int ncols, int kmax, const std::vector<int>& steps, const std::vector<esc::DevModel>& ms,
                  double tol, bool graph, std::vector<std::vector<double>>& A, std::vector<std::vector<double>>& B,
                  int head = 0) {
    const size_t nd = (size_t)ncols * esc::CFB_GRID * 2 + (size_t)ncols * kmax * 2 + (size_t)ncols * (kmax + 1);
    ensure_t(h->d_cfs, h->cfs_bytes, nd * sizeof(double));
    ensure_t(h->d_cfi, h->cfi_bytes, (2 * (size_t)ncols + 2) * sizeof(int));
    auto setup = [&](auto& cb, void* bufs, const void* dg) {
        typedef typename std::remove_reference<decltype(cb)>::type CB;
        cb.ncols = ncols; cb.kmax = kmax; cb.D = h->D; cb.tol = tol; cb.use_graph = graph;
        cb.bufs = bufs;
        cb.d_part = h->d_cfs;
        cb.d_alpha = cb.d_part + (size_t)ncols * esc::CFB_GRID * 2;
        cb.d_b2 = cb.d_alpha + (size_t)ncols * kmax * 2;
        cb.d_active = h->d_cfi;
        cb.d_steps = h->d_cfi + ncols;
        cb.d_it = h->d_cfi + 2 * ncols;
        typedef typename std::conditional<std::is_same<CB, esc::CFBatch<float>>::value, float, double>::type RR;
        cb.hv_column = [h, &ms, dg](int c, const void* in, void* out, const int* active, cudaStream_t s) {
            esc::launch_hv_tiled<RR>(ms[c], h->passes, in, out, h->D, dg, s, active);
        };
    };
    ESC_CUDA(cudaMemsetAsync(h->d_cfs, 0, nd * sizeof(double), h->stream));
    esc::CFBatch<R> cb;
    setup(cb, h->d_cfb, diag_for(h, sizeof(R) == 4 ? ESC_C64 : ESC_C128));
    head = std::min(head, kmax);
    void* dd = nullptr;
    if (sizeof(R) == 4 && head > 0) {
        const size_t vs = (size_t)ncols * h->D;   // states per set
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); fr = 0; }
        const size_t need = 3 * vs * 16 + (h->d_diag[0] ? 0 : (size_t)h->D * 8);
        if (fr > need + ((size_t)1 << 30) && cudaMalloc(&dd, 3 * vs * 16) == cudaSuccess) {
            char* d1 = (char*)dd + vs * 16;
            esc::launch_convert_c64_to_c128((char*)h->d_cfb + vs * 8, d1, (int64_t)vs, h->stream);
            std::vector<int> hs(ncols);
            for (int c = 0; c < ncols; c++) hs[c] = std::min(steps[c], head);
            ESC_CUDA(cudaMemcpyAsync(cb.d_steps, hs.data(), ncols * sizeof(int), cudaMemcpyHostToDevice, h->stream));
            esc::CFBatch<double> c64;
            setup(c64, dd, diag_for(h, ESC_C128));
            c64.run(h->stream);   // synchronises
            // columns that ran the whole head without stopping continue in complex64
            std::vector<double> b2((size_t)ncols * (kmax + 1));
            ESC_CUDA(cudaMemcpy(b2.data(), cb.d_b2, b2.size() * sizeof(double), cudaMemcpyDeviceToHost));
            std::vector<int> act(ncols, 0);
            for (int c = 0; c < ncols; c++) {
                const double b0 = std::sqrt(b2[(size_t)c * (kmax + 1)]);
                bool live = b0 > 0.0 && steps[c] > head;
                for (int k = 1; live && k <= head; k++)
                    if (!(std::sqrt(b2[(size_t)c * (kmax + 1) + k]) > tol * b0)) live = false;
                act[c] = live ? 1 : 0;
            }
            for (int j = 0; j < 2; j++) {
                const int set = (head + j) % 3;
                esc::launch_convert_c128_to_c64((char*)dd + set * vs * 16, (char*)h->d_cfb + set * vs * 8, (int64_t)vs,
                                                h->stream);
            }
            ESC_CUDA(cudaMemcpyAsync(cb.d_active, act.data(), ncols * sizeof(int), cudaMemcpyHostToDevice, h->stream));
            sync(h);
            cudaFree(dd);
            cb.start_it = head;
        } else {
            (void)cudaGetLastError();
            dd = nullptr;
        }
    }
    ESC_CUDA(cudaMemcpyAsync(cb.d_steps, steps.data(), ncols * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    cb.run(h->stream);
    std::vector<double> al((size_t)ncols * kmax * 2), b2((size_t)ncols * (kmax + 1));
    ESC_CUDA(cudaMemcpyAsync(al.data(), cb.d_alpha, al.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    ESC_CUDA(cudaMemcpyAsync(b2.data(), cb.d_b2, b2.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    sync(h);
    A.assign(ncols, {});
    B.assign(ncols, {});
    for (int c = 0; c < ncols; c++) {
        const double b0 = std::sqrt(b2[(size_t)c * (kmax + 1)]);
        B[c].push_back(b0);
        if (b0 == 0.0) continue;
        for (int k = 0; k < kmax; k++) {
            A[c].push_back(al[((size_t)c * kmax + k) * 2]);
            const double bn = std::sqrt(b2[(size_t)c * (kmax + 1) + k + 1]);
            B[c].push_back(bn);
            if (k + 1 >= steps[c] || !(bn > tol * b0)) break;
        }
    }
}

esc::DevModel model_with_field(const esc_handle* h, double bx, double by, double bz) {
    esc::DevModel m = h->dm;
    m.fx = 0.5 * bx; m.fy = 0.5 * by; m.fz = 0.5 * bz;
    esc::fill_float_copies(m);
    return m;
}

// ---------------------------------------------------------------------------------------------
// Spectra
// ---------------------------------------------------------------------------------------------
struct Grid {
    int nw;
    double dw, eta;
};

// One operator "channel": a combination of operator strings applied to |gs>.
std::vector<esc::OpTerm> combine(const std::vector<esc::OpTerm>& a, const std::vector<esc::OpTerm>& b, cplx cb) {
    std::vector<esc::OpTerm> t(a);
    for (auto x : b) { x.coef *= cb; t.push_back(x); }
    return t;
}

template <typename R>
struct Spectra {
    esc_handle* h;
    Pipe<R> P;
    const int64_t D;
    char* buf(int i) { return (char*)h->d_work + (size_t)i * D * Pipe<R>::ES; }
    explicit Spectra(esc_handle* hh) : h(hh), P(hh), D(hh->D) {}

    // <gs| A |gs> with A given as terms; uses work vector `slot`.
    cplx expect(const std::vector<esc::OpTerm>& t, int slot, double* d_tmp) {
        P.apply(esc::make_dev_op(t, &h->plan.perm), h->d_gs, buf(slot));
        P.dot(h->d_gs, buf(slot), d_tmp);
        double r[2];
        ESC_CUDA(cudaMemcpyAsync(r, d_tmp, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        sync(h);
        return cplx(r[0], r[1]);
    }

    // Ritz-mode overlaps O[n] = <psi_n | A gs> = sum_m Z(m,n) <L_m | A gs>  (dynamics.h:256-263)
    std::vector<cplx> ritz_overlaps(const std::vector<esc::OpTerm>& t, int slot, double* d_r, double* d_tmp,
                                    cplx* elastic) {
        const int M = h->nsteps;
        P.apply(esc::make_dev_op(t, &h->plan.perm), h->d_gs, buf(slot));
        P.dot(h->d_gs, buf(slot), d_tmp);
        esc::launch_gemv_h<R>(h->d_L, h->L_ld, M, buf(slot), D, h->d_part, part_cap_doubles(h), d_r, h->stream);
        std::vector<double> r(2 * (size_t)M), el(2);
        ESC_CUDA(cudaMemcpyAsync(r.data(), d_r, r.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        ESC_CUDA(cudaMemcpyAsync(el.data(), d_tmp, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        sync(h);
        *elastic = cplx(el[0], el[1]);
        std::vector<cplx> O(M);
        for (int n = 0; n < M; n++) {
            cplx s(0, 0);
            for (int m = 0; m < M; m++) s += h->Z[(size_t)n * M + m] * cplx(r[2 * m], r[2 * m + 1]);
            O[n] = s;
        }
        return O;
    }
};

}  // namespace

// =============================================================================================
// C ABI
// =============================================================================================
namespace {

std::vector<std::pair<int, int>> bond_pairs(const esc_handle* h) {
    std::vector<std::pair<int, int>> pairs;
    for (const auto& b : h->bonds)
        if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
    return pairs;
}

// Installs a site relabelling + pass plan: relabelled model, passes, basis permutations.  The
// bond diagonal depends on the relabelling, so cached diagonal vectors are dropped.
void install_plan(esc_handle* h, const esc::Plan& plan, int balance, int stages, int tb_bits = 0) {
    h->plan = plan;
    std::vector<esc::Bond> rb(h->bonds);
    for (auto& b : rb) { b.i = h->plan.perm[b.i]; b.j = h->plan.perm[b.j]; }
    h->dm = esc::make_dev_model(h->p, h->L, rb, h->p.Bxx, h->p.Byy, h->p.Bzz);
    h->passes = esc::make_passes(h->plan, h->dm, balance, stages, tb_bits);
    std::vector<int> inv(h->N), fwd(h->N);
    for (int s = 0; s < h->N; s++) { inv[h->plan.perm[s]] = s; fwd[s] = h->plan.perm[s]; }
    h->to_int = esc::make_perm_table(inv);    // internal bit b reads reference bit inv[b]
    h->to_ref = esc::make_perm_table(fwd);    // reference bit s reads internal bit perm[s]
    for (int i = 0; i < 2; i++)
        if (h->d_diag[i]) {
            cudaFree(h->d_diag[i]);
            h->d_diag[i] = nullptr;
            h->diag_bytes[i] = 0;
        }
}

// Run-time specialised complex64 passes (hv_jit.cu): ESC_JIT=0 off, =1 on, =require on and an
// error if it fails; by default on from 2^22 states, where the compile time is repaid.
void specialise(esc_handle* h, std::vector<esc::DevPass>& passes, int force = -1) {
    const char* je = std::getenv("ESC_JIT");
    bool jit = je ? std::strcmp(je, "0") != 0 : h->D >= (int64_t(1) << 22);
    if (force >= 0) jit = force == 1;
    if (!jit) return;
    std::string err;
    if (!esc::jit_compile(passes, err) && je && std::strcmp(je, "require") == 0)
        throw Fail(ESC_ERR_CUDA, "run-time specialisation of the H.v passes failed: " + err);
}

// Tuning file (ESC_TUNE_FILE): one line per tuned Hamiltonian and device,
//   <key> | T balance npasses | jit,stages,tb_bits per pass
// written by the self-tuner and applied by esc_create, so a tuned configuration is reused without
// timing again.  The key covers the device name and everything the plan and passes depend on.
std::string tune_key(const esc_handle* h) {
    cudaDeviceProp pr{};
    if (cudaGetDeviceProperties(&pr, h->device) != cudaSuccess) (void)cudaGetLastError();
    std::ostringstream k;
    k.precision(17);
    k << "dev=" << pr.name << " model=" << h->p.model << " Lx=" << h->p.Lx << " Ly=" << h->p.Ly << " pbc=" << h->p.pbcx
      << h->p.pbcy << " K=" << h->p.Kxx << "," << h->p.Kyy << "," << h->p.Kzz << " B=" << h->p.Bxx << "," << h->p.Byy << ","
      << h->p.Bzz << " J=" << h->p.jheis;
    return k.str();
}

void save_tuning(const esc_handle* h, int T, int balance, const std::vector<esc::DevPass>& ps) {
    const char* f = std::getenv("ESC_TUNE_FILE");
    if (!f || !*f) return;
    FILE* fp = std::fopen(f, "a");
    if (!fp) return;
    std::fprintf(fp, "%s | %d %d %d |", tune_key(h).c_str(), T, balance, (int)ps.size());
    for (const auto& p : ps) std::fprintf(fp, " %d,%d,%d", p.jit >= 0 ? 1 : 0, p.stages, p.tb_bits);
    std::fprintf(fp, "\n");
    std::fclose(fp);
}

// Applies the last matching line of ESC_TUNE_FILE; false if there is none.
bool load_tuning(esc_handle* h) {
    const char* f = std::getenv("ESC_TUNE_FILE");
    if (!f || !*f) return false;
    FILE* fp = std::fopen(f, "r");
    if (!fp) return false;
    const std::string key = tune_key(h);
    std::string found;
    char line[4096];
    while (std::fgets(line, sizeof line, fp)) {
        std::string l(line);
        if (l.compare(0, key.size(), key) == 0 && l.size() > key.size() && l[key.size()] == ' ') found = l.substr(key.size());
    }
    std::fclose(fp);
    if (found.empty()) return false;
    int T = 0, balance = 0, n = 0;
    std::istringstream in(found);
    char bar;
    in >> bar >> T >> balance >> n >> bar;
    std::vector<std::array<int, 3>> var(n);
    for (auto& v : var) {
        char c1, c2;
        in >> v[0] >> c1 >> v[1] >> c2 >> v[2];
    }
    if (!in || T < 4) return false;
    const esc::Plan plan = esc::make_plan(h->N, bond_pairs(h), T, 3, 200);
    if ((int)plan.tiles.size() != n) return false;
    install_plan(h, plan, balance, 2);
    std::vector<esc::DevPass> comp(h->passes);
    std::map<std::array<int, 2>, std::vector<esc::DevPass>> built;
    for (int p = 0; p < n; p++) {
        const std::array<int, 2> k{var[p][1], var[p][2]};
        if (!built.count(k)) {
            built[k] = esc::make_passes(h->plan, h->dm, balance, k[0], k[1]);
            if (std::any_of(var.begin(), var.end(), [&](const std::array<int, 3>& x) { return x[0] && x[1] == k[0] && x[2] == k[1]; })) {
                std::vector<esc::DevPass> sp = built[k];
                std::string err;
                if (esc::jit_compile(sp, err)) built[std::array<int, 2>{-k[0], k[1]}] = sp;
            }
        }
        const auto it = built.find(var[p][0] ? std::array<int, 2>{-k[0], k[1]} : k);
        comp[p] = (it != built.end() ? it->second : built[k])[p];
    }
    h->passes = comp;
    return true;
}

// Self-tuning of the complex64 H.v.  Plans: tile bits T in {11, 12, 13} (above 26 sites only 12:
// the others never win there -- one more pass, or one CTA per SM) x first-fit / group-minimising
// term-to-pass assignment (make_passes modes 0 and 2; the balanced mode 1 never won).  Kernel variants per plan: ahead-of-time vs run-time specialised;
// 512, 256 or 128 threads per 4096-state tile (8, 16, 32 register states each); 2 or 3 tile buffers,
// or 2 plus staged epilogue loads.  Every variant is timed pass by pass (CUDA events on the
// handle's stream, median of 3 after a warm-up); a plan's composite takes the fastest variant of
// each pass (light and heavy passes prefer different variants) and is timed as a whole; the
// fastest composite is installed.  All variants compute the same H.v up to complex64 rounding (the
// tests hold each to the oracle).  Needs two complex64 vectors of scratch; refuses once a ground
// state exists (a new plan relabels the internal basis).
std::string autotune(esc_handle* h, std::vector<double>* times) {
    if (h->have_gs) throw Fail(ESC_ERR_STATE, "autotune before the first Lanczos run (it may relabel the basis)");
    const int64_t D = h->D;
    void* buf = nullptr;
    ESC_CUDA(cudaMalloc(&buf, (size_t)D * 16));
    void* v = buf;
    void* w = (char*)buf + (size_t)D * 8;
    esc::launch_start_normal<float>(12345, v, D, h->stream);
    cudaEvent_t e0, e1;
    ESC_CUDA(cudaEventCreate(&e0));
    ESC_CUDA(cudaEventCreate(&e1));
    auto median_ms = [&](const std::vector<esc::DevPass>& ps) {
        const void* dg = diag_for(h, ESC_C64);
        esc::launch_hv_tiled<float>(h->dm, ps, v, w, D, dg, h->stream);
        std::vector<float> ms(3);
        for (float& x : ms) {
            ESC_CUDA(cudaEventRecord(e0, h->stream));
            esc::launch_hv_tiled<float>(h->dm, ps, v, w, D, dg, h->stream);
            ESC_CUDA(cudaEventRecord(e1, h->stream));
            ESC_CUDA(cudaEventSynchronize(e1));
            ESC_CUDA(cudaEventElapsedTime(&x, e0, e1));
        }
        std::sort(ms.begin(), ms.end());
        return (double)ms[1];
    };
    std::ostringstream rep;
    const esc::Plan keep = h->plan;
    const std::vector<esc::DevPass> keep_passes = h->passes;
    double best = 1e300;
    esc::Plan bplan;
    int bbal = 0, bT = 0;
    std::vector<esc::DevPass> bpasses;
    try {
        for (int T : {11, 12, 13}) {
            if (T > h->N || (h->N > 26 && T != 12)) continue;
            const esc::Plan plan = esc::make_plan(h->N, bond_pairs(h), T, 3, 200);
            for (int balance : {0, 2}) {
                std::vector<std::vector<esc::DevPass>> vars;
                std::vector<std::vector<double>> per;
                for (int tb : {9, 8, 7})
                for (int stages : {2, 3, 4})
                    for (int jit : {0, 1}) {
                        if (T == 13 && (jit || tb != 9)) continue;   // 8192-state tiles: generic kernel only
                        install_plan(h, plan, balance, stages, tb);
                        if (jit) specialise(h, h->passes, 1);
                        bool spec = false;
                        for (const auto& ps : h->passes) spec = spec || ps.jit >= 0;
                        if (jit && !spec) continue;
                        std::vector<double> t;
                        for (const auto& ps : h->passes) t.push_back(median_ms({ps}));
                        const double tot = median_ms(h->passes);
                        rep << "T=" << T << " passes=" << plan.tiles.size() << " balance=" << balance << " threads="
                            << (1 << tb) << " jit=" << jit << " stages=" << stages << ": " << tot << " ms | per pass";
                        for (double x : t) rep << " " << x;
                        rep << "\n";
                        if (times) times->push_back(tot);
                        vars.push_back(h->passes);
                        per.push_back(t);
                    }
                // composite: fastest variant of each pass
                std::vector<esc::DevPass> comp = vars[0];
                rep << "  composite T=" << T << " balance=" << balance << ": variants";
                for (size_t p = 0; p < comp.size(); p++) {
                    size_t bv = 0;
                    for (size_t k = 1; k < vars.size(); k++)
                        if (per[k][p] < per[bv][p]) bv = k;
                    comp[p] = vars[bv][p];
                    rep << " " << (comp[p].jit >= 0 ? "jit" : "aot") << "/" << comp[p].stages << "/" << (1 << comp[p].tb_bits);
                }
                install_plan(h, plan, balance, 2);   // model, permutations, diagonal of this plan
                const double tc = median_ms(comp);
                rep << ": " << tc << " ms\n";
                if (tc < best) { best = tc; bplan = plan; bbal = balance; bT = T; bpasses = comp; }
            }
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(buf);
        install_plan(h, keep, -1, 0);
        h->passes = keep_passes;
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    install_plan(h, bplan, bbal, 2);
    h->passes = bpasses;
    save_tuning(h, bT, bbal, bpasses);
    rep << "chosen: T=" << bT << " balance=" << bbal << " passes:";
    for (const auto& ps : bpasses) rep << " " << (ps.jit >= 0 ? "jit" : "aot") << "/" << ps.stages << "/" << (1 << ps.tb_bits);
    rep << " (" << best << " ms)\n";
    return rep.str();
}

}  // namespace

extern "C" {

const char* esc_last_error(const esc_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

esc_status esc_create(const esc_params* p, esc_handle** out) {
    if (!p || !out) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    *out = nullptr;
    std::unique_ptr<esc_handle> h(new esc_handle());
    esc_status st = guarded(h.get(), [&]() {
        h->p = *p;
        const std::string solver(p->solver);
        if (solver == "ED") throw Fail(ESC_ERR_PARAM, "Solver=ED (dense diagonalisation) is not provided on the GPU; use Solver=none");
        esc::build_lattice(*p, h->L);
        esc::build_bonds(*p, h->L, h->bonds);
        h->N = h->L.N;
        h->D = int64_t(1) << h->N;
        int T = 12, c = 3;
        if (const char* e = std::getenv("ESC_TILE_BITS")) T = std::atoi(e);
        if (const char* e = std::getenv("ESC_TILE_LOW")) c = std::atoi(e);
        install_plan(h.get(), esc::make_plan(h->N, bond_pairs(h.get()), T, c, 200), -1, 0);
        int ndev = 0;
        cudaError_t e = cudaGetDeviceCount(&ndev);
        if (e != cudaSuccess || ndev == 0) {
            (void)cudaGetLastError();
            throw Fail(ESC_ERR_CUDA, "no CUDA device available: this library has no CPU path");
        }
        ESC_CUDA(cudaGetDevice(&h->device));
        ESC_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        ensure_partials(h.get(), 4);
        if (!load_tuning(h.get())) {
            specialise(h.get(), h->passes);
            if (const char* e = std::getenv("ESC_AUTOTUNE"))
                if (std::atoi(e) == 1) autotune(h.get(), nullptr);
        }
    });
    if (st != ESC_OK) {
        g_err = h->err;
        esc_destroy(h.release());
        return st;
    }
    *out = h.release();
    return ESC_OK;
}

esc_status esc_autotune(esc_handle* h, char* report, size_t report_len) {
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    return guarded(h, [&]() {
        const std::string r = autotune(h, nullptr);
        if (report && report_len) {
            const size_t n = std::min(report_len - 1, r.size());
            std::memcpy(report, r.data(), n);
            report[n] = 0;
        }
    });
}

esc_status esc_destroy(esc_handle* h) {
    if (!h) return ESC_OK;
    for (void* p : {(void*)h->d_part, (void*)h->d_sc, h->d_L, h->d_work, h->d_gs, h->d_io, h->d_diag[0], h->d_diag[1],
                    h->d_cfb, (void*)h->d_cfs, (void*)h->d_cfi})
        if (p) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
    for (cudaStream_t x : {h->s_in, h->s_out})
        if (x) cudaStreamDestroy(x);
    for (int i = 0; i < 2; i++)
        for (cudaEvent_t e : {h->ev_in[i], h->ev_afree[i], h->ev_out[i], h->ev_outfree[i]})
            if (e) cudaEventDestroy(e);
    delete h;
    return ESC_OK;
}

int esc_num_sites(const esc_handle* h) { return h ? h->N : 0; }
int64_t esc_dim(const esc_handle* h) { return h ? h->D : 0; }
void* esc_stream(esc_handle* h) { return h ? (void*)h->stream : nullptr; }

esc_status esc_lattice(const esc_params* p, int* neigh, int* nsites) {
    if (!p) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    return guarded(nullptr, [&]() {
        esc::Lattice L;
        esc::build_lattice(*p, L);
        if (nsites) *nsites = L.N;
        if (neigh) std::memcpy(neigh, L.neigh.data(), L.neigh.size() * sizeof(int));
    });
}

esc_status esc_neighbors(const esc_handle* h, int* neigh) {
    if (!h || !neigh) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    std::memcpy(neigh, h->L.neigh.data(), h->L.neigh.size() * sizeof(int));
    return ESC_OK;
}

esc_status esc_basis_permutation(const esc_handle* h, int* bit_of_site) {
    if (!h || !bit_of_site) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    std::copy(h->plan.perm.begin(), h->plan.perm.end(), bit_of_site);
    return ESC_OK;
}

esc_status esc_hv(esc_handle* h, const void* in, void* out, esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (in == out) return finish(h, ESC_ERR_PARAM, "esc_hv: in and out must differ");
    return guarded(h, [&]() {
        Staged s = stage(h, in, out, 1, h->D, dt, flags);
        const void* dg = diag_for(h, dt);
        if (dt == ESC_C64) esc::launch_hv_tiled<float>(h->dm, h->passes, s.in, s.out, h->D, dg, h->stream);
        else esc::launch_hv_tiled<double>(h->dm, h->passes, s.in, s.out, h->D, dg, h->stream);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

}  // extern "C"

namespace {

// Host-buffer batch, pipelined: column c's host->device copy (stream s_in), its H.v with the
// permutations (handle stream) and its device->host copy (stream s_out) overlap with the
// neighbouring columns' -- the host link is full duplex, so column c+1 comes in while column c-1
// goes out.  Two slots of three vectors: A (copy in), B (internal-order input, later the
// reference-order result), C (internal-order result).  Events keep a slot's buffers from being
// refilled before their last reader is done.  Returns false (nothing done) when the 6 vectors do
// not fit.
template <typename R>
bool hv_host_pipelined(esc_handle* h, const char* in, char* out, int ncols, int64_t ld, const double* fields,
                       esc_dtype dt, bool internal) {
    const int64_t D = h->D;
    const size_t es = esize(dt), vb = (size_t)D * es;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); return false; }
    if (fr + h->io_bytes < 6 * vb + ((size_t)1 << 30)) return false;
    ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, 6 * vb));
    if (!h->s_in) ESC_CUDA(cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking));
    if (!h->s_out) ESC_CUDA(cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking));
    for (int i = 0; i < 2; i++)
        for (cudaEvent_t* e : {&h->ev_in[i], &h->ev_afree[i], &h->ev_out[i], &h->ev_outfree[i]})
            if (!*e) ESC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    const void* dg = diag_for(h, dt);
    // the copy streams start after the work already queued on the handle's stream
    ESC_CUDA(cudaEventRecord(h->ev_out[0], h->stream));
    ESC_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_out[0], 0));
    ESC_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_out[0], 0));
    for (int c = 0; c < ncols; c++) {
        const int s = c & 1;
        char* A = (char*)h->d_io + (size_t)(3 * s) * vb;
        char* B = A + vb;
        char* C = B + vb;
        const double* b = fields ? fields + 3 * c : nullptr;
        const esc::DevModel m = b ? model_with_field(h, b[0], b[1], b[2]) : h->dm;
        // copy in (slot's A free once column c-2 has read it)
        if (c >= 2) ESC_CUDA(cudaStreamWaitEvent(h->s_in, h->ev_afree[s], 0));
        ESC_CUDA(cudaMemcpyAsync(A, in + (size_t)c * ld * es, vb, cudaMemcpyHostToDevice, h->s_in));
        ESC_CUDA(cudaEventRecord(h->ev_in[s], h->s_in));
        // compute (slot's result buffer free once column c-2 has been copied out)
        ESC_CUDA(cudaStreamWaitEvent(h->stream, h->ev_in[s], 0));
        if (c >= 2) ESC_CUDA(cudaStreamWaitEvent(h->stream, h->ev_outfree[s], 0));
        const char* res;
        if (internal) {
            esc::launch_hv_tiled<R>(m, h->passes, A, C, D, dg, h->stream);
            ESC_CUDA(cudaEventRecord(h->ev_afree[s], h->stream));
            res = C;
        } else {
            permute(h, h->to_int, A, B, D, dt);
            ESC_CUDA(cudaEventRecord(h->ev_afree[s], h->stream));
            esc::launch_hv_tiled<R>(m, h->passes, B, C, D, dg, h->stream);
            permute(h, h->to_ref, C, B, D, dt);
            res = B;
        }
        ESC_CUDA(cudaEventRecord(h->ev_out[s], h->stream));
        // copy out
        ESC_CUDA(cudaStreamWaitEvent(h->s_out, h->ev_out[s], 0));
        ESC_CUDA(cudaMemcpyAsync(out + (size_t)c * ld * es, res, vb, cudaMemcpyDeviceToHost, h->s_out));
        ESC_CUDA(cudaEventRecord(h->ev_outfree[s], h->s_out));
    }
    ESC_CUDA(cudaStreamSynchronize(h->s_out));
    ESC_CUDA(cudaStreamSynchronize(h->s_in));
    sync(h);
    return true;
}

}  // namespace

extern "C" {

esc_status esc_hv_batched(esc_handle* h, const void* in, void* out, int ncols, int64_t ld, const double* fields,
                          esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (ncols < 1 || ncols > esc::MAX_COLS) return finish(h, ESC_ERR_PARAM, "ncols must be 1..16");
    if (ld < h->D) return finish(h, ESC_ERR_PARAM, "ld must be >= 2^N");
    return guarded(h, [&]() {
        esc::DevFields f;
        for (int c = 0; c < esc::MAX_COLS; c++) {
            const double* b = (fields && c < ncols) ? fields + 3 * c : nullptr;
            f.fx[c] = 0.5 * (b ? b[0] : h->p.Bxx);
            f.fy[c] = 0.5 * (b ? b[1] : h->p.Byy);
            f.fz[c] = 0.5 * (b ? b[2] : h->p.Bzz);
            f.fxf[c] = (float)f.fx[c]; f.fyf[c] = (float)f.fy[c]; f.fzf[c] = (float)f.fz[c];
        }
        if (!(flags & ESC_DEVICE_PTR) && ncols >= 2) {
            const bool internal = flags & ESC_INTERNAL_ORDER;
            const bool done = dt == ESC_C64
                                  ? hv_host_pipelined<float>(h, (const char*)in, (char*)out, ncols, ld, fields, dt, internal)
                                  : hv_host_pipelined<double>(h, (const char*)in, (char*)out, ncols, ld, fields, dt, internal);
            if (done) return;
        }
        Staged s = stage(h, in, out, ncols, ld, dt, flags);
        if (dt == ESC_C64) esc::launch_hv_batched<float>(h->dm, f, s.in, s.out, ncols, s.ld, h->D, h->stream);
        else esc::launch_hv_batched<double>(h->dm, f, s.in, s.out, ncols, s.ld, h->D, h->stream);
        unstage(h, s, out, ncols, ld, dt, flags);
    });
}

esc_status esc_apply_op(esc_handle* h, int op, int site, const void* in, void* out, esc_dtype dt, int flags) {
    if (!h || !in || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (in == out) return finish(h, ESC_ERR_PARAM, "esc_apply_op: in and out must differ");
    return guarded(h, [&]() {
        const esc::DevOp d = esc::make_dev_op(esc::operator_terms(op, site, h->p, h->L), &h->plan.perm);
        Staged s = stage(h, in, out, 1, h->D, dt, flags);
        if (dt == ESC_C64) esc::launch_apply<float>(d, s.in, s.out, h->D, h->stream);
        else esc::launch_apply<double>(d, s.in, s.out, h->D, h->stream);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

// Start vector into `dst` (device, internal order, normalised).  Generated in the reference basis
// order (the reference's draw order) and permuted; uses d_work as scratch.
static void start_vector_internal(esc_handle* h, int kind, int seed, void* dst, esc_dtype dt) {
    const int64_t D = h->D;
    // generation buffer: complex128 staging only for the host-generated reference start vector
    const size_t gbytes = (size_t)D * (kind == ESC_START_REFUNIFORM ? 16 : esize(dt));
    ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, gbytes));
    ensure_t(h->d_sc, h->sc_bytes, std::max<size_t>(h->sc_bytes, 64));
    void* gen = h->d_work;
    if (kind == ESC_START_REFUNIFORM) {
        std::vector<cplx> v((size_t)D);
        esc::ref_uniform_start(seed, D, v.data());
        ESC_CUDA(cudaMemcpyAsync(gen, v.data(), (size_t)D * 16, cudaMemcpyHostToDevice, h->stream));
        if (dt == ESC_C64) {
            esc::launch_convert_c128_to_c64(gen, dst, D, h->stream);
            ESC_CUDA(cudaMemcpyAsync(gen, dst, (size_t)D * 8, cudaMemcpyDeviceToDevice, h->stream));
        }
        sync(h);
    } else if (kind == ESC_START_NORMAL) {
        if (dt == ESC_C128) esc::launch_start_normal<double>((uint64_t)(int64_t)seed, gen, D, h->stream);
        else esc::launch_start_normal<float>((uint64_t)(int64_t)seed, gen, D, h->stream);
    } else {
        throw Fail(ESC_ERR_PARAM, "unknown start-vector kind");
    }
    permute(h, h->to_int, gen, dst, D, dt);
    if (dt == ESC_C128) { esc::launch_nrm2<double>(dst, D, h->d_part, h->d_sc, h->stream); esc::launch_scale_rsqrt<double>(dst, dst, h->d_sc, D, h->stream); }
    else { esc::launch_nrm2<float>(dst, D, h->d_part, h->d_sc, h->stream); esc::launch_scale_rsqrt<float>(dst, dst, h->d_sc, D, h->stream); }
}

esc_status esc_start_vector(esc_handle* h, int kind, int seed, void* out, esc_dtype dt, int flags) {
    if (!h || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    return guarded(h, [&]() {
        Staged s = stage(h, nullptr, out, 1, h->D, dt, flags);
        start_vector_internal(h, kind, seed, s.out, dt);
        unstage(h, s, out, 1, h->D, dt, flags);
    });
}

esc_status esc_lanczos_gs(esc_handle* h, const esc_lanczos_cfg* cfg, const void* start, int flags, double* E0,
                          double* alpha, double* beta, double* ritz, int* steps, void* gs_out) {
    if (!h || !cfg) return finish(h, ESC_ERR_PARAM, "null argument");
    if (cfg->steps < 2) return finish(h, ESC_ERR_PARAM, "LanczosSteps must be >= 2");
    if (cfg->lanctype < 0 || cfg->lanctype > 2) return finish(h, ESC_ERR_PARAM, "DynLanczosSolver: Use PsiOrAll==GS or All");
    return guarded(h, [&]() {
        const int64_t D = h->D;
        const esc_dtype dt = cfg->dtype;
        // start vector -> internal order in d_io[0]
        Staged s = stage(h, start, nullptr, 1, D, dt, flags);
        void* d_start = (void*)s.in;
        if (!start) {
            ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, (size_t)D * esize(dt)));
            d_start = h->d_io;
            start_vector_internal(h, h->p.start_vector, h->p.seed, d_start, dt);
        }
        if (dt == ESC_C64) lanczos_gs<float>(h, *cfg, d_start);
        else lanczos_gs<double>(h, *cfg, d_start);
        const int n = h->nsteps;
        if (steps) *steps = n;
        if (E0) *E0 = h->ritz[0];
        if (alpha) std::copy(h->alpha.begin(), h->alpha.end(), alpha);
        if (beta) std::copy(h->beta.begin(), h->beta.end(), beta);
        if (ritz) std::copy(h->ritz.begin(), h->ritz.end(), ritz);
        if (gs_out) {
            Staged g{nullptr, h->d_gs, D};
            unstage(h, g, gs_out, 1, D, dt, flags & ~ESC_ASYNC);
        }
        sync(h);
        if (h->d_io) {   // start vector and export staging are no longer needed: room for the dynamics
            cudaFree(h->d_io);
            h->d_io = nullptr;
            h->io_bytes = 0;
        }
    });
}

}  // extern "C"

namespace {

// Lehmann sum helpers (src/dynamics.h:277-316, :396-425, :133-187)
inline cplx lehmann_term(cplx a, cplx b, double w, double dE, double eta) { return std::conj(a) * b / cplx(w - dE, -eta); }

template <typename R>
void spectrum_impl(esc_handle* h, const esc_dyn_cfg& cfg, std::vector<double>& out, int& ncols) {
    Spectra<R> S(h);
    const int64_t D = h->D;
    const int N = h->N;
    const int nw = cfg.omega_steps + 1;
    const double eta = cfg.eta;
    const bool ritz = cfg.mode == ESC_DYNMODE_RITZ;
    const double Eg = h->ritz[0];
    const int M = h->nsteps;
    const int K = cfg.cf_steps > 0 ? cfg.cf_steps : M;
    ensure(h->d_work, h->work_bytes, (size_t)D * Pipe<R>::ES);   // one operator image at a time
    const size_t nsc = 2 * (size_t)std::max(M, 1) + 8 + 3 * (size_t)K + 8;
    ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, nsc * sizeof(double)));
    ensure_partials(h, std::max(M, 4));
    double* d_r = h->d_sc;
    double* d_tmp = d_r + 2 * std::max(M, 1);
    double* d_cf = d_tmp + 8;
    auto T = [&](int op, int site) { return esc::operator_terms(op, site, h->p, h->L); };
    auto omega = [&](int k) { return cfg.domega * k; };

    // CF resolvents G_A(omega) = <A gs|(z-H)^-1|A gs>, z = omega + E0 - i eta, for a list of
    // operators, run as columns of the batched CF Lanczos (batched.cu)
    // default complex128 head: 24 steps for JeJe, 48 for the larger-amplitude JsJs and local
    // spectra -- measured max |S_mixed - S_FP64| <= 3e-7 at N = 18, 24 (1000 CF steps, eta 0.05)
    const int head = cfg.fp64_head == 0 ? (cfg.kind == ESC_DYN_JEJE ? 24 : 48) : std::max(0, cfg.fp64_head);
    auto cf_runs = [&](const std::vector<std::vector<esc::OpTerm>>& ts) {
        std::vector<std::vector<cplx>> G(ts.size());
        const int width = cf_batch_width(h, Pipe<R>::ES, (int)ts.size());
        ensure(h->d_cfb, h->cfb_bytes, std::max(h->cfb_bytes, 3 * (size_t)width * D * Pipe<R>::ES));
        for (size_t r0 = 0; r0 < ts.size(); r0 += width) {
            const int nc = (int)std::min<size_t>(width, ts.size() - r0);
            char* set1 = (char*)h->d_cfb + (size_t)nc * D * Pipe<R>::ES;
            for (int c = 0; c < nc; c++)
                S.P.apply(esc::make_dev_op(ts[r0 + c], &h->plan.perm), h->d_gs, set1 + (size_t)c * D * Pipe<R>::ES);
            std::vector<int> steps(nc, K);
            std::vector<esc::DevModel> ms(nc, h->dm);
            std::vector<std::vector<double>> A, B;
            cf_batch_run<R>(h, nc, K, steps, ms, 1e-10, true, A, B, head);
            for (int c = 0; c < nc; c++) {
                std::vector<cplx> g(nw);
                for (int k = 0; k < nw; k++)
                    g[k] = esc::cf_eval(A[c].data(), B[c].data(), (int)A[c].size(), cplx(omega(k) + Eg, -eta));
                G[r0 + c] = g;
            }
        }
        return G;
    };
    auto cf_run = [&](const std::vector<esc::OpTerm>& t) { return cf_runs({t})[0]; };

    if (cfg.kind == ESC_DYN_JEJE || cfg.kind == ESC_DYN_JSJS) {
        const bool je = cfg.kind == ESC_DYN_JEJE;
        // channels: Je -> x, y, t = x+y ; Js -> x, y, z, t = x+y+z   (dynamics.h:365-367, :244-247)
        std::vector<std::vector<esc::OpTerm>> ch;
        if (je) {
            ch.push_back(T(ESC_OP_JEX_TOTAL, 0));
            ch.push_back(T(ESC_OP_JEY_TOTAL, 0));
            ch.push_back(combine(ch[0], ch[1], 1.0));
        } else {
            ch.push_back(T(ESC_OP_JSX_TOTAL, 0));
            ch.push_back(T(ESC_OP_JSY_TOTAL, 0));
            ch.push_back(T(ESC_OP_JSZ_TOTAL, 0));
            ch.push_back(combine(combine(ch[0], ch[1], 1.0), ch[2], 1.0));
        }
        const int nc = (int)ch.size();
        std::vector<cplx> el(nc);
        // pairs whose off-diagonal correlation the file needs
        std::vector<std::pair<int, int>> pairs = je ? std::vector<std::pair<int, int>>{{0, 1}}
                                                    : std::vector<std::pair<int, int>>{{0, 1}, {0, 2}, {1, 2}};
        // S[a][b][omega]
        std::vector<std::vector<std::vector<cplx>>> Sab(nc, std::vector<std::vector<cplx>>(nc, std::vector<cplx>(nw)));
        if (ritz) {
            std::vector<std::vector<cplx>> O(nc);
            for (int c = 0; c < nc; c++) O[c] = S.ritz_overlaps(ch[c], 0, d_r, d_tmp, &el[c]);
            for (int k = 0; k < nw; k++) {
                const double w = omega(k);
                for (int a = 0; a < nc; a++)
                    for (int b = 0; b < nc; b++) {
                        if (!(a == b || (a < 3 && b < 3))) continue;
                        cplx s(0, 0);
                        for (int n = 0; n < M; n++) s = s + lehmann_term(O[a][n], O[b][n], w, h->ritz[n] - Eg, eta);
                        Sab[a][b][k] = s;
                    }
            }
        } else {
            std::vector<std::vector<esc::OpTerm>> runs;
            for (int c = 0; c < nc; c++) {
                el[c] = S.expect(ch[c], 0, d_tmp);
                runs.push_back(ch[c]);
            }
            // per pair: the a+b and a+ib resolvents; for JeJe a+b is the total channel t = x+y itself
            std::vector<std::pair<int, int>> at;
            for (auto pr : pairs) {
                int ip = -1;
                if (je) ip = nc - 1;
                else { ip = (int)runs.size(); runs.push_back(combine(ch[pr.first], ch[pr.second], 1.0)); }
                at.push_back({ip, (int)runs.size()});
                runs.push_back(combine(ch[pr.first], ch[pr.second], cplx(0, 1)));
            }
            auto G = cf_runs(runs);
            for (int c = 0; c < nc; c++) Sab[c][c] = G[c];
            for (size_t q = 0; q < pairs.size(); q++) {
                const int a = pairs[q].first, b = pairs[q].second;
                const auto& Sp = G[at[q].first];
                const auto& Sq = G[at[q].second];
                for (int k = 0; k < nw; k++) {
                    const cplx X = Sp[k] - Sab[a][a][k] - Sab[b][b][k];
                    const cplx Y = Sq[k] - Sab[a][a][k] - Sab[b][b][k];
                    Sab[a][b][k] = 0.5 * (X - cplx(0, 1) * Y);
                    Sab[b][a][k] = 0.5 * (X + cplx(0, 1) * Y);
                }
            }
        }
        const int t = nc - 1;
        if (je) {
            ncols = 6;
            out.assign((size_t)nw * ncols, 0.0);
            for (int k = 0; k < nw; k++) {
                const cplx dn(omega(k), -eta);
                const cplx xx = Sab[0][0][k] - std::conj(el[0]) * el[0] / dn;
                const cplx xy = Sab[0][1][k] - std::conj(el[0]) * el[1] / dn;
                const cplx yy = Sab[1][1][k] - std::conj(el[1]) * el[1] / dn;
                const cplx yx = Sab[1][0][k];   // reference subtracts conj(Jey)*Jez[0] with Jez[0] never set (:368-369,424)
                const cplx tt = Sab[t][t][k] - std::conj(el[t]) * el[t] / dn;
                double* r = &out[(size_t)k * ncols];
                r[0] = omega(k); r[1] = xx.imag(); r[2] = yy.imag(); r[3] = xy.imag(); r[4] = yx.imag(); r[5] = tt.imag();
            }
        } else {
            ncols = 15;
            out.assign((size_t)nw * ncols, 0.0);
            const int ord[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};   // dynamics.h:318-323
            for (int k = 0; k < nw; k++) {
                const cplx dn(omega(k), -eta);
                double* r = &out[(size_t)k * ncols];
                r[0] = omega(k);
                for (int q = 0; q < 6; q++) {
                    const int a = ord[q][0], b = ord[q][1];
                    const cplx v = Sab[a][b][k] - std::conj(el[a]) * el[b] / dn;
                    r[1 + 2 * q] = v.real(); r[2 + 2 * q] = v.imag();
                }
                const cplx tt = Sab[t][t][k] - std::conj(el[t]) * el[t] / dn;
                r[13] = tt.real(); r[14] = tt.imag();
            }
        }
        return;
    }
    if (cfg.kind != ESC_DYN_LOCALSZSZ) throw std::invalid_argument("Unknown dynstr parameter");
    // LocalDynSzSz (dynamics.h:64-217): per site Sx, Sy, Sz, Sx+Sy+Sz, Spe3, Sme3
    ncols = 9;
    std::vector<cplx> acc((size_t)nw * 8, cplx(0, 0));
    const int ops[6] = {ESC_OP_SX, ESC_OP_SY, ESC_OP_SZ, ESC_OP_SXSYSZ, ESC_OP_SPE3, ESC_OP_SME3};
    for (int si = 0; si < N; si++) {
        std::vector<std::vector<esc::OpTerm>> ch(6);
        for (int c = 0; c < 6; c++) ch[c] = T(ops[c], si);
        std::vector<cplx> el(6);
        // Sab for (xx, yy, zz, xy, xz, yz, tt, pp, mm)
        std::vector<std::vector<cplx>> R9(9, std::vector<cplx>(nw));
        const int pa[9] = {0, 1, 2, 0, 0, 1, 3, 4, 5}, pb[9] = {0, 1, 2, 1, 2, 2, 3, 4, 5};
        if (ritz) {
            std::vector<std::vector<cplx>> O(6);
            for (int c = 0; c < 6; c++) O[c] = S.ritz_overlaps(ch[c], 0, d_r, d_tmp, &el[c]);
            for (int k = 0; k < nw; k++)
                for (int q = 0; q < 9; q++) {
                    cplx s(0, 0);
                    for (int n = 0; n < M; n++) s = s + lehmann_term(O[pa[q]][n], O[pb[q]][n], omega(k), h->ritz[n] - Eg, eta);
                    R9[q][k] = s;
                }
        } else {
            std::vector<std::vector<esc::OpTerm>> runs;
            for (int c = 0; c < 6; c++) {
                el[c] = S.expect(ch[c], 0, d_tmp);
                runs.push_back(ch[c]);
            }
            const int pp[3][3] = {{0, 1, 3}, {0, 2, 4}, {1, 2, 5}};
            for (auto& q : pp) {
                runs.push_back(combine(ch[q[0]], ch[q[1]], 1.0));
                runs.push_back(combine(ch[q[0]], ch[q[1]], cplx(0, 1)));
            }
            auto G = cf_runs(runs);   // 12 columns per site
            R9[0] = G[0]; R9[1] = G[1]; R9[2] = G[2]; R9[6] = G[3]; R9[7] = G[4]; R9[8] = G[5];
            for (int qi = 0; qi < 3; qi++) {
                const auto& q = pp[qi];
                const auto& Sp = G[6 + 2 * qi];
                const auto& Sq = G[7 + 2 * qi];
                for (int k = 0; k < nw; k++) {
                    const cplx X = Sp[k] - G[q[0]][k] - G[q[1]][k];
                    const cplx Y = Sq[k] - G[q[0]][k] - G[q[1]][k];
                    R9[q[2]][k] = 0.5 * (X - cplx(0, 1) * Y);
                }
            }
        }
        for (int k = 0; k < nw; k++) {
            const cplx dn(omega(k), -eta);
            cplx* A = &acc[(size_t)k * 8];
            for (int q = 0; q < 6; q++) A[q] += R9[q][k];
            A[6] += R9[7][k];
            A[7] += R9[8][k];
            A[0] -= std::conj(el[0]) * el[0] / dn; A[3] -= std::conj(el[0]) * el[1] / dn; A[4] -= std::conj(el[0]) * el[2] / dn;
            A[1] -= std::conj(el[1]) * el[1] / dn; A[5] -= std::conj(el[1]) * el[2] / dn; A[2] -= std::conj(el[2]) * el[2] / dn;
            A[6] -= el[5] * el[4] / dn;   // Sm*Sp without conjugate, as written (dynamics.h:185-186)
            A[7] -= el[4] * el[5] / dn;
        }
    }
    out.assign((size_t)nw * ncols, 0.0);
    for (int k = 0; k < nw; k++) {
        double* r = &out[(size_t)k * ncols];
        r[0] = omega(k);
        // data order: xx, yy, zz, xy, xz, yz, SmSp, SpSm (dynamics.h:189-196)
        for (int q = 0; q < 8; q++) r[1 + q] = acc[(size_t)k * 8 + q].imag();
    }
}

}  // namespace

namespace {

// Parameter-derivative operators dH/dK, dH/dJ, dH/dh (K the common Kitaev coupling, J the
// Heisenberg coupling, h the [111] field with Bxx=Byy=Bzz=-h/sqrt3), on relabelled sites.
void derivative_models(const esc_handle* h, esc::DevModel ms[3]) {
    esc_params pk = h->p, pj = h->p, ph = h->p;
    pk.Kxx = pk.Kyy = pk.Kzz = 1.0; pk.jheis = 0.0;
    pj.Kxx = pj.Kyy = pj.Kzz = 0.0; pj.jheis = 1.0;
    ph.Kxx = ph.Kyy = ph.Kzz = 0.0; ph.jheis = 0.0;
    const double s3 = -1.0 / std::sqrt(3.0);
    const esc_params* ps[3] = {&pk, &pj, &ph};
    for (int q = 0; q < 3; q++) {
        std::vector<esc::Bond> b;
        esc::build_bonds(*ps[q], h->L, b);
        for (auto& x : b) { x.i = h->plan.perm[x.i]; x.j = h->plan.perm[x.j]; }
        ms[q] = esc::make_dev_model(*ps[q], h->L, b, q == 2 ? s3 : 0.0, q == 2 ? s3 : 0.0, q == 2 ? s3 : 0.0);
    }
}

struct GradVecs {
    esc_handle* h;
    int64_t D;
    std::vector<void*> v;
    GradVecs(esc_handle* hh, int n) : h(hh), D(hh->D) {
        v.assign(n, nullptr);
        for (int i = 0; i < n; i++) {
            if (cudaMalloc(&v[i], (size_t)D * 16) != cudaSuccess) {
                (void)cudaGetLastError();
                for (int j = 0; j < i; j++) cudaFree(v[j]);
                v.clear();
                throw Fail(ESC_ERR_MEMORY, "gradient work vectors do not fit on the device");
            }
        }
    }
    ~GradVecs() { for (void* p : v) if (p) cudaFree(p); }
    void* operator[](int i) { return v[i]; }
};

cplx dotc(esc_handle* h, const void* a, const void* b) {
    esc::launch_dot<double>(a, b, h->D, h->d_part, h->d_sc, h->stream);
    double r[2];
    ESC_CUDA(cudaMemcpyAsync(r, h->d_sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    sync(h);
    return cplx(r[0], r[1]);
}
void axpby(esc_handle* h, const void* x, const void* y, void* out, cplx a, cplx b) {
    esc::launch_axpby<double>(x, y, out, a, b, h->D, h->stream);
}
void copyv(esc_handle* h, const void* x, void* y) {
    ESC_CUDA(cudaMemcpyAsync(y, x, (size_t)h->D * 16, cudaMemcpyDeviceToDevice, h->stream));
}

// Reverse sweep of G = b0^2/(z - a0 - b1^2/(z - a1 - ...)): dG/da_k, dG/db_k (k >= 0), dG/dz.
void cf_adjoint(const std::vector<double>& a, const std::vector<double>& b, cplx z, cplx& G, std::vector<cplx>& ga,
                std::vector<cplx>& gb, cplx& gz) {
    const int n = (int)a.size();
    std::vector<cplx> Dk(n);
    cplx t(0, 0);
    for (int k = n - 1; k >= 0; k--) {
        Dk[k] = z - a[k] - t;
        t = (k >= 1) ? (b[k] * b[k]) / Dk[k] : cplx(0, 0);
    }
    G = b[0] * b[0] / Dk[0];
    ga.assign(n, 0.0); gb.assign(n + 1, 0.0);
    gb[0] = 2.0 * b[0] / Dk[0];
    cplx g = -G / Dk[0];          // dG/dD_0
    gz = 0.0;
    for (int k = 0; k < n; k++) {
        ga[k] = -g;
        gz += g;
        if (k + 1 < n) {
            // D_k = z - a_k - b_{k+1}^2 / D_{k+1}
            gb[k + 1] = g * (-2.0 * b[k + 1] / Dk[k + 1]);
            g = g * (b[k + 1] * b[k + 1]) / (Dk[k + 1] * Dk[k + 1]);
        }
    }
}

void grad_impl(esc_handle* h, const esc_dyn_cfg* cfg, double* dE0, double* dS) {
    const int64_t D = h->D;
    ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)64 * sizeof(double)));
    ensure_partials(h, 4);
    esc::DevModel dm[3];
    derivative_models(h, dm);
    if (!dS) {
        // Hellmann-Feynman only (either precision)
        auto run = [&](auto tag) {
            typedef decltype(tag) R;
            ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, (size_t)D * Pipe<R>::ES));
            esc::launch_dot<R>(h->d_gs, h->d_gs, D, h->d_part, h->d_sc + 8, h->stream);
            for (int q = 0; q < 3; q++) {
                esc::launch_hv<R>(dm[q], h->d_gs, h->d_work, D, h->stream);
                esc::launch_dot<R>(h->d_gs, h->d_work, D, h->d_part, h->d_sc + 2 * q, h->stream);
            }
            double r[10];
            ESC_CUDA(cudaMemcpyAsync(r, h->d_sc, 10 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            sync(h);
            for (int q = 0; q < 3; q++) dE0[q] = r[2 * q] / r[8];
        };
        if (h->basis_dt == ESC_C64) run(float()); else run(double());
        return;
    }
    // ---- FP64 gradient of Im S_tt(omega) --------------------------------------------------------
    const bool je = cfg->kind == ESC_DYN_JEJE;
    if (!je && cfg->kind != ESC_DYN_JSJS) throw Fail(ESC_ERR_PARAM, "dS(omega) is provided for the JeJe and JsJs tt channels");
    const double K = h->p.Kxx;
    if (!(h->p.Kxx == h->p.Kyy && h->p.Kyy == h->p.Kzz) || K == 0.0)
        throw Fail(ESC_ERR_PARAM, "gradients are with respect to a common nonzero Kitaev coupling Kxx=Kyy=Kzz");
    const int steps = cfg->cf_steps > 0 ? cfg->cf_steps : h->nsteps;
    const int nw = cfg->omega_steps + 1;
    // vectors: 0 gs(normalised) 1 tmp 2..4 dH_q gs -> later dgs_q, 5..7 dphi_q, CG (8..11), Lanczos
    // q_prev 12, q 13, w 14, tangents dq_prev 15..17, dq 18..20, dw 21..23
    GradVecs V(h, 24);
    void* gs = V[0];
    copyv(h, h->d_gs, gs);
    const double ngs = std::sqrt(dotc(h, gs, gs).real());
    axpby(h, gs, gs, gs, cplx(1.0 / ngs, 0), cplx(0, 0));
    const double E0 = h->ritz[0];
    double dE[3];
    for (int q = 0; q < 3; q++) {
        esc::launch_hv<double>(dm[q], gs, V[2 + q], D, h->stream);
        dE[q] = dotc(h, gs, V[2 + q]).real();
        dE0[q] = dE[q];
    }
    auto Hv = [&](const void* in, void* out) {
        esc::launch_hv_tiled<double>(h->dm, h->passes, in, out, D, diag_for(h, ESC_C128), h->stream);
    };
    auto project = [&](void* x) {   // x -= <gs|x> gs
        const cplx c = dotc(h, gs, x);
        axpby(h, x, gs, x, cplx(1, 0), -c);
    };
    // Sternheimer: (H - E0) dgs = -(dH - dE) gs, dgs orthogonal to gs  (projected conjugate gradients)
    for (int q = 0; q < 3; q++) {
        void *x = V[8], *r = V[9], *p = V[10], *Ap = V[11];
        axpby(h, V[2 + q], gs, r, cplx(-1, 0), cplx(dE[q], 0));
        project(r);
        ESC_CUDA(cudaMemsetAsync(x, 0, (size_t)D * 16, h->stream));
        copyv(h, r, p);
        double rr = dotc(h, r, r).real();
        const double rr0 = rr;
        for (int it = 0; it < 3000 && rr > 1e-26 * rr0; it++) {
            Hv(p, Ap);
            axpby(h, Ap, p, Ap, cplx(1, 0), cplx(-E0, 0));
            project(Ap);
            const double pAp = dotc(h, p, Ap).real();
            if (!(pAp > 0)) break;
            const double al = rr / pAp;
            axpby(h, x, p, x, cplx(1, 0), cplx(al, 0));
            axpby(h, r, Ap, r, cplx(1, 0), cplx(-al, 0));
            const double rn = dotc(h, r, r).real();
            axpby(h, r, p, p, cplx(1, 0), cplx(rn / rr, 0));
            rr = rn;
        }
        project(x);
        copyv(h, x, V[2 + q]);   // dgs_q
    }
    // phi = A gs, dphi_q = (dA/dq) gs + A dgs_q; A homogeneous of degree 2 (Je) or 1 (Js) in K
    const esc::DevOp A = esc::make_dev_op(esc::operator_terms(je ? ESC_OP_JE_TOTAL : ESC_OP_JS_TOTAL, 0, h->p, h->L),
                                          &h->plan.perm);
    const double deg = je ? 2.0 : 1.0;
    void* phi = V[1];
    esc::launch_apply<double>(A, gs, phi, D, h->stream);
    for (int q = 0; q < 3; q++) esc::launch_apply<double>(A, V[2 + q], V[5 + q], D, h->stream);
    axpby(h, V[5], phi, V[5], cplx(1, 0), cplx(deg / K, 0));
    // elastic term m = <gs|A|gs> (real), dm_q = 2 Re <phi|dgs_q> + <gs|dA|gs>
    const double m = dotc(h, gs, phi).real();
    double dmel[3];
    for (int q = 0; q < 3; q++) dmel[q] = 2.0 * dotc(h, phi, V[2 + q]).real() + (q == 0 ? deg / K * m : 0.0);
    // tangent Lanczos on phi
    const double b0 = std::sqrt(dotc(h, phi, phi).real());
    double db0[3];
    for (int q = 0; q < 3; q++) db0[q] = dotc(h, phi, V[5 + q]).real() / b0;
    void *qp = V[12], *qc = V[13], *w = V[14];
    void* dqp[3] = {V[15], V[16], V[17]};
    void* dqc[3] = {V[18], V[19], V[20]};
    void* dw[3] = {V[21], V[22], V[23]};
    axpby(h, phi, phi, qc, cplx(1.0 / b0, 0), cplx(0, 0));
    for (int q = 0; q < 3; q++) {
        // dq0 = (dphi - db0 q0) / b0
        axpby(h, V[5 + q], qc, dqc[q], cplx(1.0 / b0, 0), cplx(-db0[q] / b0, 0));
        ESC_CUDA(cudaMemsetAsync(dqp[q], 0, (size_t)D * 16, h->stream));
    }
    ESC_CUDA(cudaMemsetAsync(qp, 0, (size_t)D * 16, h->stream));
    std::vector<double> a, b{b0}, da[3], db[3];
    for (int q = 0; q < 3; q++) db[q].push_back(db0[q]);
    void* tmp = V[8];
    for (int k = 0; k < steps; k++) {
        Hv(qc, w);                                   // w = H q
        const double ak = dotc(h, qc, w).real();
        double dak[3];
        for (int q = 0; q < 3; q++) {
            Hv(dqc[q], dw[q]);                       // dw = H dq + dH q
            esc::launch_hv<double>(dm[q], qc, tmp, D, h->stream);
            axpby(h, dw[q], tmp, dw[q], cplx(1, 0), cplx(1, 0));
            dak[q] = (dotc(h, dqc[q], w) + dotc(h, qc, dw[q])).real();
        }
        const double bk = b.back();
        // w = Hq - a q - b q_prev ; dw -= da q + a dq + db q_prev + b dq_prev
        axpby(h, w, qc, w, cplx(1, 0), cplx(-ak, 0));
        if (k > 0) axpby(h, w, qp, w, cplx(1, 0), cplx(-bk, 0));
        for (int q = 0; q < 3; q++) {
            axpby(h, dw[q], qc, dw[q], cplx(1, 0), cplx(-dak[q], 0));
            axpby(h, dw[q], dqc[q], dw[q], cplx(1, 0), cplx(-ak, 0));
            if (k > 0) {
                axpby(h, dw[q], qp, dw[q], cplx(1, 0), cplx(-db[q].back(), 0));
                axpby(h, dw[q], dqp[q], dw[q], cplx(1, 0), cplx(-bk, 0));
            }
        }
        a.push_back(ak);
        for (int q = 0; q < 3; q++) da[q].push_back(dak[q]);
        const double bn = std::sqrt(dotc(h, w, w).real());
        if (k + 1 == steps || !(bn > 1e-10 * b0)) break;
        double dbn[3];
        for (int q = 0; q < 3; q++) dbn[q] = dotc(h, w, dw[q]).real() / bn;
        b.push_back(bn);
        for (int q = 0; q < 3; q++) db[q].push_back(dbn[q]);
        // rotate: q_prev <- q, q <- w / bn ; dq_prev <- dq, dq <- (dw - dbn q_new) / bn
        std::swap(qp, qc);                            // qp = old q
        axpby(h, w, w, qc, cplx(1.0 / bn, 0), cplx(0, 0));
        for (int q = 0; q < 3; q++) {
            std::swap(dqp[q], dqc[q]);
            axpby(h, dw[q], qc, dqc[q], cplx(1.0 / bn, 0), cplx(-dbn[q] / bn, 0));
        }
    }
    // assemble d Im S_tt(omega) per parameter
    const double eta = cfg->eta;
    std::vector<cplx> ga, gb;
    for (int kw = 0; kw < nw; kw++) {
        const double om = cfg->domega * kw;
        const cplx z(om + E0, -eta);
        cplx G, gz;
        cf_adjoint(a, b, z, G, ga, gb, gz);
        const cplx dn(om, -eta);
        for (int q = 0; q < 3; q++) {
            cplx dG = gz * dE[q];
            for (size_t k = 0; k < a.size(); k++) dG += ga[k] * da[q][k];
            for (size_t k = 0; k < b.size() && k < gb.size(); k++) dG += gb[k] * db[q][k];
            const cplx del = 2.0 * m * dmel[q] / dn;
            dS[(size_t)kw * 3 + q] = (dG - del).imag();
        }
    }
    sync(h);
}

}  // namespace

namespace {

// Observables::TwoPointCorr (src/Observables.h:131-158): C(si, sj) = <gs| A_si B_sj |gs> for
// si >= sj, and C(sj, si) = the same value (the reference mirrors it without conjugation).
// GPU form: U_j = B_sj |gs> for all j; for a Hermitian A, Phi_i = A_si |gs> and one GEMV per
// column gives <Phi_i|U_j> for all i (2N operator applications instead of N(N+1)/2); otherwise
// A_si U_j is applied per pair and dotted with |gs>.  Falls back to the pairwise form when the
// 2N vectors do not fit in device memory.
bool hermitian_op(int op) {
    switch (op) {
        case ESC_OP_SP: case ESC_OP_SM: case ESC_OP_SPE3: case ESC_OP_SME3: return false;
        default: return true;
    }
}

template <typename R>
void two_point_impl(esc_handle* h, int opA, int opB, std::vector<cplx>& C) {
    Pipe<R> P(h);
    const int N = h->N;
    const int64_t D = h->D;
    const size_t ES = Pipe<R>::ES;
    auto T = [&](int op, int site) { return esc::make_dev_op(esc::operator_terms(op, site, h->p, h->L), &h->plan.perm); };
    C.assign((size_t)N * N, cplx(0, 0));
    ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)(2 * N + 8) * sizeof(double)));
    ensure_partials(h, N + 2);
    double* d_r = h->d_sc;
    std::vector<double> r(2 * (size_t)N);
    void* U = nullptr;
    void* Phi = nullptr;
    const bool herm = hermitian_op(opA);
    if (cudaMalloc(&U, (size_t)N * D * ES) != cudaSuccess || (herm && cudaMalloc(&Phi, (size_t)N * D * ES) != cudaSuccess)) {
        (void)cudaGetLastError();
        if (U) cudaFree(U);
        U = Phi = nullptr;
    }
    try {
        if (U && herm) {
            for (int j = 0; j < N; j++) P.apply(T(opB, j), h->d_gs, (char*)U + (size_t)j * D * ES);
            for (int i = 0; i < N; i++) P.apply(T(opA, i), h->d_gs, (char*)Phi + (size_t)i * D * ES);
            for (int j = 0; j < N; j++) {
                esc::launch_gemv_h<R>(Phi, D, N, (char*)U + (size_t)j * D * ES, D, h->d_part, part_cap_doubles(h), d_r,
                                      h->stream);
                ESC_CUDA(cudaMemcpyAsync(r.data(), d_r, r.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
                sync(h);
                for (int i = j; i < N; i++) C[(size_t)i * N + j] = C[(size_t)j * N + i] = cplx(r[2 * i], r[2 * i + 1]);
            }
        } else {
            ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, 2 * (size_t)D * ES));
            char* u = (char*)h->d_work;
            char* w = u + (size_t)D * ES;
            for (int j = 0; j < N; j++) {
                P.apply(T(opB, j), h->d_gs, u);
                for (int i = j; i < N; i++) {
                    P.apply(T(opA, i), u, w);
                    P.dot(h->d_gs, w, d_r);
                    double c[2];
                    ESC_CUDA(cudaMemcpyAsync(c, d_r, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
                    sync(h);
                    C[(size_t)i * N + j] = C[(size_t)j * N + i] = cplx(c[0], c[1]);
                }
            }
        }
    } catch (...) {
        (void)cudaStreamSynchronize(h->stream);
        if (U) cudaFree(U);
        if (Phi) cudaFree(Phi);
        throw;
    }
    sync(h);
    if (U) cudaFree(U);
    if (Phi) cudaFree(Phi);
}

}  // namespace

extern "C" {

esc_status esc_spectrum(esc_handle* h, const esc_dyn_cfg* cfg, double* out, int* nrows, int* ncols) {
    if (!h || !cfg) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (cfg->mode == ESC_DYNMODE_RITZ && !h->have_basis)
        return finish(h, ESC_ERR_STATE, "You need to set LancType=All for Dynamical calculations --- you dummy!");
    if (cfg->omega_steps < 0) return finish(h, ESC_ERR_PARAM, "omega_steps must be >= 0");
    if (!out) {   // size query: nothing is computed
        const int nc = cfg->kind == ESC_DYN_JEJE ? 6 : cfg->kind == ESC_DYN_JSJS ? 15 : cfg->kind == ESC_DYN_LOCALSZSZ ? 9 : 0;
        if (!nc) return finish(h, ESC_ERR_PARAM, "Unknown dynstr parameter");
        if (nrows) *nrows = cfg->omega_steps + 1;
        if (ncols) *ncols = nc;
        return finish(h, ESC_OK, "");
    }
    return guarded(h, [&]() {
        std::vector<double> s;
        int nc = 0;
        // Ritz mode runs in the precision of the ground state and its Krylov basis.  CF mode runs
        // in complex64 when either the ground state or cfg->dtype is complex64; a complex128
        // ground state is then rounded once to complex64 for the duration of the call.
        const esc_dtype dt = h->basis_dt;
        if (dt == ESC_C64) {
            spectrum_impl<float>(h, *cfg, s, nc);
        } else if (cfg->mode == ESC_DYNMODE_CF && cfg->dtype == ESC_C64) {
            void* g32 = nullptr;
            ESC_CUDA(cudaMalloc(&g32, (size_t)h->D * 8));
            esc::launch_convert_c128_to_c64(h->d_gs, g32, h->D, h->stream);
            void* g64 = h->d_gs;
            h->d_gs = g32;
            try {
                spectrum_impl<float>(h, *cfg, s, nc);
            } catch (...) {
                h->d_gs = g64;
                (void)cudaStreamSynchronize(h->stream);
                cudaFree(g32);
                throw;
            }
            h->d_gs = g64;
            sync(h);
            cudaFree(g32);
        } else {
            spectrum_impl<double>(h, *cfg, s, nc);
        }
        if (nrows) *nrows = cfg->omega_steps + 1;
        if (ncols) *ncols = nc;
        if (out) std::copy(s.begin(), s.end(), out);
    });
}

esc_status esc_two_point(esc_handle* h, int opA, int opB, double* out) {
    if (!h || !out) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    for (int op : {opA, opB})
        if (op < 0 || op > ESC_OP_JSXJSYJSZ) return finish(h, ESC_ERR_PARAM, "Unknown Operator label");
    return guarded(h, [&]() {
        std::vector<cplx> C;
        if (h->basis_dt == ESC_C64) two_point_impl<float>(h, opA, opB, C);
        else two_point_impl<double>(h, opA, opB, C);
        std::memcpy(out, C.data(), C.size() * sizeof(cplx));
    });
}

esc_status esc_measure_local(esc_handle* h, double* s_out, double* je_out) {
    if (!h) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    return guarded(h, [&]() {
        auto run = [&](auto tag) {
            typedef decltype(tag) R;
            Spectra<R> S(h);
            ensure(h->d_work, h->work_bytes, std::max(h->work_bytes, (size_t)h->D * Pipe<R>::ES));
            ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)16 * sizeof(double)));
            double* d_tmp = h->d_sc;
            for (int s = 0; s < h->N; s++) {
                if (s_out) {
                    const int ops[3] = {ESC_OP_SX, ESC_OP_SY, ESC_OP_SZ};
                    for (int c = 0; c < 3; c++) {
                        const cplx v = S.expect(esc::operator_terms(ops[c], s, h->p, h->L), 0, d_tmp);
                        s_out[(s * 3 + c) * 2] = v.real(); s_out[(s * 3 + c) * 2 + 1] = v.imag();
                    }
                }
                if (je_out) {
                    const int ops[2] = {ESC_OP_JEX, ESC_OP_JEY};
                    for (int c = 0; c < 2; c++) {
                        const cplx v = S.expect(esc::operator_terms(ops[c], s, h->p, h->L), 0, d_tmp);
                        je_out[(s * 2 + c) * 2] = v.real(); je_out[(s * 2 + c) * 2 + 1] = v.imag();
                    }
                }
            }
        };
        if (h->basis_dt == ESC_C64) run(float()); else run(double());
    });
}

esc_status esc_grad(esc_handle* h, const esc_dyn_cfg* cfg, double* dE0, double* dS) {
    if (!h || !dE0) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    if (dS && !cfg) return finish(h, ESC_ERR_PARAM, "dS needs a dynamics configuration");
    if (dS && h->basis_dt != ESC_C128) return finish(h, ESC_ERR_STATE, "dS(omega) gradients run in FP64: compute the ground state with ESC_C128");
    return guarded(h, [&]() { grad_impl(h, cfg, dE0, dS); });
}

}  // extern "C"

extern "C" esc_status esc_plan(const esc_params* p, int tile_bits, int low_bits, int* bit_of_site, int* npasses) {
    if (!p) return finish(nullptr, ESC_ERR_PARAM, "null argument");
    return guarded(nullptr, [&]() {
        esc::Lattice L;
        std::vector<esc::Bond> bonds;
        esc::build_lattice(*p, L);
        esc::build_bonds(*p, L, bonds);
        std::vector<std::pair<int, int>> pairs;
        for (const auto& b : bonds)
            if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
        esc::Plan P = esc::make_plan(L.N, pairs, tile_bits > 0 ? tile_bits : 12, low_bits > 0 ? low_bits : 3, 200);
        std::vector<esc::Bond> rb(bonds);
        for (auto& b : rb) { b.i = P.perm[b.i]; b.j = P.perm[b.j]; }
        const esc::DevModel m = esc::make_dev_model(*p, L, rb, p->Bxx, p->Byy, p->Bzz);
        const auto passes = esc::make_passes(P, m);   // throws if a term fits no tile
        if (bit_of_site) std::copy(P.perm.begin(), P.perm.end(), bit_of_site);
        if (npasses) *npasses = (int)passes.size();
    });
}

extern "C" esc_status esc_rayleigh(esc_handle* h, const void* v, esc_dtype dt, int flags, double* E) {
    if (!h || !E) return finish(h, ESC_ERR_PARAM, "null argument");
    if (!v && !h->have_gs) return finish(h, ESC_ERR_STATE, "no ground state: call esc_lanczos_gs first");
    return guarded(h, [&]() {
        // v == NULL: the handle's ground state, in place (no copy of the vector)
        if (!v) {
            dt = h->basis_dt;
            flags = ESC_DEVICE_PTR | ESC_INTERNAL_ORDER;
        }
        Staged s = stage(h, v ? v : h->d_gs, nullptr, 1, h->D, dt, flags);
        ensure_partials(h, 4);
        std::vector<double> num;
        const int maxb = esc::RED_MAX_BLOCKS;
        if (dt == ESC_C64) esc::launch_energy<float>(h->dm, h->passes, s.in, h->D, h->d_part, maxb, num, h->stream);
        else esc::launch_energy<double>(h->dm, h->passes, s.in, h->D, h->d_part, maxb, num, h->stream);
        ensure_t(h->d_sc, h->sc_bytes, std::max<size_t>(h->sc_bytes, 64));
        if (dt == ESC_C64) esc::launch_dot<float>(s.in, s.in, h->D, h->d_part, h->d_sc, h->stream);
        else esc::launch_dot<double>(s.in, s.in, h->D, h->d_part, h->d_sc, h->stream);
        double nn[2];
        ESC_CUDA(cudaMemcpyAsync(nn, h->d_sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        sync(h);
        *E = num[0] / nn[0];
    });
}

extern "C" esc_status esc_cf_batched(esc_handle* h, const esc_cf_batch_cfg* cfg, const void* starts, int64_t ld,
                                     int flags, double* a, double* b, int* lens) {
    if (!h || !cfg || !starts) return finish(h, ESC_ERR_PARAM, "null argument");
    if (cfg->ncols < 1 || cfg->ncols > esc::MAX_COLS) return finish(h, ESC_ERR_PARAM, "ncols must be 1..16");
    if (cfg->max_steps < 1) return finish(h, ESC_ERR_PARAM, "max_steps must be >= 1");
    if (ld < h->D) return finish(h, ESC_ERR_PARAM, "ld must be >= 2^N");
    return guarded(h, [&]() {
        const int nc = cfg->ncols, K = cfg->max_steps;
        const esc_dtype dt = cfg->dtype;
        const size_t es = esize(dt), vb = (size_t)h->D * es;
        ensure(h->d_cfb, h->cfb_bytes, std::max(h->cfb_bytes, 3 * (size_t)nc * vb));
        char* set1 = (char*)h->d_cfb + (size_t)nc * vb;
        for (int c = 0; c < nc; c++) {
            const char* src = (const char*)starts + (size_t)c * ld * es;
            const bool dev = flags & ESC_DEVICE_PTR, internal = flags & ESC_INTERNAL_ORDER;
            if (internal) {
                ESC_CUDA(cudaMemcpyAsync(set1 + c * vb, src, vb, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream));
            } else if (dev) {
                permute(h, h->to_int, src, set1 + c * vb, h->D, dt);
            } else {
                ensure(h->d_io, h->io_bytes, std::max(h->io_bytes, vb));
                ESC_CUDA(cudaMemcpyAsync(h->d_io, src, vb, cudaMemcpyHostToDevice, h->stream));
                permute(h, h->to_int, h->d_io, set1 + c * vb, h->D, dt);
            }
        }
        std::vector<int> steps(nc, K);
        if (cfg->steps)
            for (int c = 0; c < nc; c++) steps[c] = std::max(1, std::min(K, cfg->steps[c]));
        std::vector<esc::DevModel> ms(nc, h->dm);
        if (cfg->fields)
            for (int c = 0; c < nc; c++) ms[c] = model_with_field(h, cfg->fields[3 * c], cfg->fields[3 * c + 1], cfg->fields[3 * c + 2]);
        const double tol = cfg->tol > 0 ? cfg->tol : 1e-10;
        std::vector<std::vector<double>> A, B;
        if (dt == ESC_C64) cf_batch_run<float>(h, nc, K, steps, ms, tol, cfg->use_graph != 0, A, B);
        else cf_batch_run<double>(h, nc, K, steps, ms, tol, cfg->use_graph != 0, A, B);
        for (int c = 0; c < nc; c++) {
            if (lens) lens[c] = (int)A[c].size();
            if (a) for (size_t k = 0; k < A[c].size(); k++) a[(size_t)c * K + k] = A[c][k];
            if (b) for (size_t k = 0; k < B[c].size(); k++) b[(size_t)c * (K + 1) + k] = B[c][k];
        }
    });
}
