// abi_common.h -- the handle behind the C ABI and the helpers that the implementation files
// (esc_abi.cpp, lanczos.cpp, spectra.cpp, grad.cpp, tune.cpp) share.  Internal: not installed.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "esc_internal.h"

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
    int cols_per_launch = esc::MAX_COLS;   // columns per multi-column H.V launch (self-tuner's choice)
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
    unsigned* slab_sync = nullptr;                     // slab-pair error flag + counters (DevModel::slab_sync)
    unsigned long long slab_seen = 0;                  // slab-pair launches seen at the last check
    void* d_diag[2] = {nullptr, nullptr};              // diagonal of the bond terms per dtype
    size_t diag_bytes[2] = {0, 0};
    // ground-state Lanczos results
    int nsteps = 0;
    bool have_gs = false, have_basis = false;
    bool exact = false;   // the basis holds exact eigenvectors (Solver=ED): Ritz overlaps need no Z
    esc_dtype basis_dt = ESC_C128;
    int64_t L_ld = 0;
    std::vector<double> alpha, beta, ritz, Z;
};

namespace escabi {

using esc::cplx;

struct Fail : std::runtime_error {
    esc_status st;
    Fail(esc_status s, const std::string& m) : std::runtime_error(m), st(s) {}
};

// Records msg as the last error (per thread and on the handle) and returns st.
esc_status finish(esc_handle* h, esc_status st, const std::string& msg);

// Runs f, mapping exceptions to status codes: nothing throws across the C ABI.
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

size_t esize(esc_dtype dt);
bool bad_dtype(int dt);   // not ESC_C128 / ESC_C64
void ensure(void*& p, size_t& cap, size_t need);
template <typename T>
void ensure_t(T*& p, size_t& cap, size_t need) {
    void* q = p;
    ensure(q, cap, need);
    p = (T*)q;
}

void sync(esc_handle* h);
const void* diag_for(esc_handle* h, esc_dtype dt);
void ensure_partials(esc_handle* h, int rows);
int64_t part_cap_doubles(esc_handle* h);
void permute(esc_handle* h, const esc::DevPerm& p, const void* in, void* out, int64_t n, esc_dtype dt);

// Staged input/output (esc_abi.cpp): kernels work in the internal basis order.
struct Staged {
    const void* in;
    void* out;
    int64_t ld;
};
Staged stage(esc_handle* h, const void* in, void* out, int cols, int64_t ld, esc_dtype dt, int flags);
void unstage(esc_handle* h, const Staged& s, void* out, int cols, int64_t ld, esc_dtype dt, int flags);
void release_staging(esc_handle* h, size_t keep);

esc::DevModel model_with_field(const esc_handle* h, double bx, double by, double bz);
std::vector<std::pair<int, int>> bond_pairs(const esc_handle* h);
void install_plan(esc_handle* h, const esc::Plan& plan, int balance, int stages, int tb_bits = 0);
void specialise(esc_handle* h, std::vector<esc::DevPass>& passes, int force = -1);
void start_vector_internal(esc_handle* h, int kind, int seed, void* dst, esc_dtype dt);

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


// lanczos.cpp
template <typename R> void lanczos_gs(esc_handle* h, const esc_lanczos_cfg& cfg, const void* d_start);
void refine_gs(esc_handle* h, int steps, double* E, double* rnorm);
// exactdiag.cpp
void exact_diag(esc_handle* h);
template <typename RR>
std::function<int(const void*, void*, const int*, double*, cudaStream_t)> hv_all_columns(
        esc_handle* h, const std::vector<esc::DevModel>& ms, const void* dg);
int cf_batch_width(esc_handle* h, size_t es, int want);
template <typename R>
void cf_batch_run(esc_handle* h, int ncols, int kmax, const std::vector<int>& steps, const std::vector<esc::DevModel>& ms,
                  double tol, bool graph, std::vector<std::vector<double>>& A, std::vector<std::vector<double>>& B,
                  int head = 0);

// ---------------------------------------------------------------------------------------------
// Spectra
// ---------------------------------------------------------------------------------------------
struct Grid {
    int nw;
    double dw, eta;
};

// One operator "channel": a combination of operator strings applied to |gs>.
inline std::vector<esc::OpTerm> combine(const std::vector<esc::OpTerm>& a, const std::vector<esc::OpTerm>& b, cplx cb) {
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
            if (h->exact) { O[n] = cplx(r[2 * n], r[2 * n + 1]); continue; }   // eigenvectors themselves
            cplx s(0, 0);
            for (int m = 0; m < M; m++) s += h->Z[(size_t)n * M + m] * cplx(r[2 * m], r[2 * m + 1]);
            O[n] = s;
        }
        return O;
    }
};

// spectra.cpp
template <typename R> void spectrum_impl(esc_handle* h, const esc_dyn_cfg& cfg, std::vector<double>& out, int& ncols);
template <typename R> void two_point_impl(esc_handle* h, int opA, int opB, std::vector<cplx>& C);
// grad.cpp
void grad_impl(esc_handle* h, const esc_dyn_cfg* cfg, double* dE0, double* dS);
// tune.cpp
bool load_tuning(esc_handle* h);
std::string autotune(esc_handle* h, std::vector<double>* times);

}  // namespace escabi
