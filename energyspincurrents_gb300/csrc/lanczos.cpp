// lanczos.cpp -- the ground-state Lanczos (DynLanczosSolver::Lanczos_Nirav) and the batched
// continued-fraction recurrences on the device; the host keeps only scalars and the tridiagonal.
#include <functional>
#include <type_traits>

#include "abi_common.h"

namespace escabi {

// Columns of a CFBatch for the model list ms (one field per column) on the handle's passes, in
// launches of at most h->cols_per_launch columns (the self-tuner's choice; all by default).
template <typename RR>
std::function<int(const void*, void*, const int*, double*, cudaStream_t)> hv_all_columns(
        esc_handle* h, const std::vector<esc::DevModel>& ms, const void* dg) {
    esc::DevCols cols = esc::single_column(ms[0]);
    cols.ncols = (int)ms.size();
    cols.ld = h->D;
    for (size_t c = 0; c < ms.size(); c++) {
        cols.f.fx[c] = ms[c].fx; cols.f.fy[c] = ms[c].fy; cols.f.fz[c] = ms[c].fz;
        cols.f.fxf[c] = ms[c].fxf; cols.f.fyf[c] = ms[c].fyf; cols.f.fzf[c] = ms[c].fzf;
    }
    const esc::DevModel m0 = ms[0];
    const int k = std::max(1, std::min(h->cols_per_launch, esc::MAX_COLS));
    return [h, cols, m0, dg, k](const void* in, void* out, const int* active, double* part, cudaStream_t s) {
        int G = 0;
        for (int c0 = 0; c0 < cols.ncols; c0 += k) {
            esc::DevCols c = cols;
            c.ncols = std::min(k, cols.ncols - c0);
            c.col0 = c0;
            for (int i = 0; i < c.ncols; i++) {
                c.f.fx[i] = cols.f.fx[c0 + i]; c.f.fy[i] = cols.f.fy[c0 + i]; c.f.fz[i] = cols.f.fz[c0 + i];
                c.f.fxf[i] = cols.f.fxf[c0 + i]; c.f.fyf[i] = cols.f.fyf[c0 + i]; c.f.fzf[i] = cols.f.fzf[c0 + i];
            }
            c.dotp = part;
            const size_t off = (size_t)c0 * cols.ld * 2 * sizeof(RR);
            G = esc::launch_hv_cols<RR>(m0, c, h->passes, (const char*)in + off, (char*)out + off, h->D, dg, s,
                                        active ? active + c0 : nullptr);
        }
        return G;
    };
}

// Exit step of a run with LanczosEps > 0: the first iteration whose lowest Ritz value moved by
// less than eps (src/DynLanczosSolver.h:125-151), from the recorded coefficients.
static int exit_iteration(const std::vector<double>& a, const std::vector<double>& b, double eps) {
    const int M = (int)a.size();
    double E0 = 1.0;
    for (int iter = 1; iter < M; iter++) {
        std::vector<double> d(a.begin(), a.begin() + iter + 1), e(iter + 1, 0.0);
        for (int i = 0; i < iter; i++) e[i] = b[i + 1];
        if (!esc::tridiag_eig(iter + 1, d, e, nullptr)) throw Fail(ESC_ERR_NUMERIC, "diag: tridiagonal eigensolver failed");
        const double diff = std::fabs(E0 - d[0]);
        E0 = d[0];
        if (diff < eps) return iter;
    }
    return M - 1;
}

// Ground-state Lanczos, DynLanczosSolver::Lanczos_Nirav (src/DynLanczosSolver.h:38-239).
//
// Without reorthogonalisation (OnlyEgs, and GS / All with Reortho=0) the recurrence runs on the
// batched engine (batched.cu) with one column: unnormalised vectors u_k = beta_k v_k, alpha from
// the epilogue of the last H.v pass, the update fused with its norm, every iteration captured in a
// CUDA graph -- per step the H.v passes plus one streaming update, no separate dot or rescale
// sweeps.  Same alpha, beta and Ritz values as the normalised recurrence (mathematically; the
// rounding differs).  The run stops early only on beta = 0 or NaN, which are reported.
//   GS: three vectors; |gs> = sum_m Z(m,0) v_m rebuilt in a second sweep that regenerates the
//   vectors bit for bit (same kernels, same inputs) and accumulates them.
//   All: every u_k kept, rescaled to v_k afterwards (Ritz-mode spectra need the basis).
// With reorthogonalisation (the reference's mode) the normalised recurrence below runs as the
// reference does, with full Gram-Schmidt against every stored vector.
template <typename R>
void lanczos_gs(esc_handle* h, const esc_lanczos_cfg& cfg, const void* d_start) {
    Pipe<R> P(h);
    const int64_t D = h->D;
    const size_t ES = Pipe<R>::ES;
    const int M = cfg.steps;
    const bool recompute = cfg.lanctype == 1 && !cfg.reortho;
    const bool store = cfg.lanctype != 0 && !recompute;  // OnlyEgs keeps no basis (returns a zero vector)
    const bool reo = store && cfg.reortho;
    h->have_gs = h->have_basis = false;
    h->exact = false;
    if (!reo) {
        // ---- unnormalised recurrence on the batched engine --------------------------------------
        const size_t nd = (size_t)esc::CFB_GRID * 2 + (size_t)M * 2 + (size_t)(M + 1) + (size_t)(M + 2);
        ensure_t(h->d_cfs, h->cfs_bytes, std::max(h->cfs_bytes, nd * sizeof(double)));
        ensure_t(h->d_cfi, h->cfi_bytes, std::max(h->cfi_bytes, (size_t)4 * sizeof(int)));
        ensure(h->d_L, h->L_bytes, (size_t)(store ? M + 1 + 3 : 3) * D * ES);
        ensure_partials(h, 4);
        ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)16 * sizeof(double)));
        char* ring = (char*)h->d_L + (store ? (size_t)(M + 1) * D * ES : 0);   // 3 rotating vectors
        char* basis = (char*)h->d_L;                                             // All: u_0 .. u_M
        const void* dg = diag_for(h, sizeof(R) == 4 ? ESC_C64 : ESC_C128);
        const std::vector<esc::DevModel> ms{h->dm};
        double* zc = nullptr;
        auto make = [&](esc::CFBatch<R>& cb) {
            cb.ncols = 1; cb.kmax = M; cb.D = D; cb.tol = 0.0; cb.use_graph = true;
            cb.bufs = ring;
            cb.d_part = h->d_cfs;
            cb.d_alpha = cb.d_part + (size_t)esc::CFB_GRID * 2;
            cb.d_b2 = cb.d_alpha + (size_t)M * 2;
            zc = cb.d_b2 + (M + 1);
            cb.d_active = h->d_cfi;
            cb.d_steps = h->d_cfi + 1;
            cb.d_it = h->d_cfi + 2;
            cb.hv_all = hv_all_columns<R>(h, ms, dg);
        };
        // u_0 = normalised start, in the ring's set 1 (the engine's first "cur")
        auto load_start = [&]() {
            P.nrm2(d_start, h->d_sc);
            P.scale(d_start, ring + D * ES, h->d_sc);
        };
        ESC_CUDA(cudaMemsetAsync(h->d_cfs, 0, nd * sizeof(double), h->stream));
        ESC_CUDA(cudaMemcpyAsync(h->d_cfi + 1, &M, sizeof(int), cudaMemcpyHostToDevice, h->stream));
        esc::CFBatch<R> cb;
        make(cb);
        load_start();
        if (store) {
            ESC_CUDA(cudaMemcpyAsync(basis, ring + D * ES, D * ES, cudaMemcpyDeviceToDevice, h->stream));
            cb.after_update = [&](const void* w, cudaStream_t s) {
                esc::launch_store_iter<R>(w, basis, D, cb.d_it, cb.d_active, s);
            };
        }
        cb.run(h->stream);   // synchronises
        std::vector<double> al((size_t)M * 2), b2(M + 1);
        ESC_CUDA(cudaMemcpy(al.data(), cb.d_alpha, al.size() * sizeof(double), cudaMemcpyDeviceToHost));
        ESC_CUDA(cudaMemcpy(b2.data(), cb.d_b2, b2.size() * sizeof(double), cudaMemcpyDeviceToHost));
        std::vector<double> a, b{0.0};
        int n = 0;
        for (; n < M; n++) {
            a.push_back(al[2 * (size_t)n]);
            b.push_back(std::sqrt(b2[n + 1]));
            if (!std::isfinite(a.back()) || !std::isfinite(b.back()))
                throw Fail(ESC_ERR_NUMERIC, "NaN/Inf in Lanczos coefficients at step " + std::to_string(n));
            if (n + 1 < M && !(b.back() > 0.0))
                throw Fail(ESC_ERR_NUMERIC, "Lanczos breakdown: beta=0 at step " + std::to_string(n + 1) +
                                                " (Krylov space exhausted; use fewer LanczosSteps)");
        }
        const int nx = cfg.eps > 0.0 ? exit_iteration(a, b, cfg.eps) + 1 : M;   // EXITiter (:164)
        h->alpha.assign(a.begin(), a.begin() + nx);
        h->beta.assign(b.begin(), b.begin() + nx + 1);
        std::vector<double> d(h->alpha), e(nx, 0.0);
        for (int i = 0; i < nx - 1; i++) e[i] = h->beta[i + 1];
        h->Z.clear();
        if (!esc::tridiag_eig(nx, d, e, (store || recompute) ? &h->Z : nullptr))
            throw Fail(ESC_ERR_NUMERIC, "diag: tridiagonal eigensolver failed");
        h->ritz = d;
        h->nsteps = nx;
        ensure(h->d_gs, h->gs_bytes, (size_t)D * ES);
        if (recompute) {
            // second sweep: the same kernels on the same inputs regenerate u_0 .. u_{nx-1}; gs
            // accumulates Z(m,0) v_m = Z(m,0) / beta_m u_m  (beta_0 = |u_0| after normalisation)
            std::vector<double> z(nx);
            for (int m = 0; m < nx; m++) z[m] = h->Z[m] / std::sqrt(b2[m]);
            ESC_CUDA(cudaMemsetAsync(h->d_cfs, 0, nd * sizeof(double), h->stream));
            ESC_CUDA(cudaMemcpyAsync(zc, z.data(), nx * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            const int steps = nx - 1;
            esc::CFBatch<R> cb2;
            make(cb2);
            if (steps > 0) {
                ESC_CUDA(cudaMemcpyAsync(cb2.d_steps, &steps, sizeof(int), cudaMemcpyHostToDevice, h->stream));
                cb2.kmax = M;
            }
            load_start();
            ESC_CUDA(cudaMemsetAsync(h->d_gs, 0, (size_t)D * ES, h->stream));
            esc::launch_axpy_dev<R>(ring + D * ES, h->d_gs, zc, D, h->stream);
            if (steps > 0) {
                cb2.after_update = [&](const void* w, cudaStream_t s) {
                    esc::launch_accum_iter<R>(w, h->d_gs, D, cb2.d_it, zc, cb2.d_active, s);
                };
                cb2.run(h->stream);
            }
        } else if (store) {
            // v_m = u_m / beta_m (beta_m^2 = b2[m], on the device), then PsiAll[0] = sum_m v_m Z(m,0)
            for (int m = 0; m < nx; m++) {
                char* L = basis + (size_t)m * D * ES;
                P.scale(L, L, cb.d_b2 + m);
            }
            ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)(nx + 8) * sizeof(double)));
            double* d_z = h->d_sc;
            ESC_CUDA(cudaMemcpyAsync(d_z, h->Z.data(), nx * sizeof(double), cudaMemcpyHostToDevice, h->stream));
            esc::launch_lincomb<R>(basis, D, nx, d_z, h->d_gs, D, h->stream);
            h->have_basis = cfg.lanctype == 2;
        } else {
            ESC_CUDA(cudaMemsetAsync(h->d_gs, 0, (size_t)D * ES, h->stream));   // OnlyEgs returns zeros (:178-180)
        }
        if (recompute || store) {
            // the Lanczos vectors lose orthogonality once the ground state has converged, so the
            // sum is not a unit vector: normalise it
            P.nrm2(h->d_gs, h->d_sc + 3);
            P.scale(h->d_gs, h->d_gs, h->d_sc + 3);
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
        return;
    }
    // ---- normalised recurrence with full reorthogonalisation (the reference's mode) ---------------
    const int nvec = M + 1;
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
    ensure_partials(h, M + 2);
    ESC_CUDA(cudaMemsetAsync(h->d_sc, 0, n_sc * sizeof(double), h->stream));
    auto Lv = [&](int i) -> char* { return (char*)h->d_L + (size_t)i * D * ES; };
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
    if (!esc::tridiag_eig(n, d, e, &h->Z)) throw Fail(ESC_ERR_NUMERIC, "diag: tridiagonal eigensolver failed");
    h->ritz = d;
    h->nsteps = n;
    ensure(h->d_gs, h->gs_bytes, (size_t)D * ES);
    // PsiAll[0] = sum_m L_m Z(m,0) (:208-234), without forming the other Ritz vectors
    ESC_CUDA(cudaMemcpyAsync(d_z, h->Z.data(), n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    esc::launch_lincomb<R>(h->d_L, D, n, d_z, h->d_gs, D, h->stream);
    h->have_basis = cfg.lanctype == 2;
    h->basis_dt = sizeof(R) == 8 ? ESC_C128 : ESC_C64;
    h->L_ld = D;
    h->have_gs = true;
    sync(h);
}

// FP64 residual refinement of the handle's ground state (a complex64 ground state in particular):
// locally optimal conjugate-gradient steps (LOBPCG with one vector) in FP64.  Per step, with psi
// normalised: r = H psi - E psi, E = <psi|H psi> (tiled complex128 passes); p = the previous update
// direction, orthonormalised against psi and r^ = r/|r|; psi <- lowest Ritz vector of H on
// span{psi, r^, p^}.  In that basis <r^|H psi> = |r| and <p^|H psi> = 0, and <r^|H r^>, <p^|H p^> and
// the cross term <r^|H p^> (by polarisation, from r^ + p^ and r^ + i p^) come from the FP64 energy
// sweep, which forms no H v: three complex128 vectors in all.  A phase on p^ makes the 3x3 matrix
// real tridiagonal.  rnorm[s] = |r| before step s, rnorm[steps] after the last.  The refined vector
// replaces the handle's ground state (complex128 from then on; a Ritz basis no longer matches it)
// and its energy the lowest Ritz value.
void refine_gs(esc_handle* h, int steps, double* E_out, double* rnorm) {
    const int64_t D = h->D;
    void* psi = nullptr;
    void* r = nullptr;
    void* p = nullptr;
    // the complex64 ground state and the float diagonal make room for three complex128 vectors
    if (h->d_diag[1]) { cudaFree(h->d_diag[1]); h->d_diag[1] = nullptr; h->diag_bytes[1] = 0; }
    release_staging(h, 0);
    if (cudaMalloc(&psi, (size_t)D * 16) != cudaSuccess) {
        (void)cudaGetLastError();
        throw Fail(ESC_ERR_MEMORY, "refinement vectors do not fit on the device");
    }
    if (h->basis_dt == ESC_C64) esc::launch_convert_c64_to_c128(h->d_gs, psi, D, h->stream);
    else ESC_CUDA(cudaMemcpyAsync(psi, h->d_gs, (size_t)D * 16, cudaMemcpyDeviceToDevice, h->stream));
    sync(h);
    cudaFree(h->d_gs);
    h->d_gs = psi;   // from here on the ground state is complex128 (refined in place)
    h->gs_bytes = (size_t)D * 16;
    h->basis_dt = ESC_C128;
    h->have_basis = false;
    h->exact = false;
    if (cudaMalloc(&r, (size_t)D * 16) != cudaSuccess || cudaMalloc(&p, (size_t)D * 16) != cudaSuccess) {
        (void)cudaGetLastError();
        if (r) cudaFree(r);
        throw Fail(ESC_ERR_MEMORY, "refinement vectors do not fit on the device");
    }
    struct Free {
        void* a;
        void* b;
        ~Free() { cudaFree(a); cudaFree(b); }
    } guard{r, p};
    ensure_partials(h, 4);
    ensure_t(h->d_sc, h->sc_bytes, std::max(h->sc_bytes, (size_t)16 * sizeof(double)));
    Pipe<double> P(h);
    auto dot = [&](const void* a, const void* b) {
        double v[2];
        P.dot(a, b, h->d_sc);
        ESC_CUDA(cudaMemcpyAsync(v, h->d_sc, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        sync(h);
        return cplx(v[0], v[1]);
    };
    auto axpby = [&](const void* x, const void* y, void* out, cplx a, cplx b) {
        esc::launch_axpby<double>(x, y, out, a, b, D, h->stream);
    };
    auto sweep = [&](const void* v) {     // <v|H|v> in FP64, no H v formed
        std::vector<double> e;
        esc::launch_energy<double>(h->dm, h->passes, v, D, h->d_part, esc::RED_MAX_BLOCKS, e, h->stream);
        return e[0];
    };
    axpby(psi, psi, psi, cplx(1.0 / std::sqrt(dot(psi, psi).real()), 0), cplx(0, 0));
    double E = 0.0;
    bool have_p = false;
    for (int s = 0;; s++) {
        P.hv(psi, r);                                              // r = H psi
        E = dot(psi, r).real();
        axpby(r, psi, r, cplx(1, 0), cplx(-E, 0));                 // r -= E psi
        const double rho = std::sqrt(dot(r, r).real());
        if (rnorm) rnorm[s] = rho;
        if (s == steps || !(rho > 0.0)) {
            for (int q = s + 1; rnorm && q <= steps; q++) rnorm[q] = rho;
            break;
        }
        axpby(r, psi, r, cplx(1.0 / rho, 0), cplx(0, 0));          // r^
        axpby(r, psi, r, cplx(1, 0), -dot(psi, r));                // re-orthogonalise against psi
        axpby(r, psi, r, cplx(1.0 / std::sqrt(dot(r, r).real()), 0), cplx(0, 0));
        const double h22 = sweep(r);
        double h33 = 0.0, h23 = 0.0;
        cplx ph(1, 0);
        if (have_p) {
            axpby(p, psi, p, cplx(1, 0), -dot(psi, p));            // p^ orthonormal to psi and r^
            axpby(p, r, p, cplx(1, 0), -dot(r, p));
            const double np = std::sqrt(dot(p, p).real());
            have_p = np > 1e-14;
            if (have_p) {
                axpby(p, r, p, cplx(1.0 / np, 0), cplx(0, 0));
                h33 = sweep(p);
                axpby(p, r, p, cplx(1, 0), cplx(1, 0));            // r^ + p^
                const double s1 = sweep(p);
                axpby(p, r, p, cplx(0, 1), cplx(0, -1));           // i (r^ + p^) - i r^ = i p^ ... then + r^
                axpby(p, r, p, cplx(1, 0), cplx(1, 0));            // r^ + i p^
                const double s2 = sweep(p);
                axpby(p, r, p, cplx(0, -1), cplx(0, 1));           // -i (r^ + i p^) + i r^ = p^
                const cplx c23(0.5 * (s1 - h22 - h33), -0.5 * (s2 - h22 - h33));   // <r^|H p^>
                h23 = std::abs(c23);
                ph = h23 > 0.0 ? std::conj(c23) / h23 : cplx(1, 0);   // <r^|H (ph p^)> = |c23|
            }
        }
        // lowest Ritz pair of the real tridiagonal [[E, rho, 0], [rho, h22, h23], [0, h23, h33]]
        const int n = have_p ? 3 : 2;
        std::vector<double> d{E, h22, h33}, e{rho, h23, 0.0}, Z;
        d.resize(n);
        e.resize(n);
        if (!esc::tridiag_eig(n, d, e, &Z)) throw Fail(ESC_ERR_NUMERIC, "refinement: 3x3 eigensolver failed");
        double z1 = Z[0], z2 = Z[1], z3 = n == 3 ? Z[2] : 0.0;
        if (z1 < 0) { z1 = -z1; z2 = -z2; z3 = -z3; }
        // new direction p = z2 r^ + z3 ph p^, then psi <- z1 psi + p
        if (have_p) axpby(p, r, p, z3 * ph, cplx(z2, 0));
        else axpby(r, r, p, cplx(z2, 0), cplx(0, 0));
        axpby(psi, p, psi, cplx(z1, 0), cplx(1, 0));
        axpby(psi, psi, psi, cplx(1.0 / std::sqrt(dot(psi, psi).real()), 0), cplx(0, 0));
        have_p = true;
    }
    if (!h->ritz.empty()) h->ritz[0] = E;
    if (E_out) *E_out = E;
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
                  int head) {
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
        cb.hv_all = hv_all_columns<RR>(h, ms, dg);
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

template std::function<int(const void*, void*, const int*, double*, cudaStream_t)> hv_all_columns<float>(
        esc_handle*, const std::vector<esc::DevModel>&, const void*);
template std::function<int(const void*, void*, const int*, double*, cudaStream_t)> hv_all_columns<double>(
        esc_handle*, const std::vector<esc::DevModel>&, const void*);
template void lanczos_gs<float>(esc_handle*, const esc_lanczos_cfg&, const void*);
template void lanczos_gs<double>(esc_handle*, const esc_lanczos_cfg&, const void*);
template void cf_batch_run<float>(esc_handle*, int, int, const std::vector<int>&, const std::vector<esc::DevModel>&, double,
                                  bool, std::vector<std::vector<double>>&, std::vector<std::vector<double>>&, int);
template void cf_batch_run<double>(esc_handle*, int, int, const std::vector<int>&, const std::vector<esc::DevModel>&, double,
                                   bool, std::vector<std::vector<double>>&, std::vector<std::vector<double>>&, int);

}  // namespace escabi
