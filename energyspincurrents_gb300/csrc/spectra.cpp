// spectra.cpp -- dynamical correlations (dynamics.h: DynJeJe, DynJsJs, LocalDynSzSz) in Ritz and
// continued-fraction modes, and Observables::TwoPointCorr.
#include "abi_common.h"

namespace escabi {

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

template void spectrum_impl<float>(esc_handle*, const esc_dyn_cfg&, std::vector<double>&, int&);
template void spectrum_impl<double>(esc_handle*, const esc_dyn_cfg&, std::vector<double>&, int&);
template void two_point_impl<float>(esc_handle*, int, int, std::vector<cplx>&);
template void two_point_impl<double>(esc_handle*, int, int, std::vector<cplx>&);

}  // namespace escabi
