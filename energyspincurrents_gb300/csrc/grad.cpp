// grad.cpp -- parameter derivatives of E0 and of the CF spectra (an extension; no reference
// counterpart).
#include "abi_common.h"

namespace escabi {

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

// dH/dq on the tiled passes: the derivative model's terms assigned to the handle's plan (same
// site relabelling and tiles), with its own bond diagonal.
struct DerivOps {
    esc_handle* h;
    std::vector<esc::DevPass> passes[3];
    void* diag = nullptr;       // 3 x D entries of R
    size_t rsize = 8;
    DerivOps(esc_handle* hh, const esc::DevModel (&dm)[3], size_t r) : h(hh), rsize(r) {
        for (int q = 0; q < 3; q++) passes[q] = esc::make_passes(h->plan, dm[q], 0, 2, 9);
        if (cudaMalloc(&diag, 3 * (size_t)h->D * rsize) != cudaSuccess) {
            (void)cudaGetLastError();
            diag = nullptr;
            throw Fail(ESC_ERR_MEMORY, "derivative diagonals do not fit on the device");
        }
        for (int q = 0; q < 3; q++) {
            if (rsize == 8) esc::launch_diag<double>(dm[q], dq(q), h->D, h->stream);
            else esc::launch_diag<float>(dm[q], dq(q), h->D, h->stream);
        }
    }
    ~DerivOps() { if (diag) cudaFree(diag); }
    void* dq(int q) const { return (char*)diag + (size_t)q * h->D * rsize; }
    template <typename R>
    void hv(const esc::DevModel& m, int q, const void* in, void* out) const {
        esc::launch_hv_tiled<R>(m, passes[q], in, out, h->D, dq(q), h->stream);
    }
};

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
            const DerivOps ops(h, dm, sizeof(R));
            esc::launch_dot<R>(h->d_gs, h->d_gs, D, h->d_part, h->d_sc + 8, h->stream);
            for (int q = 0; q < 3; q++) {
                ops.hv<R>(dm[q], q, h->d_gs, h->d_work);
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
    const DerivOps ops(h, dm, 8);
    void* gs = V[0];
    copyv(h, h->d_gs, gs);
    const double ngs = std::sqrt(dotc(h, gs, gs).real());
    axpby(h, gs, gs, gs, cplx(1.0 / ngs, 0), cplx(0, 0));
    const double E0 = h->ritz[0];
    double dE[3];
    for (int q = 0; q < 3; q++) {
        ops.hv<double>(dm[q], q, gs, V[2 + q]);
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
        for (int it = 0; it < 20000 && rr > 1e-26 * rr0; it++) {
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
            ops.hv<double>(dm[q], q, qc, tmp);
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

}  // namespace escabi
