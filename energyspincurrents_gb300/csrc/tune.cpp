// tune.cpp -- the self-tuner of the complex64 H.v and its tuning file.
#include <array>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>

#include "abi_common.h"

namespace escabi {

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

// Slab pairs of a composite (passes picked from several variant sets): one specialised module for
// the composite, so that a pair kernel joins the two passes as they are; passes the tuner picked
// ahead of time stay ahead of time.
std::vector<esc::DevPass> with_pairs(const std::vector<esc::DevPass>& comp, int N) {
    std::vector<esc::DevPass> cp = comp;
    esc::mark_pairs(cp, N);
    bool jit = false;
    for (auto& p : cp) {
        jit = jit || p.jit >= 0;
        p.jit_pair = -1;
    }
    std::string err;
    if (jit && esc::jit_compile(cp, err))
        for (size_t i = 0; i < cp.size(); i++)
            if (comp[i].jit < 0) cp[i].jit = -1;
    // pairs without a kernel (e.g. the two passes chose different thread counts) run singly
    for (size_t i = 0; i + 1 < cp.size(); i++)
        if (cp[i].pair && !esc::pair_launchable(cp[i], cp[i + 1])) cp[i].pair = 0;
    return cp;
}
std::vector<esc::DevPass> without_pairs(const std::vector<esc::DevPass>& comp) {
    std::vector<esc::DevPass> cu = comp;
    for (auto& p : cu) {
        p.pair = 0;
        p.jit_pair = -1;
    }
    return cu;
}
bool has_pairs(const std::vector<esc::DevPass>& ps) {
    for (const auto& p : ps)
        if (p.pair) return true;
    return false;
}

void save_tuning(const esc_handle* h, int T, int balance, const std::vector<esc::DevPass>& ps) {
    const char* f = std::getenv("ESC_TUNE_FILE");
    if (!f || !*f) return;
    FILE* fp = std::fopen(f, "a");
    if (!fp) return;
    std::fprintf(fp, "%s | %d %d %d |", tune_key(h).c_str(), T, balance, (int)ps.size());
    for (const auto& p : ps) std::fprintf(fp, " %d,%d,%d", p.jit >= 0 ? 1 : 0, p.stages, p.tb_bits);
    std::fprintf(fp, " | %d | %d\n", h->cols_per_launch, has_pairs(ps) ? 1 : 0);
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
    int k = 0, pairs = 0;
    if (in >> bar >> k && bar == '|' && k >= 1 && k <= esc::MAX_COLS) h->cols_per_launch = k;
    if (!(in >> bar >> pairs) || bar != '|') pairs = 0;
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
    h->passes = pairs && h->dm.slab_sync ? with_pairs(comp, h->N) : without_pairs(comp);
    return true;
}

// The installed composite against the plan's ahead-of-time 512-thread kernel on one complex64
// vector: a tuned configuration must compute the same H.v (to complex64 rounding).  On a mismatch
// the handle returns to the plan and passes it had before tuning, and the report says so.
std::string verify_composite(esc_handle* h, const esc::Plan& plan, int balance, const esc::Plan& keep,
                             const std::vector<esc::DevPass>& keep_passes, bool& verified) {
    const int64_t D = h->D;
    void* buf = nullptr;
    ESC_CUDA(cudaMalloc(&buf, (size_t)D * 24));
    char* v = (char*)buf;
    char* a = v + (size_t)D * 8;
    char* b = a + (size_t)D * 8;
    esc::launch_start_normal<float>(4242, v, D, h->stream);
    const void* dg = diag_for(h, ESC_C64);
    const std::vector<esc::DevPass> ref = without_pairs(esc::make_passes(plan, h->dm, balance, 2, 9));
    esc::launch_hv_tiled<float>(h->dm, h->passes, v, a, D, dg, h->stream);
    esc::launch_hv_tiled<float>(h->dm, ref, v, b, D, dg, h->stream);
    std::vector<float> x((size_t)D * 2), y((size_t)D * 2);
    ESC_CUDA(cudaMemcpyAsync(x.data(), a, (size_t)D * 8, cudaMemcpyDeviceToHost, h->stream));
    ESC_CUDA(cudaMemcpyAsync(y.data(), b, (size_t)D * 8, cudaMemcpyDeviceToHost, h->stream));
    sync(h);
    cudaFree(buf);
    double dmax = 0.0, ymax = 0.0;
    for (size_t i = 0; i < x.size(); i++) {
        dmax = std::max(dmax, (double)std::fabs(x[i] - y[i]));
        ymax = std::max(ymax, (double)std::fabs(y[i]));
    }
    const double rel = dmax / std::max(ymax, 1e-300);
    std::ostringstream o;
    verified = rel <= 1e-5;
    if (!verified) {
        install_plan(h, keep, -1, 0);
        h->passes = keep_passes;
        o << "verification FAILED (relative difference " << rel << " against the ahead-of-time kernel): the "
          << "configuration before tuning is kept\n";
    } else {
        o << "verified against the ahead-of-time kernel: relative difference " << rel << "\n";
    }
    return o.str();
}

// Columns per launch of the multi-column H.V (batched recurrences): the installed passes applied
// to nb complex64 columns (as many as fit, at most 16) in launches of k = 1, 2, 4, ... columns; the
// k with the lowest time per column is kept (h->cols_per_launch).
std::string tune_columns(esc_handle* h) {
    const int64_t D = h->D;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { (void)cudaGetLastError(); return ""; }
    const size_t per = (size_t)D * 16;   // one complex64 column in and out
    const int nb = (int)std::min<size_t>(esc::MAX_COLS, fr > ((size_t)2 << 30) ? (fr - ((size_t)2 << 30)) / per : 0);
    if (nb < 2) return "columns: not timed (fewer than two columns fit)\n";
    void* buf = nullptr;
    ESC_CUDA(cudaMalloc(&buf, (size_t)nb * per));
    char* in = (char*)buf;
    char* out = in + (size_t)nb * D * 8;
    esc::launch_start_normal<float>(777, in, (int64_t)nb * D, h->stream);
    const void* dg = diag_for(h, ESC_C64);
    std::vector<esc::DevModel> ms(nb, h->dm);
    cudaEvent_t e0, e1;
    ESC_CUDA(cudaEventCreate(&e0));
    ESC_CUDA(cudaEventCreate(&e1));
    std::ostringstream rep;
    rep << "columns (" << nb << " complex64 columns):";
    std::vector<std::pair<int, double>> tk;
    for (int k = 1; k <= nb; k *= 2) {
        h->cols_per_launch = k;
        auto f = hv_all_columns<float>(h, ms, dg);
        f(in, out, nullptr, nullptr, h->stream);
        std::vector<float> ms3(3);
        for (float& x : ms3) {
            ESC_CUDA(cudaEventRecord(e0, h->stream));
            f(in, out, nullptr, nullptr, h->stream);
            ESC_CUDA(cudaEventRecord(e1, h->stream));
            ESC_CUDA(cudaEventSynchronize(e1));
            ESC_CUDA(cudaEventElapsedTime(&x, e0, e1));
        }
        std::sort(ms3.begin(), ms3.end());
        const double pc = ms3[1] / nb;
        rep << " k=" << k << " " << pc << " ms/column";
        tk.push_back({k, pc});
    }
    rep << "\n";
    // the most columns per launch whose time per column is within 0.5 % of the fastest (fewer launches)
    double best = 1e300;
    for (auto& x : tk) best = std::min(best, x.second);
    int bk = 1;
    for (auto& x : tk)
        if (x.second <= best * 1.005) bk = x.first;
    h->cols_per_launch = bk >= nb ? esc::MAX_COLS : bk;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return rep.str();
}

// Self-tuning of the complex64 H.v.  Plans: tile bits T in {11, 12, 13} (above 26 sites 12 and 13:
// 11 needs one pass more there) x first-fit / group-minimising
// term-to-pass assignment (make_passes modes 0 and 2; the balanced mode 1 never won).  Kernel variants per plan: ahead-of-time vs run-time specialised;
// 512, 256 or 128 threads per 4096-state tile (8, 16, 32 register states each), 1024, 512 or 256
// (the latter specialised only) per 8192-state tile (8, 16, 32); 2 or 3 tile buffers, or 2 plus staged
// epilogue loads (issued with the item, or one item ahead).  Every variant is timed pass by pass (CUDA events on the
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
            if (T > h->N || (h->N > 26 && T == 11)) continue;
            const esc::Plan plan = esc::make_plan(h->N, bond_pairs(h), T, 3, 200);
            for (int balance : {0, 2}) {
                std::vector<std::vector<esc::DevPass>> vars;
                std::vector<std::vector<double>> per;
                for (int tb : {10, 9, 8, 7})
                for (int stages : {2, 3, 4, 5})
                    for (int jit : {0, 1}) {
                        // 8192-state tiles: 1024 or 512 threads, or 256 specialised; 4096: 512 / 256 / 128
                        if (T == 13 && (tb == 7 || (tb == 8 && !jit))) continue;
                        if (T != 13 && tb == 10) continue;
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
                const std::vector<esc::DevPass> cu = without_pairs(comp);
                const double tc = median_ms(cu);
                rep << ": " << tc << " ms";
                if (tc < best) { best = tc; bplan = plan; bbal = balance; bT = T; bpasses = cu; }
                const std::vector<esc::DevPass> cp = h->dm.slab_sync ? with_pairs(comp, h->N) : cu;
                if (has_pairs(cp)) {
                    // the same composite with its slab pairs in one launch each
                    const double tp = median_ms(cp);
                    rep << ", slab pairs " << tp << " ms";
                    if (tp < best) { best = tp; bplan = plan; bbal = balance; bT = T; bpasses = cp; }
                }
                rep << "\n";
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
    bool verified = false;
    rep << verify_composite(h, bplan, bbal, keep, keep_passes, verified);
    rep << tune_columns(h);
    if (verified) save_tuning(h, bT, bbal, bpasses);
    rep << "chosen: T=" << bT << " balance=" << bbal << " passes:";
    for (const auto& ps : bpasses) rep << " " << (ps.jit >= 0 ? "jit" : "aot") << "/" << ps.stages << "/" << (1 << ps.tb_bits);
    if (has_pairs(bpasses)) {
        int np = 0;
        for (const auto& ps : bpasses) np += ps.pair ? 1 : 0;
        rep << " slab pairs " << np;
    }
    rep << " columns per launch " << h->cols_per_launch << " (" << best << " ms)\n";
    return rep.str();
}

}  // namespace escabi
