// LanczosCond.cpp -- drop-in replacement of the reference executable (main.cpp:41-202).
//
//   LanczosCond <inputfile>
//
// Reads the same Key=value input file, runs the ground-state Lanczos and the requested dynamics
// on the GPU through the C ABI (include/esc.h), prints the reference's log lines and writes
// JsJs_outSpectrum.real / JeJe_outSpectrum.real (and 2SSLocal_outSpectrum.real when the
// added key LocalSzSzDynamics=1 is set) into the working directory in the reference's format.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "esc.h"
#include "esc_internal.h"

typedef std::complex<double> dcomplex;

static void die(esc_handle* h, esc_status st, const char* where) {
    std::cerr << where << " failed (" << int(st) << "): " << esc_last_error(h) << std::endl;
    std::exit(1);
}

static void print_params(const esc_params& p) {
    std::cout << "____________________________________" << std::endl;
    std::cout << "NumberofSitesLx = " << p.Lx << "\nNumberofSitesLy = " << p.Ly << "\nRandomSeed = " << p.seed
              << "\nModel = " << p.model << "\nSolver = " << p.solver << "\nKxx = " << p.Kxx << "\nKyy = " << p.Kyy
              << "\nKzz = " << p.Kzz << "\nBxx = " << p.Bxx << "\nByy = " << p.Byy << "\nBzz = " << p.Bzz
              << "\nTemperature = " << p.temperature << "\nLanczosEps = " << p.lanczos_eps
              << "\nIsPeriodicX = " << p.pbcx << "\nIsPeriodicY = " << p.pbcy << "\nLancType = " << p.lanctype
              << "\nThreads = " << p.threads << "\nLanczosSteps = " << p.lanczos_steps << std::endl;
    if (p.jheis != 0.0) std::cout << "Jheis = " << p.jheis << std::endl;
    std::cout << "____________________________________" << std::endl << std::endl;
}

// Spectrum files in the reference's stream format (default precision 6, " \t " separators,
// rows ending in " \n "): src/dynamics.h:198-204, :325-328, :432-435.
static void write_spectrum(const char* fname, int kind, const std::vector<double>& s, int nrows, int ncols) {
    std::ofstream f(fname);
    for (int k = 0; k < nrows; k++) {
        const double* r = &s[(size_t)k * ncols];
        f << r[0] << " \t ";
        if (kind == ESC_DYN_JEJE) {
            for (int q = 1; q <= 4; q++) f << r[q] << " \t ";
            f << r[5];
        } else if (kind == ESC_DYN_JSJS) {
            for (int q = 1; q <= 12; q += 2) f << r[q] << " \t " << r[q + 1] << " \t ";
            f << r[13] << " \t " << r[14];
        } else {
            for (int q = 1; q <= 8; q++) f << r[q] << " \t ";
        }
        f << " \n ";
    }
}

// The reference's main after the ground state (main.cpp:92-202): local expectation values, then
// the dynamics the input file asks for, each written to its spectrum file.
static int run_observables_and_dynamics(esc_handle* h, const esc_params& p, bool measure, esc_dtype dtype) {
    const int N = esc_num_sites(h);
    esc_status st = ESC_OK;
    if (measure) {
        std::vector<dcomplex> s(3 * (size_t)N), je(2 * (size_t)N);
        const bool complete = std::string(p.model) == "Kitaev";
        st = esc_measure_local(h, (double*)s.data(), complete ? (double*)je.data() : nullptr);
        if (st != ESC_OK) die(h, st, "esc_measure_local");
        std::cout << "\n-------- measuring: site, <sx>, <sy>, <sz>, <spin_total>, <sp>, <sm> --------" << std::endl;
        const dcomplex I(0.0, 1.0);
        for (int si = 0; si < N; si++) {
            const dcomplex sx = s[3 * si], sy = s[3 * si + 1], sz = s[3 * si + 2];
            std::cout << si << " \t " << sx << " \t " << sy << " \t " << sz << " \t " << sx + sy + sz << " \t "
                      << sx + I * sy << " \t " << sx - I * sy << std::endl;
        }
        if (complete) {
            std::cout << "\n-------- measuring: site, <Je_xi>, <Je_yi>, <Je_zi>, <Je_total> --------" << std::endl;
            for (int si = 0; si < N; si++)
                std::cout << si << " \t " << je[2 * si] << " \t " << je[2 * si + 1] << " \t " << " \t "
                          << je[2 * si] + je[2 * si + 1] << std::endl;
        }
    }

    auto dyn = [&](int kind, const char* banner, const char* fname) {
        std::cout << " ==================================================================== " << std::endl;
        std::cout << banner << std::endl;
        std::cout << " ==================================================================== " << std::endl;
        esc_dyn_cfg dc{kind, p.dyn_mode, p.omega_steps, p.domega, p.eta,
                       p.dyn_lanczos_steps > 0 ? p.dyn_lanczos_steps : p.lanczos_steps, dtype};
        int nr = 0, nc = 0;
        esc_status s2 = esc_spectrum(h, &dc, nullptr, &nr, &nc);
        if (s2 != ESC_OK) die(h, s2, "esc_spectrum");
        std::vector<double> out((size_t)nr * nc);
        s2 = esc_spectrum(h, &dc, out.data(), &nr, &nc);
        if (s2 != ESC_OK) die(h, s2, "esc_spectrum");
        write_spectrum(fname, kind, out, nr, nc);
        std::cout << std::setprecision(8);
        const int every = kind == ESC_DYN_JEJE ? 1 : 200;
        for (int k = 0; k < nr; k += every) {
            for (int q = 0; q < nc; q++) std::cout << out[(size_t)k * nc + q] << " \t ";
            std::cout << " \n ";
        }
        std::cout << " " << std::endl << std::endl;
    };
    if (p.local_skw) dyn(ESC_DYN_JSJS, "                   Spin Dynamical Correlations		                   ", "JsJs_outSpectrum.real");
    if (p.energy_curr_dyn) dyn(ESC_DYN_JEJE, "              Energy Current Dynamical Correlations				   ", "JeJe_outSpectrum.real");
    if (p.local_szsz_dyn) dyn(ESC_DYN_LOCALSZSZ, "                 Local Spin Dynamical Correlations                  ", "2SSLocal_outSpectrum.real");
    esc_destroy(h);
    return 0;
}

int main(int argc, char* argv[]) {
    std::cout << "Hello, World!" << std::endl;
    if (argc != 2) throw std::invalid_argument("USE:: executable inputfile");
    std::cout << argv[1] << std::endl;
    esc_params p;
    char err[512];
    std::cout << "____________________________________" << std::endl;
    std::cout << " - Reading the inputfile: " << argv[1] << std::endl;
    if (esc_params_from_file(argv[1], &p, err, sizeof(err)) != ESC_OK) {
        std::cerr << err << std::endl;
        return 1;
    }
    print_params(p);
    esc_handle* h = nullptr;
    esc_status st = esc_create(&p, &h);
    if (st != ESC_OK) die(nullptr, st, "esc_create");
    const int N = esc_num_sites(h);
    const int64_t D = esc_dim(h);
    std::cout << "number of ket basis: " << D << std::endl;

    if (std::string(p.solver) == "ED") {
        // main.cpp:79-83: ExactDiag (src/Exactdiag.h:36-81) + fillFromED
        std::cout << "Begin Exact Diagonalization! --- " << std::endl;
        std::vector<double> ev((size_t)D);
        st = esc_exact_diag(h, ev.data(), nullptr, 0);
        if (st != ESC_OK) die(h, st, "esc_exact_diag");
        for (double x : ev) std::cout << x << ", ";
        std::cout << " Ground-state energy:= " << std::setprecision(16) << ev[0] << std::endl;
        std::cout << std::setprecision(8) << std::fixed;
        return run_observables_and_dynamics(h, p, true, ESC_C128);
    }
    const int M = p.lanczos_steps;
    const int lt = std::string(p.lanctype) == "OnlyEgs" ? 0 : std::string(p.lanctype) == "GS" ? 1 : 2;
    esc_lanczos_cfg cfg{M, p.lanczos_eps, lt, p.reortho, p.precision ? ESC_C64 : ESC_C128};
    std::vector<double> alpha(M), beta(M + 1), ritz(M);
    double E0 = 0;
    int steps = 0;
    std::cout << "Begin Lanczos! --- " << std::endl;
    st = esc_lanczos_gs(h, &cfg, nullptr, 0, &E0, alpha.data(), beta.data(), ritz.data(), &steps, nullptr);
    if (st != ESC_OK) die(h, st, "esc_lanczos_gs");
    // per-iteration lowest Ritz value (src/DynLanczosSolver.h:133-137), recomputed on the host
    double prev = 1.0, diff = 0.0, D0 = 0.0;
    for (int it = 1; it < steps; it++) {
        std::vector<double> d(alpha.begin(), alpha.begin() + it + 1), e(it + 1, 0.0);
        for (int i = 0; i < it; i++) e[i] = beta[i + 1];
        esc::tridiag_eig(it + 1, d, e, nullptr);
        D0 = d[0];
        diff = std::fabs(prev - D0);
        prev = D0;
        std::cout << it << " \t " << std::setprecision(16) << D0 << " \t  Eps: " << diff << std::endl;
    }
    std::cout << "  Lowest Eigen Value: " << E0 << std::endl;
    std::cout << "  With Lanczos EPS:   " << diff << std::endl;
    std::cout << "  Alpha and beta of Tridiag Matrix : ";
    for (int m = 0; m < steps; m++) std::cout << "(" << alpha[m] << "," << beta[m] << ") ";
    std::cout << std::endl << std::endl;
    std::cout << std::setprecision(6) << std::fixed << " Ritz values: ";
    for (int i = 0; i < steps; i++) std::cout << ritz[i] << " ";
    std::cout << std::endl;
    std::cout << std::setprecision(8) << std::fixed;

    return run_observables_and_dynamics(h, p, lt != 0, cfg.dtype);
}

