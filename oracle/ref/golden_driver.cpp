// Golden-vector driver: calls the reference's own, unmodified classes (compiled from the
// reference source tree) and dumps their results at full precision.  Test infrastructure only.
//
// usage: golden_driver <paramfile> <outdir> <testvector.bin>
//   The reference code runs with the CWD set to <outdir>, so its spectrum writers
//   (src/dynamics.h:121,267,386) create their files there.  `ofstream` is redirected to a
//   stream with precision 17 so that those files carry every digit.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include <omp.h>
#include <unistd.h>
#include <Eigen/Dense>
#include <unsupported/Eigen/CXX11/Tensor>

struct golden_ofstream : public std::ofstream {
    golden_ofstream() { this->precision(17); }
};
using namespace std;
#define ofstream golden_ofstream
#include "Memusage.h"
#include "Matrix.h"
#include "ParametersEngine.h"
#include "Lattice.h"
#include "QuantumBasis.h"
#include "Hamiltonian.h"
#include "Exactdiag.h"
#include "Observables.h"
#include "dynamics.h"
#undef ofstream

static void dump(const std::string& path, const void* p, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    fwrite(p, 1, bytes, f);
    fclose(f);
}

int main(int argc, char** argv) {
    if (argc != 4) { fprintf(stderr, "usage: %s params outdir testvec\n", argv[0]); return 2; }
    std::string pfile = argv[1], outdir = argv[2], tvfile = argv[3];
    ConstVariables P(pfile);
    omp_set_dynamic(0);
    omp_set_num_threads(P.Threads);
    Lattice Lat(P);
    QBasis Basis(P);
    Hamiltonian H(P, Lat, Basis);
    H.TightB_Ham();
    H.Diagonal();
    Observables Obs(P, Lat, Basis, H);
    DynLanczosSolver Lan(P, Basis, H);
    const int N = P.NumberofSites;
    const int D = (int)Basis.basis.size();
    if (chdir(outdir.c_str()) != 0) { perror("chdir"); return 2; }

    std::vector<int> nb(N * 3, -1);
    int ncol = (P.Model == "Kitaev") ? 3 : 2;
    for (int i = 0; i < N; i++) for (int c = 0; c < ncol; c++) nb[i * 3 + c] = Lat.N1neigh_(i, c);
    dump("neigh.bin", nb.data(), nb.size() * sizeof(int));
    // Current operators read neighbours of neighbours; on open clusters some are missing (-1) and
    // the reference would index out of range, so operators and dynamics run on complete tables only.
    bool complete = (P.Model == "Kitaev");
    for (int i = 0; i < N * ncol; i++) if (nb[(i / ncol) * 3 + i % ncol] < 0) complete = false;
    dump("hdiag.bin", H.HDiag.data(), H.HDiag.size() * sizeof(std::complex<double>));

    Eigen::VectorXcd x(D);
    {
        FILE* f = fopen(tvfile.c_str(), "rb");
        if (!f || fread(&x[0], sizeof(std::complex<double>), D, f) != (size_t)D) { fprintf(stderr, "testvec\n"); return 2; }
        fclose(f);
    }
    Eigen::VectorXcd hx = H.MatrixVectorMult(x);
    dump("hx.bin", &hx[0], D * sizeof(std::complex<double>));

    // operators on the test vector, every site where the operator is defined
    const char* ops[] = {"Sx", "Sy", "Sz", "Sp", "Sm", "Spe3", "Sme3", "Jsx", "Jsy", "Jsz", "Jex", "Jey",
                         "JexJeyJez", "JsxJsyJsz"};
    if (complete) {
        for (const char* op : ops) {
            std::vector<std::complex<double>> all((size_t)N * D);
            for (int s = 0; s < N; s++) {
                Eigen::VectorXcd o = Obs.ApplyOp(x, op, s);
                std::copy(o.d.begin(), o.d.end(), all.begin() + (size_t)s * D);
            }
            dump(std::string("op_") + op + ".bin", all.data(), all.size() * sizeof(std::complex<double>));
        }
        Eigen::VectorXcd t;
        t = Obs.ApplyJsxTotal(x); dump("op_JsxTotal.bin", &t[0], D * 16);
        t = Obs.ApplyJsyTotal(x); dump("op_JsyTotal.bin", &t[0], D * 16);
        t = Obs.ApplyJszTotal(x); dump("op_JszTotal.bin", &t[0], D * 16);
        t = Obs.ApplyJexTotal(x); dump("op_JexTotal.bin", &t[0], D * 16);
        t = Obs.ApplyJeyTotal(x); dump("op_JeyTotal.bin", &t[0], D * 16);
    }

    std::cout << "@@LANCZOS_BEGIN" << std::endl;
    Eigen::VectorXcd Psi = Lan.Lanczos_Nirav(P.LancType);
    std::cout << "@@LANCZOS_END" << std::endl;
    dump("ritz.bin", &Lan.TriDeval[0], Lan.TriDeval.size() * sizeof(double));
    dump("psi.bin", &Psi[0], D * sizeof(std::complex<double>));
    if (complete && P.LancType == "All") {
        Eigen::VectorXcd Sxi, Syi, Szi, Spi, Smi;
        std::cout << std::setprecision(17);
        Obs.measureLocalS(Psi, Sxi, Syi, Szi, Spi, Smi);
        std::vector<std::complex<double>> loc;
        for (int s = 0; s < N; s++) { loc.push_back(Sxi[s]); loc.push_back(Syi[s]); loc.push_back(Szi[s]); }
        dump("localS.bin", loc.data(), loc.size() * 16);
        // Observables::measureLocalJe (src/Observables.h:88-104) only prints: its lines (site,
        // <Je_x>, <Je_y>, total) are captured between markers at precision 17
        std::cout << "@@LOCALJE_BEGIN" << std::endl;
        Obs.measureLocalJe(Psi);
        std::cout << "@@LOCALJE_END" << std::endl;
        // Observables::TwoPointCorr (src/Observables.h:131-158), its commented drivers in main.cpp:118-183
        const char* pairs[][2] = {{"Sz", "Sz"}, {"Sx", "Sy"}, {"Sp", "Sm"}, {"Jsx", "Jsy"}, {"Jex", "Jey"}};
        for (auto& pr : pairs) {
            Eigen::MatrixXcd C = Obs.TwoPointCorr(pr[0], pr[1], Psi);
            std::vector<std::complex<double>> c;
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++) c.push_back(C(i, j));
            dump(std::string("corr_") + pr[0] + "_" + pr[1] + ".bin", c.data(), c.size() * 16);
        }
        std::string a = "Energy Current", b = "Spin Current", c = "LocalSzSz";
        StartDynamics(a, P, Lat, Basis, H, Lan, Psi);
        StartDynamics(b, P, Lat, Basis, H, Lan, Psi);
        StartDynamics(c, P, Lat, Basis, H, Lan, Psi);
    }
    return 0;
}
