// esc_oracle.cpp -- CPU restatement of the reference Lanczos exact-diagonalisation path.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library: only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it. Nothing in the
// product (energyspincurrents_gb300/, include/) links, loads or calls it.
//
// Every routine restates one piece of fengshi96/EnergySpinCurrents and cites the file:line
// it follows.  Structure deliberately mirrors the reference (COO lists + OpenMP scatter with
// per-thread output copies, sequential Gram-Schmidt, explicit Ritz vectors), so that the
// oracle's rounding behaviour is that of the reference algorithm, not of the GPU design.
//
// Extensions that the reference does not have (Heisenberg J on every nearest-neighbour bond,
// continued-fraction spectra, a matrix-free gather for large N) are marked "EXTENSION".
//
// Build: g++ -O2 -fopenmp -shared -fPIC (see oracle/build_oracle.py).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>
#include <omp.h>

typedef std::complex<double> cplx;
typedef std::complex<float> cplxf;

// ---------------------------------------------------------------------------------------------
// Lattice.  Honeycomb1: src/Lattice.h:434-576.  Chain: src/Lattice.h:60-195.
// neigh is N x ncol row-major; honeycomb columns are 0=z, 1=y, 2=x (src/Lattice.h:497-522).
// ---------------------------------------------------------------------------------------------
struct OrLattice {
    int N = 0, ncol = 0;
    std::vector<int> neigh, indx, indy;
};

static void honeycomb1(int Lx, int Ly, bool pbcx, bool pbcy, OrLattice& L) {
    const int N = Lx * Ly;
    const int LLX = Lx, LLY = Ly / 2;                         // src/Lattice.h:437-438
    L.N = N; L.ncol = 3;
    L.neigh.assign(N * 3, -1);
    L.indx.assign(N, 0); L.indy.assign(N, 0);
    const double scalex = 2.0, scaley = 4.0 / std::sqrt(3.0);  // :441
    double t1x = 1.0 * scalex;                                 // :443
    double t2x = 0.5 * scalex, t2y = std::sqrt(3.0) / 2.0 * scaley;  // :450-451 ("right")
    const int ncr = LLX * 2 + LLY, ncc = LLY * 2;              // Nc_ is (2LLX+LLY) x 2LLY, :457
    std::vector<int> Nc(ncr * ncc, -1);
    auto nc = [&](int x, int y) -> int {
        // The reference indexes a column-major Matrix<int> without lower-bound checks.
        // All indices reached by Honeycomb1 on valid lattices are in range; out-of-range
        // reads are treated as "no site".
        if (x < 0 || y < 0 || x >= ncr || y >= ncc) return -1;
        return Nc[x + y * ncr];
    };
    int xv = 0, counter = 0;
    for (int i = 0; i < LLX; i++) {                            // :461-486
        if (i == 0) xv = 0; else xv = int(xv + t1x);
        int x0 = xv, y0 = 0, x1 = int(xv + 1.0), y1 = 1;
        for (int j = 0; j < LLY; j++) {
            int cxa = int(x0 + j * t2x), cxb = int(x1 + j * t2x);
            int cya = int(y0 + j * t2y), cyb = int(y1 + j * t2y);
            L.indx[counter] = cxa; L.indy[counter] = cya; Nc[cxa + cya * ncr] = counter; counter++;
            L.indx[counter] = cxb; L.indy[counter] = cyb; Nc[cxb + cyb * ncr] = counter; counter++;
        }
    }
    int xmax = *std::max_element(L.indx.begin(), L.indx.end());
    int ymax = *std::max_element(L.indy.begin(), L.indy.end());
    auto setn = [&](int i, int j, int c) { L.neigh[i * 3 + c] = j; L.neigh[j * 3 + c] = i; };
    for (int i = 0; i < N; i++) {                              // :493-565
        int ix = L.indx[i], iy = L.indy[i];
        int jx = ix + 1, jy = iy + 1;                          // x bond, column 2
        if (jx < xmax + 1 && jy < ymax + 1 && nc(jx, jy) != -1) setn(i, nc(jx, jy), 2);
        jx = ix + 1; jy = iy - 1;                              // y bond, column 1
        if (jx < xmax + 1 && jy < ymax && jy >= 0 && nc(jx, jy) != -1) setn(i, nc(jx, jy), 1);
        jx = ix; jy = iy + 1;                                  // z bond, column 0
        if (jx < xmax && jy < ymax + 1 && nc(jx, jy) != -1) setn(i, nc(jx, jy), 0);
        if (pbcy) {                                            // :530-537
            jx = ix - LLY; jy = 0;
            if (jx < xmax && iy == ymax && nc(jx, jy) != -1) setn(i, nc(jx, jy), 0);
        }
        if (pbcx && iy % 2 == 0 && nc(ix, iy) < LLY * 2) {     // :548-555
            jx = ix + LLX * 2 - 1; jy = iy + 1;
            if (jx < xmax + 1 && iy < ymax + 1 && nc(jx, jy) != -1) setn(i, nc(jx, jy), 1);
        }
    }
}

static void chain(int N, bool pbcx, OrLattice& L) {          // src/Lattice.h:60-136 (N1neigh only)
    L.N = N; L.ncol = 2;
    L.neigh.assign(N * 2, -1);
    L.indx.resize(N); L.indy.assign(N, 0);
    for (int i = 0; i < N; i++) L.indx[i] = i;
    for (int i = 0; i < N; i++) {
        if (i + 1 < N) L.neigh[i * 2 + 0] = i + 1;
        if (i - 1 > -1) L.neigh[i * 2 + 1] = i - 1;
        if (pbcx) {
            if (i == N - 1) L.neigh[i * 2 + 0] = 0;
            if (i == 0) L.neigh[i * 2 + 1] = N - 1;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Model: connectors (src/Hamiltonian.h:230-328, HeisenbergChain :382-475), COO lists
// (TightB_Ham :94-206), diagonal (Diagonal :331-377), H.v (MatrixVectorMult :480-557).
// ---------------------------------------------------------------------------------------------
struct Bond { int i, j; double k; };

struct OrModel {
    int N = 0; int64_t D = 0; int threads = 1;
    bool kitaev = true;
    double Kxx = 0, Kyy = 0, Kzz = 0, Bxx = 0, Byy = 0, Bzz = 0, J = 0;
    OrLattice lat;
    std::vector<Bond> xb, yb, zb;      // reference connector lists (value = coupling)
    std::vector<Bond> nn;              // EXTENSION: every nearest-neighbour bond once (for J)
    bool coo = false;
    std::vector<int64_t> Sxx_init, Sxx_final, Syy_init, Syy_final;
    std::vector<cplx> HTSxx, HTSyy, HDiag;
    // results of the last ground-state Lanczos (src/DynLanczosSolver.h:33-35)
    std::vector<double> TriDeval;
    std::vector<double> TrEVec;        // n x n column-major, real (eigenvectors of the real tridiagonal)
    std::vector<cplx> alpha, beta;
    std::vector<cplx> PsiAll;          // nPsi x D
    int nPsi = 0;
    std::vector<cplx> Psi;
};

static inline int findBit(int64_t k, int s) { return int((k >> s) & 1); }

static void connectors(OrModel& m) {
    const OrLattice& L = m.lat;
    const int N = L.N;
    // Dense N x N coupling matrices as in the reference; scanned row-major for the bond order.
    std::vector<double> kx(N * N, 0.0), ky(N * N, 0.0), kz(N * N, 0.0);
    if (m.kitaev) {
        for (int i = 0; i < N; i++) {                          // :239-264
            int j = L.neigh[i * 3 + 0]; if (i < j) kz[i * N + j] = m.Kzz;
            j = L.neigh[i * 3 + 2];     if (i < j) kx[i * N + j] = m.Kxx;
            j = L.neigh[i * 3 + 1];     if (i < j) ky[i * N + j] = m.Kyy;
        }
    } else {
        for (int i = 0; i < N; i++) {                          // :392-414
            for (int c = 0; c < 2; c++) {
                int j = L.neigh[i * 2 + c];
                if (i < j) { kx[i * N + j] = m.Kxx; ky[i * N + j] = m.Kyy; kz[i * N + j] = m.Kzz; }
            }
        }
    }
    auto collect = [&](const std::vector<double>& a, std::vector<Bond>& out) {
        out.clear();
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++)
                if (a[i * N + j] != 0.0) out.push_back({i, j, a[i * N + j]});
        // An empty family becomes one placeholder entry (numNonZeros==0 -> 1, :283-287); a family
        // of size one is skipped by TightB_Ham/Diagonal (`if(K_Conn.size()==1) break;`, :116,143,347).
        if (out.size() <= 1) out.clear();
    };
    collect(kx, m.xb); collect(ky, m.yb); collect(kz, m.zb);
    // EXTENSION (Jheis): every lattice nearest-neighbour pair once, i<j, row-major order.
    m.nn.clear();
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) {
            bool is_nn = false;
            for (int c = 0; c < L.ncol; c++) if (L.neigh[i * L.ncol + c] == j && i < j) is_nn = true;
            if (is_nn) m.nn.push_back({i, j, 1.0});
        }
}

// Single-spin matrix elements, src/QuantumBasis.h:48-74 (bit 0 = up = +1/2).
static inline cplx cSz(int64_t k, int s) { return findBit(k, s) == 0 ? cplx(0.5, 0.0) : cplx(-0.5, 0.0); }
static inline cplx cSy(int64_t k, int s) { return findBit(k, s) == 0 ? cplx(0.0, 0.5) : cplx(0.0, -0.5); }

static void build_coo(OrModel& m) {
    const int64_t D = m.D;
    const int N = m.N;
    m.Sxx_init.clear(); m.Sxx_final.clear(); m.HTSxx.clear();
    m.Syy_init.clear(); m.Syy_final.clear(); m.HTSyy.clear();
    for (const Bond& b : m.xb)                                 // :113-132
        for (int64_t ket = 0; ket < D; ket++) {
            int64_t k1 = ket ^ (int64_t(1) << b.i), k2 = k1 ^ (int64_t(1) << b.j);
            m.Sxx_init.push_back(ket); m.Sxx_final.push_back(k2);
            m.HTSxx.push_back(cplx(0.5, 0) * cplx(0.5, 0) * b.k);
        }
    for (const Bond& b : m.yb)                                 // :140-158
        for (int64_t ket = 0; ket < D; ket++) {
            cplx Syi = cSy(ket, b.i);
            int64_t k1 = ket ^ (int64_t(1) << b.i);
            cplx Syj = cSy(k1, b.j);
            int64_t k2 = k1 ^ (int64_t(1) << b.j);
            m.Syy_init.push_back(ket); m.Syy_final.push_back(k2);
            m.HTSyy.push_back(Syi * Syj * b.k);
        }
    for (int64_t ket = 0; ket < D; ket++)                      // :167-179
        for (int s = 0; s < N; s++) {
            m.Sxx_init.push_back(ket ^ (int64_t(1) << s)); m.Sxx_final.push_back(ket);
            m.HTSxx.push_back(cplx(0.5, 0) * m.Bxx);
        }
    for (int64_t ket = 0; ket < D; ket++)                      // :186-198
        for (int s = 0; s < N; s++) {
            cplx coef = cSy(ket, s);
            m.Syy_init.push_back(ket ^ (int64_t(1) << s)); m.Syy_final.push_back(ket);
            m.HTSyy.push_back(m.Byy * coef);
        }
    if (m.J != 0.0) {
        // EXTENSION: J S_i.S_j on every nearest-neighbour bond: SxSx and SySy into the COO lists.
        for (const Bond& b : m.nn)
            for (int64_t ket = 0; ket < D; ket++) {
                int64_t k2 = ket ^ (int64_t(1) << b.i) ^ (int64_t(1) << b.j);
                m.Sxx_init.push_back(ket); m.Sxx_final.push_back(k2);
                m.HTSxx.push_back(cplx(0.25, 0) * m.J);
                cplx Syi = cSy(ket, b.i), Syj = cSy(ket ^ (int64_t(1) << b.i), b.j);
                m.Syy_init.push_back(ket); m.Syy_final.push_back(k2);
                m.HTSyy.push_back(Syi * Syj * m.J);
            }
    }
    // Diagonal, :331-377
    m.HDiag.assign(D, cplx(0, 0));
    for (const Bond& b : m.zb) {
#pragma omp parallel for num_threads(m.threads)
        for (int64_t k = 0; k < D; k++) m.HDiag[k] += b.k * cSz(k, b.i) * cSz(k, b.j);
    }
#pragma omp parallel for num_threads(m.threads)
    for (int64_t k = 0; k < D; k++) {
        cplx SzT = 0;
        for (int s = 0; s < N; s++) SzT += cSz(k, s);
        m.HDiag[k] += m.Bzz * SzT;
    }
    if (m.J != 0.0) {                                          // EXTENSION: J SzSz
        for (const Bond& b : m.nn) {
#pragma omp parallel for num_threads(m.threads)
            for (int64_t k = 0; k < D; k++) m.HDiag[k] += m.J * cSz(k, b.i) * cSz(k, b.j);
        }
    }
    m.coo = true;
}

// H.v exactly as the reference: diagonal pass, xx pass, yy pass into per-thread copies, then the
// thread reduction (src/Hamiltonian.h:480-557).
static void hv_coo(const OrModel& m, const cplx* vin, cplx* vout) {
    const int T = m.threads;
    const int64_t D = m.D;
    std::vector<std::vector<cplx>> tv(T, std::vector<cplx>(D, cplx(0, 0)));
#pragma omp parallel for num_threads(T) schedule(static)
    for (int64_t i = 0; i < D; i++) tv[omp_get_thread_num()][i] += m.HDiag[i] * vin[i];
    const int64_t nx = (int64_t)m.HTSxx.size(), ny = (int64_t)m.HTSyy.size();
#pragma omp parallel for num_threads(T) schedule(static)
    for (int64_t i = 0; i < nx; i++) tv[omp_get_thread_num()][m.Sxx_init[i]] += m.HTSxx[i] * vin[m.Sxx_final[i]];
#pragma omp parallel for num_threads(T) schedule(static)
    for (int64_t i = 0; i < ny; i++) tv[omp_get_thread_num()][m.Syy_init[i]] += m.HTSyy[i] * vin[m.Syy_final[i]];
#pragma omp parallel for num_threads(T) schedule(static)
    for (int64_t h = 0; h < D; h++) {
        cplx s(0, 0);
        for (int t = 0; t < T; t++) s += tv[t][h];
        vout[h] = s;
    }
}

// EXTENSION: matrix-free gather restatement of the same operator for rows [r0, r1).  Used where
// the COO lists cannot be stored (N >= 22) and as the timed CPU baseline.  Same terms as
// build_coo: x bonds K/4, y bonds K*(bits equal ? -1/4 : +1/4), field x Bx/2, field y
// By*(bit_s(k)=1 ? +i/2 : -i/2) on the partner k^2^s, diagonal zz bonds + Bz, optional J.
template <typename R>
static void hv_matfree(const OrModel& m, const std::complex<R>* vin, std::complex<R>* vout,
                       int64_t r0, int64_t r1, int threads) {
    typedef std::complex<R> C;
    const int N = m.N;
    // Rows in blocks of 2^16; within a block the terms are applied one after another, so every term
    // streams through one contiguous source block (k ^ mask for k in an aligned block) instead of
    // gathering 2.5N scattered partners per row, and terms that read the same source block (same
    // mask bits above the block) run back to back while it is in cache.
    struct Term { int64_t mask; int kind, i, j; double c; };   // kind: 0 x bond, 1 y bond, 2 J bond, 3 field
    std::vector<Term> terms;
    for (const Bond& b : m.xb) terms.push_back({(int64_t(1) << b.i) | (int64_t(1) << b.j), 0, b.i, b.j, 0.25 * b.k});
    for (const Bond& b : m.yb) terms.push_back({(int64_t(1) << b.i) | (int64_t(1) << b.j), 1, b.i, b.j, 0.25 * b.k});
    if (m.J != 0.0)
        for (const Bond& b : m.nn) terms.push_back({(int64_t(1) << b.i) | (int64_t(1) << b.j), 2, b.i, b.j, 0.5 * m.J});
    for (int s = 0; s < N; s++) terms.push_back({int64_t(1) << s, 3, s, s, 0.0});
    const int SB = 16;
    const int64_t B = int64_t(1) << SB;
    std::stable_sort(terms.begin(), terms.end(), [&](const Term& a, const Term& b) { return (a.mask >> SB) < (b.mask >> SB); });
    const int64_t nblk = (r1 - r0 + B - 1) / B;
#pragma omp parallel num_threads(threads)
    {
        std::vector<C> acc(B);
#pragma omp for schedule(static)
        for (int64_t q = 0; q < nblk; q++) {
            const int64_t k0 = r0 + q * B, k1 = std::min(r1, k0 + B);
            for (int64_t k = k0; k < k1; k++) {
                double dg = 0.0;
                for (const Bond& b : m.zb) dg += b.k * ((findBit(k, b.i) == findBit(k, b.j)) ? 0.25 : -0.25);
                for (int s = 0; s < N; s++) dg += m.Bzz * (findBit(k, s) ? -0.5 : 0.5);
                for (const Bond& b : m.nn) if (m.J != 0.0) dg += m.J * ((findBit(k, b.i) == findBit(k, b.j)) ? 0.25 : -0.25);
                acc[k - k0] = C(R(dg), 0) * vin[k];
            }
            for (const Term& t : terms) {
                const std::complex<R>* src = vin;
                const int64_t mk = t.mask;
                switch (t.kind) {
                    case 0: {
                        const C c(R(t.c), 0);
                        for (int64_t k = k0; k < k1; k++) acc[k - k0] += c * src[k ^ mk];
                        break;
                    }
                    case 1:
                        for (int64_t k = k0; k < k1; k++) {
                            const double c = (findBit(k, t.i) == findBit(k, t.j)) ? -t.c : t.c;
                            acc[k - k0] += C(R(c), 0) * src[k ^ mk];
                        }
                        break;
                    case 2: {
                        const C c(R(t.c), 0);
                        for (int64_t k = k0; k < k1; k++)
                            if (findBit(k, t.i) != findBit(k, t.j)) acc[k - k0] += c * src[k ^ mk];
                        break;
                    }
                    default:
                        for (int64_t k = k0; k < k1; k++) {
                            const C f(R(0.5 * m.Bxx), R(findBit(k, t.i) ? 0.5 * m.Byy : -0.5 * m.Byy));
                            acc[k - k0] += f * src[k ^ mk];
                        }
                }
            }
            for (int64_t k = k0; k < k1; k++) vout[k - r0] = acc[k - k0];
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Linear algebra helpers with Eigen semantics: a.dot(b) = sum conj(a_i) b_i; normalize divides
// by the 2-norm (src/DynLanczosSolver.h:76,95,100).  Sequential sums.
// ---------------------------------------------------------------------------------------------
static cplx vdot(const cplx* a, const cplx* b, int64_t n) {
    cplx s(0, 0);
    for (int64_t i = 0; i < n; i++) s += std::conj(a[i]) * b[i];
    return s;
}
static double vnorm(const cplx* a, int64_t n) {
    double s = 0;
    for (int64_t i = 0; i < n; i++) s += std::norm(a[i]);
    return std::sqrt(s);
}
static void vnormalize(cplx* a, int64_t n) {
    double z = vnorm(a, n);
    if (z > 0) for (int64_t i = 0; i < n; i++) a[i] /= z;
}

// Uniform start vector: src/DynLanczosSolver.h:465-474 with the generator of
// src/ParametersEngine.h:19,62-64,152-154: std::mt19937_64(seed) and
// uniform_real_distribution<double>(0,1), i.e. generate_canonical<double,53> = double(x)/2^64.
static double canon(std::mt19937_64& g) {
    double r = double(g() - g.min()) / 18446744073709551616.0;
    if (r >= 1.0) r = std::nextafter(1.0, 0.0);
    return r;
}

// ---------------------------------------------------------------------------------------------
// Symmetric tridiagonal eigensolver (implicit QL with Wilkinson-type shifts; the classical
// algorithm of Bowdler, Martin, Reinsch & Wilkinson, Numer. Math. 11 (1968)).  Stands in for
// LAPACK zheev on the Hermitian tridiagonal built in src/DynLanczosSolver.h:371-414 (alpha is
// real up to rounding, beta real).  Eigenvalues ascending; z is n x n column-major.
// ---------------------------------------------------------------------------------------------
static int tridiag_ql(int n, std::vector<double>& d, std::vector<double> e, std::vector<double>* z) {
    // e[i] couples i and i+1 (i < n-1); e[n-1] = 0.
    e.resize(n); if (n > 0) e[n - 1] = 0.0;
    if (z) { z->assign((size_t)n * n, 0.0); for (int i = 0; i < n; i++) (*z)[i + (size_t)i * n] = 1.0; }
    const double eps = std::numeric_limits<double>::epsilon();
    for (int l = 0; l < n; l++) {
        int iter = 0;
        while (true) {
            int m = l;
            for (; m < n - 1; m++) {
                double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= eps * dd) break;
            }
            if (m == l) break;
            if (++iter > 60) return -1;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
            double s = 1.0, c = 1.0, p = 0.0;
            int i = m - 1;
            for (; i >= l; i--) {
                double f = s * e[i], b = c * e[i];
                r = std::hypot(f, g);
                e[i + 1] = r;
                if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; break; }
                s = f / r; c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
                if (z) {
                    for (int k = 0; k < n; k++) {
                        double* zi = &(*z)[(size_t)i * n];
                        double* zi1 = &(*z)[(size_t)(i + 1) * n];
                        double t = zi1[k];
                        zi1[k] = s * zi[k] + c * t;
                        zi[k] = c * zi[k] - s * t;
                    }
                }
            }
            if (r == 0.0 && i >= l) continue;
            d[l] -= p; e[l] = g; e[m] = 0.0;
        }
    }
    // sort ascending (selection sort keeps vectors paired)
    for (int i = 0; i < n - 1; i++) {
        int k = i;
        for (int j = i + 1; j < n; j++) if (d[j] < d[k]) k = j;
        if (k != i) {
            std::swap(d[i], d[k]);
            if (z) for (int r2 = 0; r2 < n; r2++) std::swap((*z)[r2 + (size_t)i * n], (*z)[r2 + (size_t)k * n]);
        }
    }
    return 0;
}

static double TriDiag(bool vectors, const std::vector<cplx>& alpha, const std::vector<cplx>& beta,
                      std::vector<double>& Z, std::vector<double>& eigs) {
    int n = (int)alpha.size();
    std::vector<double> d(n), e(n, 0.0);
    for (int i = 0; i < n; i++) d[i] = alpha[i].real();
    for (int i = 0; i < n - 1; i++) e[i] = beta[i + 1].real();
    int rc = tridiag_ql(n, d, e, vectors ? &Z : nullptr);
    if (rc != 0) throw std::runtime_error("tridiagonal eigensolver did not converge");
    eigs = d;
    return eigs[0];
}

// ---------------------------------------------------------------------------------------------
// Ground-state Lanczos: src/DynLanczosSolver.h:38-239 (Lanczos_Nirav).
// ---------------------------------------------------------------------------------------------
static int lanczos_nirav(OrModel& m, const cplx* start, int MAXiter, double LanczosEps,
                         const std::string& PsiOrAll, int* exit_iter) {
    const int64_t N = m.D;
    std::vector<cplx> V0(start, start + N), V1(N), V2(N);
    std::vector<std::vector<cplx>> LancBasis(MAXiter + 1);
    std::vector<cplx>& alpha = m.alpha; std::vector<cplx>& beta = m.beta;
    alpha.clear(); beta.clear();
    std::vector<double> TrEVec;
    double E0, D0 = 0, diff = 0;
    beta.push_back(cplx(0, 0));
    LancBasis[0] = V0;
    hv_coo(m, V0.data(), V1.data());
    alpha.push_back(vdot(V0.data(), V1.data(), N));
    for (int64_t h = 0; h < N; h++) V1[h] = V1[h] - alpha[0] * V0[h];
    beta.push_back(cplx(vnorm(V1.data(), N), 0));
    vnormalize(V1.data(), N);
    LancBasis[1] = V1;
    int Lexit = 0, iter = 0;
    E0 = 1.0;
    while (Lexit != 1) {
        iter++;
        hv_coo(m, V1.data(), V2.data());
        alpha.push_back(vdot(V1.data(), V2.data(), N));
        for (int64_t h = 0; h < N; h++) V2[h] = V2[h] - alpha[iter] * V1[h] - beta[iter] * V0[h];
        beta.push_back(cplx(vnorm(V2.data(), N), 0));
        vnormalize(V2.data(), N);
        LancBasis[iter + 1] = V2;
        if (PsiOrAll != "OnlyEgs") {                           // :105-119 (modified Gram-Schmidt)
            std::vector<cplx>& w = LancBasis[iter + 1];
            for (int i = 0; i < iter + 1; i++) {
                cplx rij = vdot(LancBasis[i].data(), w.data(), N);
                for (int64_t h = 0; h < N; h++) w[h] -= LancBasis[i][h] * rij;
            }
            vnormalize(w.data(), N);
            V2 = w;
        }
        V0 = V1; V1 = V2;
        D0 = TriDiag(false, alpha, beta, TrEVec, m.TriDeval);  // :125
        diff = std::fabs(E0 - D0);
        if (diff < LanczosEps) { Lexit = 1; E0 = D0; } else { E0 = D0; }
        if (iter == MAXiter - 1 || Lexit == 1) {
            Lexit = 1;
            D0 = TriDiag(true, alpha, beta, m.TrEVec, m.TriDeval);
        }
    }
    int EXITiter = iter + 1;
    *exit_iter = EXITiter;
    m.Psi.assign(N, cplx(0, 0));
    if (PsiOrAll == "OnlyEgs") { m.nPsi = 0; m.PsiAll.clear(); return 0; }
    int loopval = (PsiOrAll == "GS") ? 1 : EXITiter;           // :181-234
    m.nPsi = loopval;
    m.PsiAll.assign((size_t)loopval * N, cplx(0, 0));
    const int n = EXITiter;
#pragma omp parallel for num_threads(m.threads)
    for (int k = 0; k < loopval; k++) {
        cplx* pk = &m.PsiAll[(size_t)k * N];
        for (int64_t h = 0; h < N; h++)
            for (int mm = 0; mm < EXITiter; mm++) pk[h] += LancBasis[mm][h] * m.TrEVec[mm + (size_t)k * n];
    }
    std::copy(m.PsiAll.begin(), m.PsiAll.begin() + N, m.Psi.begin());
    return 0;
}

// EXTENSION: the same three-term recurrence without reorthogonalisation (src/DynLanczosSolver.h:
// 73-101 with the reortho block :105-119 skipped, as LancType=OnlyEgs does) on three vectors and
// the matrix-free H.v, for bases whose M+1 vectors or COO lists do not fit (N >= 22).  E0 and the
// tridiagonal come from the first sweep; a second sweep regenerates the Lanczos vectors (same
// operations, so bit-identical) and forms |gs> = sum_m Z(m,0) L_m (:208-234 for k = 0), then
// normalises it (the vectors are not orthogonal without reorthogonalisation).
static void lanczos3(OrModel& m, const cplx* start, int M, std::vector<double>& a, std::vector<double>& b,
                     std::vector<double>& ritz, std::vector<cplx>* gs) {
    const int64_t D = m.D;
    std::vector<cplx> V0(D), V1(start, start + D), V2(D);
    auto sweep = [&](const std::vector<double>* z, std::vector<cplx>* acc) {
        std::fill(V0.begin(), V0.end(), cplx(0, 0));
        std::copy(start, start + D, V1.begin());
        vnormalize(V1.data(), D);
        if (acc) for (int64_t h = 0; h < D; h++) (*acc)[h] = V1[h] * (*z)[0];
        for (int it = 0; it < M; it++) {
            hv_matfree<double>(m, V1.data(), V2.data(), 0, D, m.threads);
            const double al = vdot(V1.data(), V2.data(), D).real();
            const double be = it ? b[it] : 0.0;
            if (!acc) a[it] = al;
            for (int64_t h = 0; h < D; h++) V2[h] = V2[h] - (acc ? a[it] : al) * V1[h] - be * V0[h];
            if (it + 1 == M) break;
            const double bn = vnorm(V2.data(), D);
            if (!acc) b[it + 1] = bn;
            for (int64_t h = 0; h < D; h++) V2[h] /= (acc ? b[it + 1] : bn);
            std::swap(V0, V1);
            std::swap(V1, V2);
            if (acc) for (int64_t h = 0; h < D; h++) (*acc)[h] += V1[h] * (*z)[it + 1];
        }
    };
    a.assign(M, 0.0);
    b.assign(M + 1, 0.0);
    sweep(nullptr, nullptr);
    std::vector<double> d(a), e(M, 0.0), Z;
    for (int i = 0; i + 1 < M; i++) e[i] = b[i + 1];
    if (tridiag_ql(M, d, e, gs ? &Z : nullptr) != 0) throw std::runtime_error("tridiagonal eigensolver failed");
    ritz = d;
    if (gs) {
        std::vector<double> z0(Z.begin(), Z.begin() + M);   // column 0: eigenvector of the lowest Ritz value
        gs->assign(D, cplx(0, 0));
        sweep(&z0, gs);
        vnormalize(gs->data(), D);
    }
}

// ---------------------------------------------------------------------------------------------
// Operators, src/Observables.h (scatter form, out(ket_out) += coef * in(ket)).
// ---------------------------------------------------------------------------------------------
typedef std::vector<cplx> VecC;

static VecC ApplySz(const OrModel& m, const VecC& v, int i) {        // :429-445
    VecC out(m.D, cplx(0, 0));
    for (int64_t k = 0; k < m.D; k++) out[k] += cSz(k, i) * v[k];
    return out;
}
static VecC ApplySx(const OrModel& m, const VecC& v, int i) {        // :506-521
    VecC out(m.D, cplx(0, 0));
    for (int64_t k = 0; k < m.D; k++) out[k ^ (int64_t(1) << i)] += cplx(0.5, 0.0) * v[k];
    return out;
}
static VecC ApplySy(const OrModel& m, const VecC& v, int i) {        // :488-503
    VecC out(m.D, cplx(0, 0));
    for (int64_t k = 0; k < m.D; k++) out[k ^ (int64_t(1) << i)] += cSy(k, i) * v[k];
    return out;
}
static VecC vsub(const VecC& a, const VecC& b) { VecC o(a.size()); for (size_t i = 0; i < a.size(); i++) o[i] = a[i] - b[i]; return o; }
static VecC vadd(const VecC& a, const VecC& b) { VecC o(a.size()); for (size_t i = 0; i < a.size(); i++) o[i] = a[i] + b[i]; return o; }
static VecC vscale(double s, const VecC& a) { VecC o(a.size()); for (size_t i = 0; i < a.size(); i++) o[i] = s * a[i]; return o; }
static VecC vscalec(cplx s, const VecC& a) { VecC o(a.size()); for (size_t i = 0; i < a.size(); i++) o[i] = s * a[i]; return o; }
static int nb(const OrModel& m, int i, int c) {
    int j = m.lat.neigh[i * m.lat.ncol + c];
    if (j < 0 || j >= m.N) throw std::runtime_error("operator needs a neighbour that does not exist");
    return j;
}

static VecC ApplyJsz(const OrModel& m, const VecC& v, int si) {      // :161-199
    VecC L2 = vscale(m.Kyy, ApplySx(m, ApplySy(m, v, nb(m, si, 1)), si));
    VecC R2 = vscale(m.Kxx, ApplySy(m, ApplySx(m, v, nb(m, si, 2)), si));
    return vsub(L2, R2);
}
static VecC ApplyJsy(const OrModel& m, const VecC& v, int si) {      // :202-240
    VecC L2 = vscale(m.Kxx, ApplySz(m, ApplySx(m, v, nb(m, si, 2)), si));
    VecC R2 = vscale(m.Kzz, ApplySx(m, ApplySz(m, v, nb(m, si, 0)), si));
    return vsub(L2, R2);
}
static VecC ApplyJsx(const OrModel& m, const VecC& v, int si) {      // :243-281
    VecC L2 = vscale(m.Kzz, ApplySy(m, ApplySz(m, v, nb(m, si, 0)), si));
    VecC R2 = vscale(m.Kyy, ApplySz(m, ApplySy(m, v, nb(m, si, 1)), si));
    return vsub(L2, R2);
}
static VecC ApplyJey(const OrModel& m, const VecC& v, int si) {      // :321-354
    int iy = nb(m, si, 1), iypx = nb(m, iy, 2), iypz = nb(m, iy, 0);
    VecC L3 = vscale(m.Kxx * m.Kyy, ApplySy(m, ApplySz(m, ApplySx(m, v, iypx), iy), si));
    VecC R3 = vscale(m.Kyy * m.Kzz, ApplySy(m, ApplySx(m, ApplySz(m, v, iypz), iy), si));
    return vsub(L3, R3);
}
static VecC ApplyJex(const OrModel& m, const VecC& v, int si) {      // :358-389
    int ix = nb(m, si, 2), ixpy = nb(m, ix, 1), ixpz = nb(m, ix, 0);
    VecC L3 = vscale(m.Kxx * m.Kyy, ApplySx(m, ApplySz(m, ApplySy(m, v, ixpy), ix), si));
    VecC R3 = vscale(m.Kxx * m.Kzz, ApplySx(m, ApplySy(m, ApplySz(m, v, ixpz), ix), si));
    return vsub(R3, L3);
}
static VecC ApplySxSySz(const OrModel& m, const VecC& v, int si) {   // :592-607
    return vadd(vadd(ApplySx(m, v, si), ApplySy(m, v, si)), ApplySz(m, v, si));
}
static VecC ApplySpe3(const OrModel& m, const VecC& v, int i) {      // :539-555 (constants verbatim)
    VecC x = ApplySx(m, v, i), y = ApplySy(m, v, i), z = ApplySz(m, v, i);
    VecC o(m.D);
    for (int64_t k = 0; k < m.D; k++) o[k] = cplx(-0.408248, 0.707107) * x[k] + cplx(-0.408248, -0.707107) * y[k] + 0.816497 * z[k];
    return o;
}
static VecC ApplySme3(const OrModel& m, const VecC& v, int i) {      // :573-589
    VecC x = ApplySx(m, v, i), y = ApplySy(m, v, i), z = ApplySz(m, v, i);
    VecC o(m.D);
    for (int64_t k = 0; k < m.D; k++) o[k] = cplx(-0.408248, -0.707107) * x[k] + cplx(-0.408248, 0.707107) * y[k] + 0.816497 * z[k];
    return o;
}
static VecC ApplySp(const OrModel& m, const VecC& v, int i) { return vadd(ApplySx(m, v, i), vscalec(cplx(0, 1), ApplySy(m, v, i))); }   // :524-537
static VecC ApplySm(const OrModel& m, const VecC& v, int i) { return vsub(ApplySx(m, v, i), vscalec(cplx(0, 1), ApplySy(m, v, i))); }   // :558-571

static VecC total(const OrModel& m, const VecC& v, VecC (*f)(const OrModel&, const VecC&, int), int s0, int ds) {
    VecC out(m.D, cplx(0, 0));                                           // :448-470, :664-699
    for (int s = s0; s < m.N; s += ds) { VecC t = f(m, v, s); for (int64_t k = 0; k < m.D; k++) out[k] += t[k]; }
    return out;
}

static VecC apply_named(const OrModel& m, const VecC& v, const std::string& op, int site) {
    if (op == "Sx") return ApplySx(m, v, site);
    if (op == "Sy") return ApplySy(m, v, site);
    if (op == "Sz") return ApplySz(m, v, site);
    if (op == "Sp") return ApplySp(m, v, site);
    if (op == "Sm") return ApplySm(m, v, site);
    if (op == "Spe3") return ApplySpe3(m, v, site);
    if (op == "Sme3") return ApplySme3(m, v, site);
    if (op == "I") return v;
    if (op == "Jsx") return ApplyJsx(m, v, site);
    if (op == "Jsy") return ApplyJsy(m, v, site);
    if (op == "Jsz") return ApplyJsz(m, v, site);
    if (op == "Jex") return ApplyJex(m, v, site);
    if (op == "Jey") return ApplyJey(m, v, site);
    if (op == "JexJeyJez") return vadd(ApplyJex(m, v, site), ApplyJey(m, v, site));
    if (op == "JsxJsyJsz") return vadd(vadd(ApplyJsx(m, v, site), ApplyJsy(m, v, site)), ApplyJsz(m, v, site));
    if (op == "SxSySz") return ApplySxSySz(m, v, site);
    if (op == "JsxTotal") return total(m, v, ApplyJsx, 0, 1);
    if (op == "JsyTotal") return total(m, v, ApplyJsy, 0, 1);
    if (op == "JszTotal") return total(m, v, ApplyJsz, 0, 1);
    if (op == "JexTotal") return total(m, v, ApplyJex, 0, 2);
    if (op == "JeyTotal") return total(m, v, ApplyJey, 1, 2);
    throw std::runtime_error("Unknown Operator label");
}

// ---------------------------------------------------------------------------------------------
// Dynamics, src/dynamics.h.  Spectra are written to out[(om)*ncol + c] with column 0 = omega,
// in the column order of the reference's *_outSpectrum.real files.
// ---------------------------------------------------------------------------------------------
struct DynGrid { int omegasteps; double domega, eta; };

static void dyn_jeje(const OrModel& m, const DynGrid& g, double* out) {     // :345-460
    const int64_t D = m.D;
    VecC Jtx = total(m, m.Psi, ApplyJex, 0, 2), Jty = total(m, m.Psi, ApplyJey, 1, 2);
    VecC Jt = vadd(Jtx, Jty);
    cplx Jex0 = vdot(m.Psi.data(), Jtx.data(), D), Jey0 = vdot(m.Psi.data(), Jty.data(), D);
    cplx Jez0(0, 0);  // the reference reads an uninitialised Jez[0] here (:368-369,424); taken as 0
    cplx Jet0 = vdot(m.Psi.data(), Jt.data(), D);
    const int M = m.nPsi;
    std::vector<cplx> O((size_t)M * 3);
#pragma omp parallel for num_threads(m.threads)
    for (int n = 0; n < M; n++) {
        const cplx* ps = &m.PsiAll[(size_t)n * D];
        O[n * 3 + 0] = vdot(ps, Jtx.data(), D); O[n * 3 + 1] = vdot(ps, Jty.data(), D); O[n * 3 + 2] = vdot(ps, Jt.data(), D);
    }
    const double Eg = m.TriDeval[0];
    for (int om = 0; om <= g.omegasteps; om++) {
        double omega = g.domega * om;
        cplx I00(0, 0), I01(0, 0), I11(0, 0), I10(0, 0), sum(0, 0);
        cplx dnom1(omega, -g.eta);
        for (int n = 0; n < M; n++) {
            double En = m.TriDeval[n];
            cplx den(omega - (En - Eg), -g.eta);
            cplx x = O[n * 3], y = O[n * 3 + 1], t = O[n * 3 + 2];
            I00 = I00 + std::conj(x) * x / den; I01 = I01 + std::conj(x) * y / den;
            I11 = I11 + std::conj(y) * y / den; I10 = I10 + std::conj(y) * x / den;
            sum = sum + std::conj(t) * t / den;
        }
        I00 = I00 - std::conj(Jex0) * Jex0 / dnom1; I01 = I01 - std::conj(Jex0) * Jey0 / dnom1;
        I11 = I11 - std::conj(Jey0) * Jey0 / dnom1; I10 = I10 - std::conj(Jey0) * Jez0 / dnom1;
        sum = sum - std::conj(Jet0) * Jet0 / dnom1;
        double* row = out + (size_t)om * 6;
        row[0] = omega; row[1] = I00.imag(); row[2] = I11.imag(); row[3] = I01.imag(); row[4] = I10.imag(); row[5] = sum.imag();
    }
}

static void dyn_jsjs(const OrModel& m, const DynGrid& g, double* out) {     // :222-341
    const int64_t D = m.D;
    VecC Jtx = total(m, m.Psi, ApplyJsx, 0, 1), Jty = total(m, m.Psi, ApplyJsy, 0, 1), Jtz = total(m, m.Psi, ApplyJsz, 0, 1);
    VecC Jt = vadd(vadd(Jtx, Jty), Jtz);
    cplx JS[4] = {vdot(m.Psi.data(), Jtx.data(), D), vdot(m.Psi.data(), Jty.data(), D),
                  vdot(m.Psi.data(), Jtz.data(), D), vdot(m.Psi.data(), Jt.data(), D)};
    const int M = m.nPsi;
    std::vector<cplx> O((size_t)M * 4);
#pragma omp parallel for num_threads(m.threads)
    for (int n = 0; n < M; n++) {
        const cplx* ps = &m.PsiAll[(size_t)n * D];
        O[n * 4 + 0] = vdot(ps, Jtx.data(), D); O[n * 4 + 1] = vdot(ps, Jty.data(), D);
        O[n * 4 + 2] = vdot(ps, Jtz.data(), D); O[n * 4 + 3] = vdot(ps, Jt.data(), D);
    }
    const double Eg = m.TriDeval[0];
    for (int om = 0; om <= g.omegasteps; om++) {
        double omega = g.domega * om;
        cplx I[3][3] = {}; cplx sum(0, 0);
        cplx dnom1(omega, -g.eta);
        for (int n = 0; n < M; n++) {
            cplx den(omega - (m.TriDeval[n] - Eg), -g.eta);
            cplx x = O[n * 4], y = O[n * 4 + 1], z = O[n * 4 + 2], t = O[n * 4 + 3];
            I[0][0] = I[0][0] + std::conj(x) * x / den; I[0][1] = I[0][1] + std::conj(x) * y / den;
            I[0][2] = I[0][2] + std::conj(x) * z / den; I[1][1] = I[1][1] + std::conj(y) * y / den;
            I[1][2] = I[1][2] + std::conj(y) * z / den; I[2][2] = I[2][2] + std::conj(z) * z / den;
            sum = sum + std::conj(t) * t / den;
        }
        I[0][0] = I[0][0] - std::conj(JS[0]) * JS[0] / dnom1; I[0][1] = I[0][1] - std::conj(JS[0]) * JS[1] / dnom1;
        I[0][2] = I[0][2] - std::conj(JS[0]) * JS[2] / dnom1; I[1][1] = I[1][1] - std::conj(JS[1]) * JS[1] / dnom1;
        I[1][2] = I[1][2] - std::conj(JS[1]) * JS[2] / dnom1; I[2][2] = I[2][2] - std::conj(JS[2]) * JS[2] / dnom1;
        sum = sum - std::conj(JS[3]) * JS[3] / dnom1;
        cplx data[6] = {I[0][0], I[1][1], I[2][2], I[0][1], I[0][2], I[1][2]};
        double* row = out + (size_t)om * 15;
        row[0] = omega;
        for (int kk = 0; kk < 6; kk++) { row[1 + 2 * kk] = data[kk].real(); row[2 + 2 * kk] = data[kk].imag(); }
        row[13] = sum.real(); row[14] = sum.imag();
    }
}

static void dyn_localszsz(const OrModel& m, const DynGrid& g, double* out) {   // :64-217
    const int64_t D = m.D;
    const int N = m.N, M = m.nPsi;
    std::vector<cplx> O((size_t)6 * N * M);
    std::vector<cplx> Sx(N), Sy(N), Sz(N), St(N), Sp(N), Sm(N);
    for (int si = 0; si < N; si++) {
        VecC v[6] = {ApplySx(m, m.Psi, si), ApplySy(m, m.Psi, si), ApplySz(m, m.Psi, si),
                     ApplySxSySz(m, m.Psi, si), ApplySpe3(m, m.Psi, si), ApplySme3(m, m.Psi, si)};
        Sx[si] = vdot(m.Psi.data(), v[0].data(), D); Sy[si] = vdot(m.Psi.data(), v[1].data(), D);
        Sz[si] = vdot(m.Psi.data(), v[2].data(), D); St[si] = vdot(m.Psi.data(), v[3].data(), D);
        Sp[si] = vdot(m.Psi.data(), v[4].data(), D); Sm[si] = vdot(m.Psi.data(), v[5].data(), D);
#pragma omp parallel for num_threads(m.threads)
        for (int n = 0; n < M; n++)
            for (int c = 0; c < 6; c++) O[((size_t)c * N + si) * M + n] = vdot(&m.PsiAll[(size_t)n * D], v[c].data(), D);
    }
    const double Eg = m.TriDeval[0];
    for (int om = 0; om <= g.omegasteps; om++) {
        double omega = g.domega * om;
        cplx I00(0, 0), I01(0, 0), I02(0, 0), I11(0, 0), I12(0, 0), I22(0, 0), sum(0, 0), T0(0, 0), T1(0, 0);
        cplx dnom1(omega, -g.eta);
        for (int si = 0; si < N; si++) {
            for (int n = 0; n < M; n++) {
                cplx den(omega - (m.TriDeval[n] - Eg), -g.eta);
                auto Oc = [&](int c) { return O[((size_t)c * N + si) * M + n]; };
                cplx x = Oc(0), y = Oc(1), z = Oc(2), t = Oc(3), p = Oc(4), q = Oc(5);
                I00 = I00 + std::conj(x) * x / den; I01 = I01 + std::conj(x) * y / den; I02 = I02 + std::conj(x) * z / den;
                I11 = I11 + std::conj(y) * y / den; I12 = I12 + std::conj(y) * z / den; I22 = I22 + std::conj(z) * z / den;
                sum = sum + std::conj(t) * t / den;
                T0 = T0 + std::conj(p) * p / den; T1 = T1 + std::conj(q) * q / den;
            }
            I00 = I00 - std::conj(Sx[si]) * Sx[si] / dnom1; I01 = I01 - std::conj(Sx[si]) * Sy[si] / dnom1;
            I02 = I02 - std::conj(Sx[si]) * Sz[si] / dnom1; I11 = I11 - std::conj(Sy[si]) * Sy[si] / dnom1;
            I12 = I12 - std::conj(Sy[si]) * Sz[si] / dnom1; I22 = I22 - std::conj(Sz[si]) * Sz[si] / dnom1;
            sum = sum - std::conj(St[si]) * St[si] / dnom1;
            T0 -= Sm[si] * Sp[si] / dnom1;                     // :185-186 (no conjugate, as written)
            T1 -= Sp[si] * Sm[si] / dnom1;
        }
        cplx data[8] = {I00, I11, I22, I01, I02, I12, T0, T1};
        double* row = out + (size_t)om * 9;
        row[0] = omega;
        for (int kk = 0; kk < 8; kk++) row[1 + kk] = data[kk].imag();
    }
}

// EXTENSION: continued-fraction Lanczos coefficients from a start vector phi (three-term
// recurrence, optional full reorthogonalisation).  a[k], b[k] with b[0] = |phi|.
static int cf_lanczos(const OrModel& m, const cplx* phi, int steps, bool reortho, double* a, double* b, int* nsteps) {
    const int64_t D = m.D;
    double nrm = vnorm(phi, D);
    b[0] = nrm;
    if (nrm == 0.0) { *nsteps = 0; return 0; }
    std::vector<cplx> q0(D, cplx(0, 0)), q1(phi, phi + D), w(D);
    for (auto& x : q1) x /= nrm;
    std::vector<std::vector<cplx>> Q;
    if (reortho) Q.push_back(q1);
    int k = 0;
    for (; k < steps; k++) {
        if (m.coo) hv_coo(m, q1.data(), w.data()); else hv_matfree<double>(m, q1.data(), w.data(), 0, D, m.threads);
        double ak = vdot(q1.data(), w.data(), D).real();
        a[k] = ak;
        double bk = (k == 0) ? 0.0 : b[k];
        for (int64_t h = 0; h < D; h++) w[h] = w[h] - ak * q1[h] - bk * q0[h];
        if (reortho)
            for (auto& q : Q) { cplx r = vdot(q.data(), w.data(), D); for (int64_t h = 0; h < D; h++) w[h] -= r * q[h]; }
        double bn = vnorm(w.data(), D);
        if (k + 1 < steps) b[k + 1] = bn;
        if (bn < 1e-14 || k + 1 == steps) { k++; break; }
        q0 = q1;
        for (int64_t h = 0; h < D; h++) q1[h] = w[h] / bn;
        if (reortho) Q.push_back(q1);
    }
    *nsteps = k;
    return 0;
}

// G(z) = b0^2 / (z - a0 - b1^2/(z - a1 - ...)), z = omega + E0 - i eta; evaluated bottom-up.
static cplx cf_eval(const double* a, const double* b, int n, cplx z) {
    if (n == 0) return cplx(0, 0);
    cplx t(0, 0);
    for (int k = n - 1; k >= 1; k--) t = b[k] * b[k] / (z - a[k] - t);
    return b[0] * b[0] / (z - a[0] - t);
}

// =============================================================================================
// C API for ctypes (tests / bench CPU baseline)
// =============================================================================================
static thread_local std::string g_err;

extern "C" {

const char* or_last_error() { return g_err.c_str(); }

int or_lattice(const char* model, int Lx, int Ly, int pbcx, int pbcy, int* neigh, int* ncol) {
    OrLattice L;
    if (std::string(model) == "Kitaev") honeycomb1(Lx, Ly, pbcx, pbcy, L);
    else chain(Lx * Ly, pbcx, L);
    std::copy(L.neigh.begin(), L.neigh.end(), neigh);
    *ncol = L.ncol;
    return 0;
}

void* or_model_create(const char* model, int Lx, int Ly, int pbcx, int pbcy,
                      double Kxx, double Kyy, double Kzz, double Bxx, double Byy, double Bzz,
                      double J, int threads, int build_coo_lists) {
    try {
        OrModel* m = new OrModel();
        std::string md(model);
        m->kitaev = (md == "Kitaev");
        if (!m->kitaev && md != "HeisenbergChain") { delete m; g_err = "Unknown Model parameter"; return nullptr; }
        if (m->kitaev) honeycomb1(Lx, Ly, pbcx, pbcy, m->lat); else chain(Lx * Ly, pbcx, m->lat);
        m->N = m->lat.N; m->D = int64_t(1) << m->N;
        m->Kxx = Kxx; m->Kyy = Kyy; m->Kzz = Kzz; m->Bxx = Bxx; m->Byy = Byy; m->Bzz = Bzz; m->J = J;
        m->threads = threads > 0 ? threads : 1;
        connectors(*m);
        if (build_coo_lists) build_coo(*m);
        return m;
    } catch (std::exception& e) { g_err = e.what(); return nullptr; }
}

void or_model_destroy(void* h) { delete (OrModel*)h; }

int or_model_info(void* h, int* N, int64_t* D, int* nx, int* ny, int* nz, int* bonds /* (nx+ny+nz) x 2 */) {
    OrModel* m = (OrModel*)h;
    *N = m->N; *D = m->D; *nx = (int)m->xb.size(); *ny = (int)m->yb.size(); *nz = (int)m->zb.size();
    if (bonds) {
        int c = 0;
        for (auto* L : {&m->xb, &m->yb, &m->zb}) for (auto& b : *L) { bonds[2 * c] = b.i; bonds[2 * c + 1] = b.j; c++; }
    }
    return 0;
}

int or_hdiag(void* h, double* out /* D x 2 */) {
    OrModel* m = (OrModel*)h;
    if (!m->coo) build_coo(*m);
    std::memcpy(out, m->HDiag.data(), m->D * sizeof(cplx));
    return 0;
}

int or_hv(void* h, const double* vin, double* vout) {
    OrModel* m = (OrModel*)h;
    if (m->coo) hv_coo(*m, (const cplx*)vin, (cplx*)vout);
    else hv_matfree<double>(*m, (const cplx*)vin, (cplx*)vout, 0, m->D, m->threads);
    return 0;
}

int or_hv_rows(void* h, const double* vin, double* vout, int64_t r0, int64_t r1, int threads) {
    OrModel* m = (OrModel*)h;
    hv_matfree<double>(*m, (const cplx*)vin, (cplx*)vout, r0, r1, threads);
    return 0;
}

int or_hv_rows_c64(void* h, const float* vin, float* vout, int64_t r0, int64_t r1, int threads) {
    OrModel* m = (OrModel*)h;
    hv_matfree<float>(*m, (const cplxf*)vin, (cplxf*)vout, r0, r1, threads);
    return 0;
}

int or_random_start(int64_t seed, int64_t D, double* out, int normalize) {
    std::mt19937_64 g((uint64_t)(int)seed);                    // RandomSeed is an int in the reference
    cplx* v = (cplx*)out;
    for (int64_t i = 0; i < D; i++) {
        double re = -1.0 + canon(g) * 2.0;
        double im = -1.0 + canon(g) * 2.0;
        v[i] = cplx(re, im);
    }
    if (normalize) vnormalize(v, D);
    return 0;
}

int or_tridiag(int n, const double* d_in, const double* e_in, double* evals, double* evecs) {
    std::vector<double> d(d_in, d_in + n), e(e_in, e_in + n);
    std::vector<double> z;
    int rc = tridiag_ql(n, d, e, evecs ? &z : nullptr);
    std::copy(d.begin(), d.end(), evals);
    if (evecs) std::copy(z.begin(), z.end(), evecs);
    return rc;
}

int or_lanczos(void* h, const double* start, int M, double eps, const char* lanctype,
               double* alpha /* M */, double* beta /* M+1 */, double* ritz /* M */, int* nsteps) {
    OrModel* m = (OrModel*)h;
    try {
        if (!m->coo) build_coo(*m);
        int ex = 0;
        lanczos_nirav(*m, (const cplx*)start, M, eps, lanctype, &ex);
        *nsteps = ex;
        for (int i = 0; i < ex; i++) alpha[i] = m->alpha[i].real();
        for (int i = 0; i <= ex && i < (int)m->beta.size(); i++) beta[i] = m->beta[i].real();
        for (int i = 0; i < ex; i++) ritz[i] = m->TriDeval[i];
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int or_lanczos3(void* h, const double* start, int M, double* alpha, double* beta, double* ritz, double* gs_out) {
    OrModel* m = (OrModel*)h;
    try {
        std::vector<double> a, b, r;
        std::vector<cplx> gs;
        lanczos3(*m, (const cplx*)start, M, a, b, r, gs_out ? &gs : nullptr);
        std::copy(a.begin(), a.end(), alpha);
        std::copy(b.begin(), b.end(), beta);
        std::copy(r.begin(), r.end(), ritz);
        if (gs_out) std::memcpy(gs_out, gs.data(), gs.size() * sizeof(cplx));
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int or_get_psi(void* h, double* out) {
    OrModel* m = (OrModel*)h;
    std::memcpy(out, m->Psi.data(), m->D * sizeof(cplx));
    return 0;
}

int or_set_ritz(void* h, int n, const double* evals, const double* psiall /* n x D */) {
    // Solver=ED path (src/DynLanczosSolver.h:269-283, fillFromED): eigenpairs supplied by the caller.
    OrModel* m = (OrModel*)h;
    m->TriDeval.assign(evals, evals + n);
    m->nPsi = n;
    m->PsiAll.assign((const cplx*)psiall, (const cplx*)psiall + (size_t)n * m->D);
    m->Psi.assign(m->PsiAll.begin(), m->PsiAll.begin() + m->D);
    return 0;
}

int or_apply(void* h, const char* op, int site, const double* vin, double* vout) {
    OrModel* m = (OrModel*)h;
    try {
        VecC v((const cplx*)vin, (const cplx*)vin + m->D);
        VecC o = apply_named(*m, v, op, site);
        std::memcpy(vout, o.data(), m->D * sizeof(cplx));
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int or_dynamics(void* h, const char* which, int omegasteps, double domega, double eta, double* out) {
    OrModel* m = (OrModel*)h;
    try {
        DynGrid g{omegasteps, domega, eta};
        std::string w(which);
        if (w == "Energy Current") dyn_jeje(*m, g, out);
        else if (w == "Spin Current") dyn_jsjs(*m, g, out);
        else if (w == "LocalSzSz") dyn_localszsz(*m, g, out);
        else { g_err = "Unknown dynstr parameter"; return 1; }
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int or_cf_lanczos(void* h, const double* phi, int steps, int reortho, double* a, double* b, int* nsteps) {
    OrModel* m = (OrModel*)h;
    return cf_lanczos(*m, (const cplx*)phi, steps, reortho != 0, a, b, nsteps);
}

int or_cf_eval(const double* a, const double* b, int n, double E0, int nomega, const double* omega,
               double eta, double* out /* nomega x 2 */) {
    for (int i = 0; i < nomega; i++) {
        cplx g = cf_eval(a, b, n, cplx(omega[i] + E0, -eta));
        out[2 * i] = g.real(); out[2 * i + 1] = g.imag();
    }
    return 0;
}

// Observables::TwoPointCorr (src/Observables.h:131-158): for sj, out1 = B_sj |gs>; for si >= sj,
// Corr(si,sj) = <gs| A_si out1> and Corr(sj,si) = the same value (not its conjugate).  psi NULL:
// the model's ground state.  out: N x N complex, row-major.
int or_two_point(void* h, const char* opA, const char* opB, const double* psi, double* out) {
    OrModel* m = (OrModel*)h;
    try {
        const int N = m->N;
        const VecC gs = psi ? VecC((const cplx*)psi, (const cplx*)psi + m->D) : m->Psi;
        std::vector<cplx> C((size_t)N * N);
        for (int sj = 0; sj < N; sj++) {
            const VecC out1 = apply_named(*m, gs, opB, sj);
            for (int si = sj; si < N; si++) {
                const VecC out2 = apply_named(*m, out1, opA, si);
                const cplx c = vdot(gs.data(), out2.data(), m->D);
                C[(size_t)si * N + sj] = c;
                C[(size_t)sj * N + si] = c;
            }
        }
        std::memcpy(out, C.data(), C.size() * sizeof(cplx));
        return 0;
    } catch (std::exception& e) { g_err = e.what(); return 1; }
}

int or_dot(int64_t D, const double* a, const double* b, double* out) {
    cplx r = vdot((const cplx*)a, (const cplx*)b, D);
    out[0] = r.real(); out[1] = r.imag();
    return 0;
}

}  // extern "C"
