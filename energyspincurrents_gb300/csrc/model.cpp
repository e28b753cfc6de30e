// model.cpp -- lattice, bond tables and operator strings of the Kitaev(-Heisenberg) model.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>

#include "esc_internal.h"

namespace esc {

// Honeycomb cluster of Lattice::Honeycomb1 (src/Lattice.h:434-576).  Cell (i, j), i < Lx,
// j < Ly/2, holds an a-site at (2i+j, 2j) and a b-site at (2i+1+j, 2j+1) with indices
// 2(i*Ly/2+j) and +1 (:460-486).  Neighbour columns: 2 = x at (+1,+1), 1 = y at (+1,-1),
// 0 = z at (0,+1) (:497-522), periodic wraps as in :530-564 (including the reference's
// boundary tests, e.g. `jx < xmax` for the z column).
static void honeycomb(int Lx, int Ly, bool pbcx, bool pbcy, Lattice& L) {
    const int N = Lx * Ly, LLX = Lx, LLY = Ly / 2;
    L.N = N; L.ncol = 3;
    L.neigh.assign((size_t)N * 3, -1);
    L.indx.assign(N, 0); L.indy.assign(N, 0);
    const int ncr = 2 * LLX + LLY, ncc = 2 * LLY;
    std::vector<int> Nc((size_t)ncr * ncc, -1);
    auto site_at = [&](int x, int y) { return (x < 0 || y < 0 || x >= ncr || y >= ncc) ? -1 : Nc[x + (size_t)y * ncr]; };
    int c = 0;
    for (int i = 0; i < LLX; i++)
        for (int j = 0; j < LLY; j++) {
            // t1 = (2, 0), t2 = (1, 2): the reference's scaled lattice vectors evaluate to these
            // integers exactly (sqrt(3)/2 * 4/sqrt(3) == 2.0 in IEEE double).
            const int xa = 2 * i + j, ya = 2 * j, xb = 2 * i + 1 + j, yb = 2 * j + 1;
            L.indx[c] = xa; L.indy[c] = ya; Nc[xa + (size_t)ya * ncr] = c; c++;
            L.indx[c] = xb; L.indy[c] = yb; Nc[xb + (size_t)yb * ncr] = c; c++;
        }
    const int xmax = N ? *std::max_element(L.indx.begin(), L.indx.end()) : 0;
    const int ymax = N ? *std::max_element(L.indy.begin(), L.indy.end()) : 0;
    auto link = [&](int i, int j, int col) { L.neigh[(size_t)i * 3 + col] = j; L.neigh[(size_t)j * 3 + col] = i; };
    for (int i = 0; i < N; i++) {
        const int ix = L.indx[i], iy = L.indy[i];
        int j;
        if (ix + 1 < xmax + 1 && iy + 1 < ymax + 1 && (j = site_at(ix + 1, iy + 1)) != -1) link(i, j, 2);
        if (ix + 1 < xmax + 1 && iy - 1 < ymax && iy - 1 >= 0 && (j = site_at(ix + 1, iy - 1)) != -1) link(i, j, 1);
        if (ix < xmax && iy + 1 < ymax + 1 && (j = site_at(ix, iy + 1)) != -1) link(i, j, 0);
        if (pbcy && ix - LLY < xmax && iy == ymax && (j = site_at(ix - LLY, 0)) != -1) link(i, j, 0);
        if (pbcx && iy % 2 == 0 && site_at(ix, iy) < LLY * 2) {
            const int jx = ix + 2 * LLX - 1, jy = iy + 1;
            if (jx < xmax + 1 && iy < ymax + 1 && (j = site_at(jx, jy)) != -1) link(i, j, 1);
        }
    }
}

// Lattice::Chain (src/Lattice.h:60-136): column 0 = +x neighbour, 1 = -x neighbour.
static void chain(int N, bool pbcx, Lattice& L) {
    L.N = N; L.ncol = 2;
    L.neigh.assign((size_t)N * 3, -1);
    L.indx.resize(N); L.indy.assign(N, 0);
    for (int i = 0; i < N; i++) {
        L.indx[i] = i;
        if (i + 1 < N) L.neigh[(size_t)i * 3 + 0] = i + 1;
        if (i - 1 > -1) L.neigh[(size_t)i * 3 + 1] = i - 1;
        if (pbcx) {
            if (i == N - 1) L.neigh[(size_t)i * 3 + 0] = 0;
            if (i == 0) L.neigh[(size_t)i * 3 + 1] = N - 1;
        }
    }
}

void build_lattice(const esc_params& p, Lattice& L) {
    const std::string model(p.model);
    const int N = p.Lx * p.Ly;
    if (N <= 0 || N > MAX_SITES) throw std::invalid_argument("number of sites must be in 1.." + std::to_string(MAX_SITES));
    if (model == "Kitaev") {
        if (p.Ly % 2 != 0) throw std::invalid_argument("Kitaev honeycomb needs an even NumberofSitesLy");
        honeycomb(p.Lx, p.Ly, p.pbcx != 0, p.pbcy != 0, L);
    } else if (model == "HeisenbergChain") {
        chain(N, p.pbcx != 0, L);
    } else {
        throw std::invalid_argument("Unknown Model parameter");   // src/Hamiltonian.h:51-52
    }
}

// Bond families as built by Hamiltonian::Connectors (src/Hamiltonian.h:230-328) or
// HeisenbergChain_Connectors (:382-475): pairs i<j scanned row-major; a family whose coupling is
// zero is empty; a family with a single bond is skipped by TightB_Ham/Diagonal
// (`if(K_Conn.size()==1) break;`, :116, :143, :347), so it is dropped here.  Jheis (extension)
// adds J to the three couplings of every nearest-neighbour pair.
void build_bonds(const esc_params& p, const Lattice& L, std::vector<Bond>& bonds) {
    bonds.clear();
    const int N = L.N;
    const bool kitaev = std::string(p.model) == "Kitaev";
    std::vector<std::pair<int, int>> fam[3];   // x, y, z
    const double K[3] = {p.Kxx, p.Kyy, p.Kzz};
    if (kitaev) {
        const int col_of[3] = {2, 1, 0};       // x, y, z columns
        for (int f = 0; f < 3; f++) {
            if (K[f] == 0.0) continue;
            for (int i = 0; i < N; i++) {
                const int j = L.neigh[(size_t)i * 3 + col_of[f]];
                if (i < j) fam[f].push_back({i, j});
            }
        }
    } else {
        for (int f = 0; f < 3; f++) {
            if (K[f] == 0.0) continue;
            std::vector<char> seen((size_t)N * N, 0);
            for (int i = 0; i < N; i++)
                for (int c = 0; c < 2; c++) {
                    const int j = L.neigh[(size_t)i * 3 + c];
                    if (i < j) seen[(size_t)i * N + j] = 1;
                }
            for (int i = 0; i < N; i++)
                for (int j = 0; j < N; j++)
                    if (seen[(size_t)i * N + j]) fam[f].push_back({i, j});
        }
    }
    for (int f = 0; f < 3; f++) {
        if (fam[f].size() <= 1) continue;      // single-bond family dropped (see above)
        for (auto& pr : fam[f]) {
            Bond b{pr.first, pr.second, kitaev ? "xyz"[f] : 'c', 0.0, 0.0, 0.0};
            (f == 0 ? b.kx : f == 1 ? b.ky : b.kz) = K[f];
            bonds.push_back(b);
        }
    }
    if (p.jheis != 0.0) {
        for (int i = 0; i < N; i++)
            for (int j = i + 1; j < N; j++) {
                bool nn = false;
                for (int c = 0; c < L.ncol; c++) nn |= (L.neigh[(size_t)i * 3 + c] == j);
                if (!nn) continue;
                auto it = std::find_if(bonds.begin(), bonds.end(), [&](const Bond& b) { return b.i == i && b.j == j; });
                if (it != bonds.end()) { it->kx += p.jheis; it->ky += p.jheis; it->kz += p.jheis; }
                else bonds.push_back(Bond{i, j, 'n', p.jheis, p.jheis, p.jheis});
            }
    }
}

DevModel make_dev_model(const esc_params& p, const Lattice& L, const std::vector<Bond>& bonds, double Bx, double By,
                        double Bz) {
    (void)p;
    DevModel m;
    std::memset(&m, 0, sizeof(m));
    m.N = L.N;
    m.fx = 0.5 * Bx; m.fy = 0.5 * By; m.fz = 0.5 * Bz;
    for (const Bond& b : bonds) {
        const unsigned long long mask = (1ull << b.i) | (1ull << b.j);
        const double ceq = 0.25 * (b.kx - b.ky), cdiff = 0.25 * (b.kx + b.ky);
        if (ceq != 0.0 || cdiff != 0.0) {
            if (m.nb >= MAX_BONDS) throw std::invalid_argument("too many bonds");
            m.b[m.nb++] = DevBond{mask, ceq, cdiff};
        }
        if (b.kz != 0.0) {
            if (m.nd >= MAX_BONDS) throw std::invalid_argument("too many bonds");
            m.d[m.nd++] = DevDiagBond{mask, b.kz};
        }
    }
    fill_float_copies(m);
    return m;
}

void fill_float_copies(DevModel& m) {
    m.fxf = (float)m.fx; m.fyf = (float)m.fy; m.fzf = (float)m.fz;
    for (int b = 0; b < m.nb; b++) { m.ceqf[b] = (float)m.b[b].ceq; m.cdifff[b] = (float)m.b[b].cdiff; }
    for (int b = 0; b < m.nd; b++) m.dqf[b] = (float)(0.25 * m.d[b].dz);
}

// ---------------------------------------------------------------------------------------------
// Operator strings.  Each reference Apply* is a product of single-site operators applied right
// to left; the term lists below keep that order (factor 0 is applied first).
// ---------------------------------------------------------------------------------------------
namespace {
struct TB {
    const esc_params& p;
    const Lattice& L;
    std::vector<OpTerm> t;
    int nb(int i, int col) const {
        const int j = (i >= 0 && i < L.N) ? L.neigh[(size_t)i * 3 + col] : -1;
        if (j < 0) throw std::invalid_argument("operator needs a neighbour that does not exist on this cluster");
        return j;
    }
    void add(cplx c, std::initializer_list<std::pair<char, int>> f) {
        OpTerm o;
        o.coef = c; o.nf = 0;
        for (auto& x : f) { o.op[o.nf] = x.first; o.site[o.nf] = x.second; o.nf++; }
        t.push_back(o);
    }
    // src/Observables.h:243-281: Kzz Sy_i Sz_z(i) - Kyy Sz_i Sy_y(i)
    void jsx(int i) { add(p.Kzz, {{'z', nb(i, 0)}, {'y', i}}); add(-p.Kyy, {{'y', nb(i, 1)}, {'z', i}}); }
    // :202-240: Kxx Sz_i Sx_x(i) - Kzz Sx_i Sz_z(i)
    void jsy(int i) { add(p.Kxx, {{'x', nb(i, 2)}, {'z', i}}); add(-p.Kzz, {{'z', nb(i, 0)}, {'x', i}}); }
    // :161-199: Kyy Sx_i Sy_y(i) - Kxx Sy_i Sx_x(i)
    void jsz(int i) { add(p.Kyy, {{'y', nb(i, 1)}, {'x', i}}); add(-p.Kxx, {{'x', nb(i, 2)}, {'y', i}}); }
    // :358-389 (A sites): KxxKzz Sx_i Sy_ix Sz_ix+z - KxxKyy Sx_i Sz_ix Sy_ix+y
    void jex(int i) {
        const int ix = nb(i, 2), ixpy = nb(ix, 1), ixpz = nb(ix, 0);
        add(p.Kxx * p.Kzz, {{'z', ixpz}, {'y', ix}, {'x', i}});
        add(-(p.Kxx * p.Kyy), {{'y', ixpy}, {'z', ix}, {'x', i}});
    }
    // :321-354 (B sites): KxxKyy Sy_i Sz_iy Sx_iy+x - KyyKzz Sy_i Sx_iy Sz_iy+z
    void jey(int i) {
        const int iy = nb(i, 1), iypx = nb(iy, 2), iypz = nb(iy, 0);
        add(p.Kxx * p.Kyy, {{'x', iypx}, {'z', iy}, {'y', i}});
        add(-(p.Kyy * p.Kzz), {{'z', iypz}, {'x', iy}, {'y', i}});
    }
};
}  // namespace

std::vector<OpTerm> operator_terms(int op, int site, const esc_params& p, const Lattice& L) {
    TB b{p, L, {}};
    const int N = L.N;
    const bool needs_site = op >= ESC_OP_SX && op <= ESC_OP_JSXJSYJSZ;
    if (needs_site && (site < 0 || site >= N)) throw std::invalid_argument("site out of range");
    const cplx I(0.0, 1.0);
    switch (op) {
        case ESC_OP_I: b.add(1.0, {}); break;
        case ESC_OP_SX: b.add(1.0, {{'x', site}}); break;
        case ESC_OP_SY: b.add(1.0, {{'y', site}}); break;
        case ESC_OP_SZ: b.add(1.0, {{'z', site}}); break;
        case ESC_OP_SP: b.add(1.0, {{'x', site}}); b.add(I, {{'y', site}}); break;        // :524-537
        case ESC_OP_SM: b.add(1.0, {{'x', site}}); b.add(-I, {{'y', site}}); break;       // :558-571
        case ESC_OP_SPE3:                                                                 // :539-555
            b.add(cplx(-0.408248, 0.707107), {{'x', site}});
            b.add(cplx(-0.408248, -0.707107), {{'y', site}});
            b.add(0.816497, {{'z', site}});
            break;
        case ESC_OP_SME3:                                                                 // :573-589
            b.add(cplx(-0.408248, -0.707107), {{'x', site}});
            b.add(cplx(-0.408248, 0.707107), {{'y', site}});
            b.add(0.816497, {{'z', site}});
            break;
        case ESC_OP_SXSYSZ: b.add(1.0, {{'x', site}}); b.add(1.0, {{'y', site}}); b.add(1.0, {{'z', site}}); break;
        case ESC_OP_JSX: b.jsx(site); break;
        case ESC_OP_JSY: b.jsy(site); break;
        case ESC_OP_JSZ: b.jsz(site); break;
        case ESC_OP_JEX: b.jex(site); break;
        case ESC_OP_JEY: b.jey(site); break;
        case ESC_OP_JEXJEYJEZ: b.jex(site); b.jey(site); break;                           // :392-407
        case ESC_OP_JSXJSYJSZ: b.jsx(site); b.jsy(site); b.jsz(site); break;              // :410-425
        case ESC_OP_JSX_TOTAL: for (int s = 0; s < N; s++) b.jsx(s); break;               // :664-674
        case ESC_OP_JSY_TOTAL: for (int s = 0; s < N; s++) b.jsy(s); break;               // :676-686
        case ESC_OP_JSZ_TOTAL: for (int s = 0; s < N; s++) b.jsz(s); break;               // :689-699
        case ESC_OP_JEX_TOTAL: for (int s = 0; s < N; s += 2) b.jex(s); break;            // :448-458
        case ESC_OP_JEY_TOTAL: for (int s = 1; s < N; s += 2) b.jey(s); break;            // :460-470
        case ESC_OP_JS_TOTAL:                                                             // dynamics.h:247
            for (int s = 0; s < N; s++) b.jsx(s);
            for (int s = 0; s < N; s++) b.jsy(s);
            for (int s = 0; s < N; s++) b.jsz(s);
            break;
        case ESC_OP_JE_TOTAL:                                                             // dynamics.h:367
            for (int s = 0; s < N; s += 2) b.jex(s);
            for (int s = 1; s < N; s += 2) b.jey(s);
            break;
        default: throw std::invalid_argument("Unknown Operator label");                   // Observables.h:64-65
    }
    return b.t;
}

DevOp make_dev_op(const std::vector<OpTerm>& terms, const std::vector<int>* perm) {
    DevOp d;
    std::memset(&d, 0, sizeof(d));
    if ((int)terms.size() > MAX_TERMS) throw std::invalid_argument("operator has too many terms");
    d.nt = (int)terms.size();
    for (int t = 0; t < d.nt; t++) {
        const OpTerm& o = terms[t];
        unsigned long long flip = 0;
        unsigned int fac = (unsigned)o.nf;
        for (int f = 0; f < o.nf; f++) {
            const int code = o.op[f] == 'x' ? 1 : o.op[f] == 'y' ? 2 : 3;
            const int bit = perm ? (*perm)[o.site[f]] : o.site[f];
            if (code != 3) flip ^= 1ull << bit;
            fac |= (unsigned)(bit & 63) << (2 + 8 * f);
            fac |= (unsigned)code << (8 + 8 * f);
        }
        d.flip[t] = flip;
        d.fac[t] = fac;
        d.cre[t] = o.coef.real();
        d.cim[t] = o.coef.imag();
        d.cref[t] = (float)o.coef.real();
        d.cimf[t] = (float)o.coef.imag();
    }
    return d;
}

}  // namespace esc
