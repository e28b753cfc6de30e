// Host-side check of the slab-pair launch arithmetic (test infrastructure, built by
// tests/test_slab_pair_indexing.py; runs on the CPU, no GPU needed).
//
// For a honeycomb cluster and tile size it builds the library's plan and passes with slab pairs
// enabled, and for every pair replays, item by item, the index arithmetic of pair_body
// (hv_pass_device.cuh): the item order (pair_item), the tile number -> global bits tables built in
// shared memory, the per-thread state offsets and the 16-byte tile copies.  It checks that every
// state is written exactly once by each pass of the pair, that a tile of pass B only reads states
// that pass A wrote in the same slab, that every tile of A(s) comes before every tile of B(s) in the
// item order (so the waits can always be satisfied), and that every address is inside the vector.
//
//     slab_pair_check Lx Ly tile_bits tb_bits     -> one line per pair, "OK" or the failure
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "esc_internal.h"
#include "hv_pass_device.cuh"

using namespace esc;

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: slab_pair_check Lx Ly tile_bits tb_bits\n");
        return 2;
    }
    const int Lx = std::atoi(argv[1]), Ly = std::atoi(argv[2]), T = std::atoi(argv[3]), tb = std::atoi(argv[4]);
    setenv("ESC_SLAB_PAIRS", "1", 1);
    esc_params p;
    std::memset(&p, 0, sizeof p);
    esc_params_default(&p);
    p.Lx = Lx;
    p.Ly = Ly;
    p.Kxx = p.Kyy = p.Kzz = -1.0;
    p.jheis = 0.05;
    p.Bxx = p.Byy = p.Bzz = 0.02;
    Lattice L;
    std::vector<Bond> bonds;
    build_lattice(p, L);
    build_bonds(p, L, bonds);
    std::vector<std::pair<int, int>> pairs;
    for (const auto& b : bonds)
        if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
    const Plan P = make_plan(L.N, pairs, T, 3, 200);
    std::vector<Bond> rb(bonds);
    for (auto& b : rb) { b.i = P.perm[b.i]; b.j = P.perm[b.j]; }
    const DevModel m = make_dev_model(p, L, rb, p.Bxx, p.Byy, p.Bzz);
    const std::vector<DevPass> ps = make_passes(P, m, 2, 2, tb);
    const int N = L.N;
    const long long D = 1ll << N;
    const int TB = 1 << tb, E = 1 << (T - tb);
    std::vector<unsigned> sync(slab_sync_words(N), 0u);
    int npairs = 0, fails = 0;
    for (size_t i = 0; i + 1 < ps.size(); i++) {
        if (!ps[i].pair) continue;
        npairs++;
        const escdev::PairTab st = make_pair_tab(ps[i], ps[i + 1], N, sync.data());
        const escdev::PassTab pt[2] = {make_pass_tab(ps[i], m), make_pass_tab(ps[i + 1], m)};
        // the shared-memory tables of pair_body
        unsigned long long lut[2][5][64];
        for (int x = 0; x < 2; x++)
            for (int c = 0; c < 5; c++)
                for (int v = 0; v < 64; v++) {
                    unsigned long long b = 0;
                    for (int q = 0; q < 6; q++)
                        if (6 * c + q < st.nrest && ((v >> q) & 1)) b |= 1ull << st.rest[x][6 * c + q];
                    lut[x][c][v] = b;
                }
        auto tile_of = [&](int x, long long t) {
            return lut[x][0][t & 63] | lut[x][1][(t >> 6) & 63] | lut[x][2][(t >> 12) & 63] | lut[x][3][(t >> 18) & 63] |
                   lut[x][4][(t >> 24) & 63];
        };
        const long long total = (2 * st.nslab) << st.inner;
        std::vector<unsigned char> written[2] = {std::vector<unsigned char>(D, 0), std::vector<unsigned char>(D, 0)};
        std::vector<int> slab_of(D, -1);
        std::vector<long long> lastA(st.nslab, -1), firstB(st.nslab, 1ll << 62);
        long long bad_addr = 0, bad_slab = 0, bad_item = 0;
        for (long long k = 0; k < total; k++) {
            int sec;
            long long s, t;
            escdev::pair_item(st, k, sec, s, t);
            if (s < 0 || s >= st.nslab || t < 0 || t >= (st.nslab << st.inner)) { bad_item++; continue; }
            if (sec == 0) lastA[s] = std::max(lastA[s], k);
            else firstB[s] = std::min(firstB[s], k);
            const escdev::PassTab& px = pt[sec];
            const unsigned long long b = tile_of(sec, t);
            for (int tid = 0; tid < TB; tid++) {
                const unsigned long long base = b | px.tabLo[(tid >> 3) & 63] | px.tabHi[tid >> 9] | (unsigned long long)(tid & 7);
                for (int j = 0; j < E; j++) {
                    const unsigned long long kk = base | px.tabLo[((TB * j) >> 3) & 63] | px.tabHi[(TB * j) >> 9];
                    if (kk >= (unsigned long long)D) { bad_addr++; continue; }
                    written[sec][kk]++;
                    if (sec == 0) slab_of[kk] = (int)s;
                    else if (slab_of[kk] != (int)s) bad_slab++;
                }
                for (int c = 0; c < E / 2; c++) {   // 16-byte copies of states 2q, 2q+1
                    const unsigned long long l0 = px.tabLo[(tid >> 2) & 63] | (unsigned long long)((2 * tid) & 7);
                    const unsigned long long l1 = px.tabLo[((tid >> 2) + 32) & 63] | (unsigned long long)((2 * tid) & 7);
                    const unsigned long long a = b | ((TB == 128 && (c & 1)) ? l1 : l0) | px.tabHi[(tid + TB * c) >> 8];
                    if (a + 1 >= (unsigned long long)D || (a & 1)) bad_addr++;
                }
            }
        }
        long long not_once = 0, order = 0;
        for (long long x = 0; x < D; x++) not_once += (written[0][x] != 1) + (written[1][x] != 1);
        for (long long s = 0; s < st.nslab; s++) order += !(lastA[s] < firstB[s]);
        const bool ok = !bad_addr && !bad_slab && !bad_item && !not_once && !order &&
                        (size_t)(SLAB_CNT0 + st.nslab) <= sync.size();
        fails += !ok;
        std::printf("pair %zu,%zu U=%d slabs=%lld items=%lld: %s (addr %lld, slab %lld, item %lld, not-once %lld, order %lld)\n",
                    i, i + 1, ps[i].slab_bits, st.nslab, total, ok ? "OK" : "FAIL", bad_addr, bad_slab, bad_item, not_once,
                    order);
    }
    std::printf("N=%d T=%d passes=%zu pairs=%d\n", N, T, ps.size(), npairs);
    return fails ? 1 : (npairs ? 0 : 3);
}
