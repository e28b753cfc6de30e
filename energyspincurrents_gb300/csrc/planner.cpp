// planner.cpp -- site relabelling and pass plan for the tiled H.v (hv_tiled.cu).
//
// The basis index has one bit per site.  A tile is the set of 2^T basis states that differ only in
// T chosen bit positions; a term of H (a bond flips two bits, a field term one) can be applied
// inside a tile held in shared memory when all its flipped bits are tile bits.  The planner
//   1. picks c "shared" sites that are tile bits of every pass (the lowest index bits, so every
//      tile is made of runs of 2^c consecutive states: coalesced loads),
//   2. covers every bond by clusters of at most T-c further sites (greedy growth that maximises
//      newly covered bonds, many random restarts, keeps the fewest passes),
//   3. numbers the sites so that pass 1 is the contiguous block of the T lowest bits and each later
//      pass's new sites are contiguous too,
//   4. assigns every term to the first pass whose tile contains it (the diagonal to pass 1).
// The relabelled model is the same Hamiltonian; only vectors crossing the C ABI are permuted.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <random>
#include <set>

#include "esc_internal.h"

namespace esc {

namespace {

struct Cand {
    std::vector<int> C;
    std::vector<std::vector<int>> S;
};

Cand greedy(int N, int T, int c, const std::vector<std::pair<int, int>>& bonds, const std::vector<std::vector<int>>& adj,
            std::mt19937_64& rng, bool low_sites_shared = false) {
    Cand r;
    std::vector<char> inC(N, 0), covered_site(N, 0);
    if (low_sites_shared) {
        // shared sites fixed to 0..c-1 (identity labelling: the reference basis order)
        for (int i = 0; i < c; i++) { r.C.push_back(i); inC[i] = 1; covered_site[i] = 1; }
    } else {
        // shared sites: a BFS path from a random start
        std::uniform_int_distribution<int> U(0, N - 1);
        int s = U(rng);
        std::vector<int> q{s};
        std::vector<char> seen(N, 0);
        seen[s] = 1;
        for (size_t h = 0; h < q.size() && (int)r.C.size() < c; h++) {
            r.C.push_back(q[h]);
            std::vector<int> nb = adj[q[h]];
            std::shuffle(nb.begin(), nb.end(), rng);
            for (int x : nb) if (!seen[x]) { seen[x] = 1; q.push_back(x); }
        }
        for (int i = 0; (int)r.C.size() < c && i < N; i++)
            if (std::find(r.C.begin(), r.C.end(), i) == r.C.end()) r.C.push_back(i);
        for (int x : r.C) { inC[x] = 1; covered_site[x] = 1; }
    }
    std::vector<char> bcov(bonds.size(), 0);
    for (size_t b = 0; b < bonds.size(); b++) bcov[b] = inC[bonds[b].first] && inC[bonds[b].second];
    const int budget = T - c;
    while (true) {
        std::vector<int> open_b;
        for (size_t b = 0; b < bonds.size(); b++) if (!bcov[b]) open_b.push_back((int)b);
        std::vector<int> open_s;
        for (int i = 0; i < N; i++) if (!covered_site[i]) open_s.push_back(i);
        if (open_b.empty() && open_s.empty()) break;
        std::vector<char> inS(N, 0);
        std::vector<int> S;
        int seed;
        if (!open_b.empty()) {
            const auto& bb = bonds[open_b[std::uniform_int_distribution<int>(0, (int)open_b.size() - 1)(rng)]];
            seed = inC[bb.first] ? bb.second : bb.first;
        } else {
            seed = open_s[std::uniform_int_distribution<int>(0, (int)open_s.size() - 1)(rng)];
        }
        S.push_back(seed); inS[seed] = 1;
        while ((int)S.size() < budget) {
            // candidate gain: uncovered bonds closed by adding x, plus half a point for an uncovered site
            double best = -1; std::vector<int> bestx;
            std::set<int> cand;
            for (int s : S) for (int x : adj[s]) if (!inS[x] && !inC[x]) cand.insert(x);
            for (int x : r.C) for (int y : adj[x]) if (!inS[y] && !inC[y]) cand.insert(y);
            if (cand.empty()) for (int i = 0; i < N; i++) if (!inS[i] && !inC[i]) cand.insert(i);
            if (cand.empty()) break;
            for (int x : cand) {
                double g = covered_site[x] ? 0.0 : 0.5;
                for (size_t b = 0; b < bonds.size(); b++) {
                    if (bcov[b]) continue;
                    int i = bonds[b].first, j = bonds[b].second;
                    if ((i == x && (inS[j] || inC[j])) || (j == x && (inS[i] || inC[i]))) g += 1.0;
                }
                if (g > best + 1e-12) { best = g; bestx.assign(1, x); }
                else if (std::abs(g - best) <= 1e-12) bestx.push_back(x);
            }
            int x = bestx[std::uniform_int_distribution<int>(0, (int)bestx.size() - 1)(rng)];
            S.push_back(x); inS[x] = 1;
        }
        for (size_t b = 0; b < bonds.size(); b++) {
            int i = bonds[b].first, j = bonds[b].second;
            if ((inS[i] || inC[i]) && (inS[j] || inC[j])) bcov[b] = 1;
        }
        for (int x : S) covered_site[x] = 1;
        r.S.push_back(S);
        if ((int)r.S.size() > 64) break;
    }
    return r;
}

}  // namespace

Plan make_plan_reference_order(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts) {
    Plan P;
    P.N = N;
    P.perm.resize(N);
    std::iota(P.perm.begin(), P.perm.end(), 0);
    if (N <= T) {
        P.T = N; P.c = std::min(c, N);
        P.tiles.push_back(P.perm);
        return P;
    }
    P.T = T; P.c = c;
    std::vector<std::vector<int>> adj(N);
    for (auto& b : bonds) { adj[b.first].push_back(b.second); adj[b.second].push_back(b.first); }
    std::mt19937_64 rng(0x5eed1234u);
    Cand best;
    size_t best_cost = ~size_t(0);
    for (int t = 0; t < restarts; t++) {
        Cand cd = greedy(N, T, c, bonds, adj, rng, true);
        size_t cost = cd.S.size() * 1000;
        for (auto& s : cd.S) cost += s.size();
        if (cost < best_cost) { best_cost = cost; best = cd; }
    }
    for (auto& S : best.S) {
        std::vector<int> bits(best.C);
        bits.insert(bits.end(), S.begin(), S.end());
        std::sort(bits.begin(), bits.end());
        P.tiles.push_back(bits);
    }
    return P;
}

Plan make_plan(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts) {
    Plan P;
    P.N = N;
    if (N <= T) {
        // one tile holds the whole vector: identity labels, one pass
        P.T = N; P.c = std::min(c, N);
        P.perm.resize(N);
        std::iota(P.perm.begin(), P.perm.end(), 0);
        std::vector<int> all(N);
        std::iota(all.begin(), all.end(), 0);
        P.tiles.push_back(all);
        return P;
    }
    P.T = T; P.c = c;
    std::vector<std::vector<int>> adj(N);
    for (auto& b : bonds) { adj[b.first].push_back(b.second); adj[b.second].push_back(b.first); }
    if (N >= 26) restarts = std::max(restarts, 20000);   // large bases: fewer passes are worth ~3 s here
    if (const char* e = std::getenv("ESC_PLAN_RESTARTS")) restarts = std::max(1, std::atoi(e));
    std::mt19937_64 rng(0x5eed1234u);
    Cand best;
    size_t best_cost = ~size_t(0);
    for (int t = 0; t < restarts; t++) {
        Cand cd = greedy(N, T, c, bonds, adj, rng);
        size_t cost = cd.S.size() * 1000;
        for (auto& s : cd.S) cost += s.size();
        if (cost < best_cost) { best_cost = cost; best = cd; }
    }
    // bit numbering: shared sites -> [0,c), first cluster -> [c, c+|S1|), later clusters' new sites next
    P.perm.assign(N, -1);
    int nextbit = 0;
    for (int x : best.C) P.perm[x] = nextbit++;
    for (auto& S : best.S)
        for (int x : S)
            if (P.perm[x] < 0) P.perm[x] = nextbit++;
    for (int i = 0; i < N; i++) if (P.perm[i] < 0) P.perm[i] = nextbit++;
    for (auto& S : best.S) {
        std::vector<int> bits;
        for (int x : best.C) bits.push_back(P.perm[x]);
        for (int x : S) bits.push_back(P.perm[x]);
        std::sort(bits.begin(), bits.end());
        P.tiles.push_back(bits);
    }
    return P;
}

}  // namespace esc
