// planner.cpp -- site relabelling and pass plan for the tiled H.v (hv_tiled.cu).
//
// The basis index has one bit per site.  A tile is the set of 2^T basis states that differ only in
// T chosen bit positions; a term of H (a bond flips two bits, a field term one) can be applied
// inside a tile held in shared memory when all its flipped bits are tile bits.  The planner
//   1. picks c "shared" sites that are tile bits of every pass (the lowest index bits, so every
//      tile is made of runs of 2^c consecutive states: coalesced loads),
//   2. covers every bond by clusters of at most T-c further sites (greedy growth that maximises
//      newly covered bonds, many random restarts, keeps the fewest passes), then looks for a
//      covering with one cluster less at a time by simulated annealing,
//   3. numbers the sites so that pass 1 is the contiguous block of the T lowest bits and each later
//      pass's new sites are contiguous too,
//   4. assigns every term to the first pass whose tile contains it (the diagonal to pass 1),
//   5. from 27 sites on, orders the passes in pairs whose tiles span few bits together, for the
//      slab-pair launches of hv_tiled.cu.
// The relabelled model is the same Hamiltonian; only vectors crossing the C ABI are permuted.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>
#include <random>
#include <set>
#include <string>

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

// exp(x) for x <= 0 from basic IEEE operations only (Taylor series of exp(x / 64), squared six
// times), so that the planner makes the same choices on every host.
double exp_basic(double x) {
    const double y = x / 64.0;
    double t = 1.0, s = 1.0;
    for (int k = 1; k <= 10; k++) { t = t * y / k; s += t; }
    for (int k = 0; k < 6; k++) s *= s;
    return s;
}

// Annealed covering with a fixed number of passes P: c shared sites plus P clusters of exactly T-c
// further sites each; the cost is the number of bonds that lie in no tile plus the number of sites
// in none.  Moves: swap one cluster site for an outside site (biased towards the ends of uncovered
// bonds), or swap a shared site with another site.  Only the bonds at the moved sites are
// re-examined, so a move costs O(P x degree).  Returns an empty candidate when no zero-cost
// covering is reached within the budget.
Cand anneal(int N, int T, int c, int P, const std::vector<std::pair<int, int>>& bonds,
            const std::vector<std::vector<int>>& adj, std::mt19937_64& rng, long iters) {
    const int free = T - c, B = (int)bonds.size();
    if (free <= 0 || c + P * free < N) return {};
    std::vector<std::vector<int>> inc(N);   // bonds at each site
    for (int b = 0; b < B; b++) { inc[bonds[b].first].push_back(b); inc[bonds[b].second].push_back(b); }
    std::uniform_real_distribution<double> U01(0.0, 1.0);
    auto rnd = [&](int n) { return std::uniform_int_distribution<int>(0, n - 1)(rng); };
    std::vector<char> inC(N, 0);
    std::vector<std::vector<char>> inS(P, std::vector<char>(N, 0));
    std::vector<std::vector<int>> S(P);
    // initial state: shared sites along a random path, clusters grown breadth-first from random seeds
    if (c > 0) {
        int s0 = rnd(N);
        std::vector<int> C{s0};
        inC[s0] = 1;
        while ((int)C.size() < c) {
            std::vector<int> nb;
            for (int x : C) for (int y : adj[x]) if (!inC[y]) nb.push_back(y);
            int y = nb.empty() ? rnd(N) : nb[rnd((int)nb.size())];
            if (!inC[y]) { inC[y] = 1; C.push_back(y); }
        }
    }
    for (int p = 0; p < P; p++) {
        std::vector<int> q{rnd(N)};
        for (size_t h = 0; h < q.size() && (int)S[p].size() < free; h++) {
            const int x = q[h];
            if (inC[x] || inS[p][x]) continue;
            inS[p][x] = 1;
            S[p].push_back(x);
            for (int y : adj[x]) q.push_back(y);
        }
        while ((int)S[p].size() < free) {
            const int x = rnd(N);
            if (!inC[x] && !inS[p][x]) { inS[p][x] = 1; S[p].push_back(x); }
        }
    }
    auto in_tile = [&](int p, int x) { return inC[x] || inS[p][x]; };
    std::vector<int> bcov(B, 0), scov(N, 0);
    for (int b = 0; b < B; b++)
        for (int p = 0; p < P; p++) bcov[b] += in_tile(p, bonds[b].first) && in_tile(p, bonds[b].second);
    for (int x = 0; x < N; x++) scov[x] = inC[x] ? P : 0;
    for (int p = 0; p < P; p++) for (int x : S[p]) scov[x]++;
    int cost = 0;
    for (int b = 0; b < B; b++) cost += bcov[b] == 0;
    for (int x = 0; x < N; x++) cost += scov[x] == 0;
    // re-examine the bonds at the given sites (each once); returns the cost change
    std::vector<int> mark(B, -1);
    int stamp = 0;
    auto refresh = [&](const int* xs, int nx) {
        int d = 0;
        stamp++;
        for (int i = 0; i < nx; i++)
            for (int b : inc[xs[i]]) {
                if (mark[b] == stamp) continue;
                mark[b] = stamp;
                int n = 0;
                for (int p = 0; p < P; p++) n += in_tile(p, bonds[b].first) && in_tile(p, bonds[b].second);
                d += (n == 0) - (bcov[b] == 0);
                bcov[b] = n;
            }
        return d;
    };
    std::vector<int> open_ends;
    const double t0 = 0.6, log_t1_t0 = -2.995732273553991;   // final temperature 0.03 = 0.05 t0
    for (long it = 0; it < iters && cost > 0; it++) {
        const double temp = t0 * exp_basic(log_t1_t0 * (double)it / (double)iters);
        if (c > 0 && rnd(20) == 0) {
            // swap shared site a with outside site b: b leaves every cluster it was in, and a takes
            // its place there (cluster sizes are kept)
            int ai = rnd(N), bi = rnd(N);
            if (!inC[ai] || inC[bi]) continue;
            std::vector<int> had;
            for (int p = 0; p < P; p++) if (inS[p][bi]) had.push_back(p);
            auto apply = [&](int a, int b2, bool fwd) {
                inC[a] = 0; inC[b2] = 1;
                for (int p : had) {
                    if (fwd) { inS[p][bi] = 0; inS[p][ai] = 1; std::replace(S[p].begin(), S[p].end(), bi, ai); }
                    else { inS[p][ai] = 0; inS[p][bi] = 1; std::replace(S[p].begin(), S[p].end(), ai, bi); }
                }
            };
            auto site_cost = [&](int x) { return scov[x] == 0 ? 1 : 0; };
            const int before = site_cost(ai) + site_cost(bi);
            apply(ai, bi, true);
            const int sa = scov[ai], sb = scov[bi];
            scov[ai] = (int)had.size();
            scov[bi] = P;
            const int xs[2] = {ai, bi};
            const int d = refresh(xs, 2) + site_cost(ai) + site_cost(bi) - before;
            if (d <= 0 || U01(rng) < exp_basic(-d / temp)) { cost += d; continue; }
            apply(bi, ai, false);
            inC[bi] = 0; inC[ai] = 1;
            scov[ai] = sa; scov[bi] = sb;
            refresh(xs, 2);
            continue;
        }
        const int p = rnd(P);
        const int xi = rnd(free), x = S[p][xi];
        int y = -1;
        if (rnd(3) != 0) {
            open_ends.clear();
            for (int b = 0; b < B; b++)
                if (bcov[b] == 0) {
                    const int i = bonds[b].first, j = bonds[b].second;
                    if (!in_tile(p, i)) open_ends.push_back(i);
                    if (!in_tile(p, j)) open_ends.push_back(j);
                }
            for (int z = 0; z < N; z++) if (scov[z] == 0) open_ends.push_back(z);
            if (!open_ends.empty()) y = open_ends[rnd((int)open_ends.size())];
        }
        if (y < 0) {
            // a neighbour of the cluster
            const int z = S[p][rnd(free)];
            y = adj[z].empty() ? rnd(N) : adj[z][rnd((int)adj[z].size())];
        }
        if (inC[y] || inS[p][y]) continue;
        const int before = (scov[x] == 0) + (scov[y] == 0);
        inS[p][x] = 0; inS[p][y] = 1; S[p][xi] = y;
        scov[x]--; scov[y]++;
        const int xs[2] = {x, y};
        const int d = refresh(xs, 2) + (scov[x] == 0) + (scov[y] == 0) - before;
        if (d <= 0 || U01(rng) < exp_basic(-d / temp)) { cost += d; continue; }
        inS[p][y] = 0; inS[p][x] = 1; S[p][xi] = x;
        scov[x]++; scov[y]--;
        refresh(xs, 2);
    }
    if (cost > 0) return {};
    Cand r;
    for (int x = 0; x < N; x++) if (inC[x]) r.C.push_back(x);
    r.S = S;
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

namespace {
Plan search_plan(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts, bool anneal_more);
}

// The search is deterministic (fixed seed) but takes seconds from 26 sites, and handle creation, the
// self-tuner and the tuning file ask for the same plans again: results are kept per process, keyed
// by everything the search reads.
Plan make_plan(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts) {
    if (N >= 26) restarts = std::max(restarts, 20000);   // large bases: fewer passes are worth ~3 s here
    if (const char* e = std::getenv("ESC_PLAN_RESTARTS")) restarts = std::max(1, std::atoi(e));
    const char* greedy_only = std::getenv("ESC_PLAN_GREEDY");
    const bool anneal_more = !greedy_only || std::atoi(greedy_only) == 0;
    std::string key = std::to_string(N) + "/" + std::to_string(T) + "/" + std::to_string(c) + "/" +
                      std::to_string(restarts) + "/" + (anneal_more ? "a" : "g") + ":";
    for (const auto& b : bonds) key += std::to_string(b.first) + "," + std::to_string(b.second) + ";";
    static std::mutex mu;
    static std::map<std::string, Plan> cache;
    {
        std::lock_guard<std::mutex> lk(mu);
        const auto it = cache.find(key);
        if (it != cache.end()) {
            Plan P = it->second;
            order_for_pairs(P);
            return P;
        }
    }
    Plan P = search_plan(N, bonds, T, c, restarts, anneal_more);
    {
        std::lock_guard<std::mutex> lk(mu);
        cache.emplace(key, P);
    }
    order_for_pairs(P);
    return P;
}

int slab_pairs_env() {
    const char* e = std::getenv("ESC_SLAB_PAIRS");
    if (!e || !*e) return -1;
    return std::atoi(e) != 0 ? 1 : 0;
}

// Pairs of passes for the slab-pair launches: the matching with the most pairs spanning at most
// SLAB_MAX_BITS bits, then the fewest bits in total (every matching of the at most a few passes is
// tried).  New order: the pair holding the first pass (first pass first), the other pairs, then the
// passes left alone.  The first pass keeps the diagonal, and every pass keeps its tile, so only
// the pass each term is assigned to (the first that holds it) and the order of the additions change.
void order_for_pairs(Plan& P) {
    const int np = (int)P.tiles.size();
    if (np < 2 || np > 12 || (P.N < SLAB_MIN_SITES && slab_pairs_env() < 0)) return;
    std::vector<unsigned long long> tm(np, 0);
    for (int i = 0; i < np; i++)
        for (int b : P.tiles[i]) tm[i] |= 1ull << b;
    auto ubits = [&](int a, int b) { return __builtin_popcountll(tm[a] | tm[b]); };
    std::vector<int> mate(np, -1), best_mate(np, -1);
    int best_pairs = -1, best_bits = 1 << 30;
    std::function<void(int, int, int)> rec = [&](int i, int pairs, int bits) {
        while (i < np && mate[i] != -1) i++;
        if (i == np) {
            if (pairs > best_pairs || (pairs == best_pairs && bits < best_bits)) {
                best_pairs = pairs;
                best_bits = bits;
                best_mate = mate;
            }
            return;
        }
        mate[i] = i;   // alone
        rec(i + 1, pairs, bits);
        for (int j = i + 1; j < np; j++)
            if (mate[j] == -1 && ubits(i, j) <= SLAB_MAX_BITS) {
                mate[i] = j;
                mate[j] = i;
                rec(i + 1, pairs + 1, bits + ubits(i, j));
                mate[j] = -1;
            }
        mate[i] = -1;
    };
    rec(0, 0, 0);
    if (best_pairs <= 0) return;
    std::vector<int> order;
    std::vector<char> used(np, 0);
    auto take = [&](int i) { order.push_back(i); used[i] = 1; };
    take(0);
    if (best_mate[0] != 0) take(best_mate[0]);
    for (int i = 1; i < np; i++)
        if (!used[i] && best_mate[i] != i) { take(i); take(best_mate[i]); }
    for (int i = 1; i < np; i++)
        if (!used[i]) take(i);
    std::vector<std::vector<int>> tiles;
    for (int i : order) tiles.push_back(P.tiles[i]);
    P.tiles = tiles;
}

namespace {

Plan search_plan(int N, const std::vector<std::pair<int, int>>& bonds, int T, int c, int restarts, bool anneal_more) {
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
    std::mt19937_64 rng(0x5eed1234u);
    Cand best;
    size_t best_cost = ~size_t(0);
    for (int t = 0; t < restarts; t++) {
        Cand cd = greedy(N, T, c, bonds, adj, rng);
        size_t cost = cd.S.size() * 1000;
        for (auto& s : cd.S) cost += s.size();
        if (cost < best_cost) { best_cost = cost; best = cd; }
    }
    // fewer passes than the greedy covering: annealed coverings with one pass less at a time
    if (anneal_more)
        for (int np = (int)best.S.size() - 1; np >= 1; np--) {
            Cand a;
            for (int t = 0; t < 8 && a.S.empty(); t++) a = anneal(N, T, c, np, bonds, adj, rng, 400000);
            if (a.S.empty()) break;
            best = a;
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

}  // namespace

}  // namespace esc
