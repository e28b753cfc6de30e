// permute.cu -- basis permutations between the reference order (bit s = site s) and the
// library's internal order (the planner's site relabelling), used at the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "esc_internal.h"

namespace esc {

template <typename R> struct PV2;
template <> struct PV2<double> { typedef double2 T; };
template <> struct PV2<float> { typedef float2 T; };

// ---------------------------------------------------------------------------------------------
// Basis permutation (reference order <-> internal order)
// ---------------------------------------------------------------------------------------------
DevPerm make_perm_table(const std::vector<int>& src_bit_of_dst_bit) {
    DevPerm t;
    std::memset(&t, 0, sizeof(t));
    const int N = (int)src_bit_of_dst_bit.size();
    for (int chunk = 0; chunk < 5; chunk++)
        for (int v = 0; v < 256; v++) {
            unsigned long long s = 0;
            for (int q = 0; q < 8; q++) {
                const int b = chunk * 8 + q;
                if (b < N && ((v >> q) & 1)) s |= 1ull << src_bit_of_dst_bit[b];
            }
            t.tab[chunk][v] = s;
        }
    t.N = N;
    for (int b = 0; b < N; b++) t.sb[b] = (signed char)src_bit_of_dst_bit[b];
    return t;
}

// Tiled bit permutation: a tile is 2^n states spanning the 5 lowest src bits and the 5 lowest dst
// bits (plus further low dst bits up to n), so that both the reads (runs over src bits 0..4) and
// the writes (runs over dst bits 0..4) move contiguous 32-state runs; the tile is transposed
// through shared memory.
struct PermTile {
    int n, nrest;
    unsigned long long rd_off[12];   // src offset of read-order tile bit m
    unsigned long long wr_off[12];   // dst offset of write-order tile bit m
    int wr_idx[12];                  // read-order position of write-order tile bit m
    unsigned char rest[MAX_SITES];   // dst bit positions of the tile number, ascending
};

static PermTile make_perm_tile(const DevPerm& p, int nmax) {
    PermTile t;
    std::memset(&t, 0, sizeof(t));
    const int N = p.N;
    std::vector<int> db(N);
    for (int q = 0; q < N; q++) db[p.sb[q]] = q;
    std::vector<int> rd;
    auto add = [&](int q) {
        if ((int)rd.size() < nmax && std::find(rd.begin(), rd.end(), q) == rd.end()) rd.push_back(q);
    };
    for (int s = 0; s < std::min(N, 5); s++) add(db[s]);      // contiguous reads
    for (int q = 0; q < N; q++) add(q);                        // contiguous writes, then low dst bits
    t.n = (int)rd.size();
    std::vector<int> wr(rd);
    std::sort(wr.begin(), wr.end());
    for (int m = 0; m < t.n; m++) {
        t.rd_off[m] = 1ull << p.sb[rd[m]];
        t.wr_off[m] = 1ull << wr[m];
        t.wr_idx[m] = (int)(std::find(rd.begin(), rd.end(), wr[m]) - rd.begin());
    }
    for (int q = 0; q < N; q++)
        if (std::find(rd.begin(), rd.end(), q) == rd.end()) t.rest[t.nrest++] = (unsigned char)q;
    return t;
}

static constexpr int PERM_BITS = 11;   // tile of 2048 states: 8 per thread, all loads in flight at once

template <typename R>
__global__ void __launch_bounds__(256) k_permute_tiled(const __grid_constant__ DevPerm p, const __grid_constant__ PermTile pt,
                                                       const typename PV2<R>::T* __restrict__ in,
                                                       typename PV2<R>::T* __restrict__ out, long long ntiles) {
    typedef typename PV2<R>::T C;
    constexpr int T = 1 << PERM_BITS, PER = T / 256;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);   // T + T/32 slots: one padding slot per 32 states
    // per-thread offsets are the same for every tile
    unsigned long long roff[PER], woff[PER];
    int widx[PER];
#pragma unroll
    for (int i = 0; i < PER; i++) {
        const int e = threadIdx.x + 256 * i;
        roff[i] = 0;
        woff[i] = 0;
        widx[i] = 0;
        for (int m = 0; m < PERM_BITS; m++)
            if ((e >> m) & 1) {
                roff[i] |= pt.rd_off[m];
                woff[i] |= pt.wr_off[m];
                widx[i] |= 1 << pt.wr_idx[m];
            }
    }
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned long long b = 0;
        for (int q = 0; q < pt.nrest; q++) b |= (((unsigned long long)t >> q) & 1ull) << pt.rest[q];
        const unsigned long long a = p.tab[0][b & 255] | p.tab[1][(b >> 8) & 255] | p.tab[2][(b >> 16) & 255] |
                                     p.tab[3][(b >> 24) & 255] | p.tab[4][(b >> 32) & 255];
        C x[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) x[i] = in[a | roff[i]];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int e = threadIdx.x + 256 * i;
            buf[e + (e >> 5)] = x[i];
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < PER; i++) x[i] = buf[widx[i] + (widx[i] >> 5)];
#pragma unroll
        for (int i = 0; i < PER; i++) out[b | woff[i]] = x[i];
        __syncthreads();
    }
}

template <typename R>
__global__ void __launch_bounds__(256) k_permute(const __grid_constant__ DevPerm p, const typename PV2<R>::T* __restrict__ in,
                                                 typename PV2<R>::T* __restrict__ out, long long D) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < D; j += stride) {
        const unsigned long long u = (unsigned long long)j;
        const unsigned long long src = p.tab[0][u & 255] | p.tab[1][(u >> 8) & 255] | p.tab[2][(u >> 16) & 255] |
                                       p.tab[3][(u >> 24) & 255] | p.tab[4][(u >> 32) & 255];
        out[j] = in[src];
    }
}

template <typename R>
void launch_permute(const DevPerm& p, const void* in, void* out, int64_t D, cudaStream_t s) {
    typedef typename PV2<R>::T C;
    if (p.N >= PERM_BITS && (int64_t(1) << p.N) == D) {
        const PermTile pt = make_perm_tile(p, PERM_BITS);
        const long long ntiles = (long long)(D >> pt.n);
        const long long g = std::min<long long>(ntiles, 152 * 8);
        const size_t smem = ((size_t(1) << pt.n) + (size_t(1) << pt.n) / 32) * sizeof(C);
        k_permute_tiled<R><<<(unsigned)g, 256, smem, s>>>(p, pt, (const C*)in, (C*)out, ntiles);
        ESC_CUDA(cudaGetLastError());
        return;
    }
    long long g = (D + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_permute<R><<<(unsigned)g, 256, 0, s>>>(p, (const C*)in, (C*)out, (long long)D);
    ESC_CUDA(cudaGetLastError());
}

template void launch_permute<double>(const DevPerm&, const void*, void*, int64_t, cudaStream_t);
template void launch_permute<float>(const DevPerm&, const void*, void*, int64_t, cudaStream_t);

}  // namespace esc
