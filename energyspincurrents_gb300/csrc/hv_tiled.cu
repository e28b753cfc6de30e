// hv_tiled.cu -- shared-memory tiled H.v for sm_103a.
//
// One launch per pass of the plan (planner.cpp).  A CTA owns one tile at a time: the 2^Tp basis
// states that differ only in the pass's tile bits.  It loads the tile (runs of 2^c consecutive
// states) into shared memory, applies every term assigned to the pass by gathering partners from
// shared memory, and writes (pass 1) or accumulates (later passes) the result.  Coefficients come
// from the tile-local bits; the diagonal (pass 1) from the global index.  Each output element is
// written by one thread: no atomics, deterministic.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "esc_internal.h"
#include "hv_pass_device.cuh"

namespace esc {

template <typename R> struct V2T;
template <> struct V2T<double> { typedef double2 T; };
template <> struct V2T<float> { typedef float2 T; };

static constexpr int TILE_THREADS = 512;

template <typename R>
__global__ void __launch_bounds__(TILE_THREADS) k_hv_pass(const __grid_constant__ DevModel m,
                                                           const __grid_constant__ DevPass p,
                                                           const typename V2T<R>::T* __restrict__ in,
                                                           typename V2T<R>::T* __restrict__ out,
                                                           long long ntiles, const int* __restrict__ active) {
    typedef typename V2T<R>::T C;
    if (active && *active == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tile = reinterpret_cast<C*>(smem_raw);
    const int Tn = 1 << p.Tp;
    const int cm = (1 << p.c) - 1;
    constexpr bool F32 = sizeof(R) == 4;
    const R fx = F32 ? (R)m.fxf : (R)m.fx, fy = F32 ? (R)m.fyf : (R)m.fy;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned long long base = 0;
        for (int q = 0; q < p.nrest; q++) base |= (((unsigned long long)t >> q) & 1ull) << p.rest[q];
        for (int e = threadIdx.x; e < Tn; e += blockDim.x) {
            const int r = e >> p.c;
            const unsigned long long k = base | p.tabLo[r & 63] | p.tabHi[r >> 6] | (unsigned long long)(e & cm);
            tile[e] = in[k];
        }
        __syncthreads();
        for (int e = threadIdx.x; e < Tn; e += blockDim.x) {
            const int r = e >> p.c;
            const unsigned long long k = base | p.tabLo[r & 63] | p.tabHi[r >> 6] | (unsigned long long)(e & cm);
            R ar = 0, ai = 0;
            if (p.diag) {
                R dg;
                if constexpr (F32) {
                    float d = 0.0f;
                    for (int b = 0; b < m.nd; b++) d += (__popcll(k & m.d[b].mask) == 1) ? -m.dqf[b] : m.dqf[b];
                    dg = fmaf(m.fzf, (float)(m.N - 2 * __popcll(k)), d);
                } else {
                    // same operations and order as HDiag (src/Hamiltonian.h:344-375): bit-identical
                    double d = 0.0;
                    for (int b = 0; b < m.nd; b++) {
                        const double q = 0.25 * m.d[b].dz;
                        d += (__popcll(k & m.d[b].mask) == 1) ? -q : q;
                    }
                    dg = __dadd_rn(d, __dmul_rn(m.fz, (double)(m.N - 2 * __popcll(k))));
                }
                const C v = tile[e];
                ar = dg * v.x;
                ai = dg * v.y;
            }
#pragma unroll 4
            for (int b = 0; b < p.nbond; b++) {
                const unsigned int lm = p.blm[b];
                const bool df = __popc((unsigned)e & lm) == 1;
                R c;
                if constexpr (F32) c = df ? p.cdifff[b] : p.ceqf[b];
                else c = df ? p.cdiff[b] : p.ceq[b];
                const C w = tile[e ^ lm];
                ar = fma(c, w.x, ar);
                ai = fma(c, w.y, ai);
            }
            R Fr = 0, Fi = 0, Gr = 0, Gi = 0;
#pragma unroll 4
            for (int f = 0; f < p.nfield; f++) {
                const unsigned int lm = p.flm[f];
                const C w = tile[e ^ lm];
                const R sg = ((unsigned)e & lm) ? (R)1 : (R)-1;
                Fr += w.x; Fi += w.y;
                Gr = fma(sg, w.x, Gr); Gi = fma(sg, w.y, Gi);
            }
            if (p.nfield) {
                ar = fma(fx, Fr, ar); ar = fma(-fy, Gi, ar);
                ai = fma(fx, Fi, ai); ai = fma(fy, Gr, ai);
            }
            if (p.accumulate) {
                const C o = out[k];
                ar += o.x;
                ai += o.y;
            }
            C o;
            o.x = ar; o.y = ai;
            out[k] = o;
        }
        __syncthreads();
    }
}

// Diagonal of the bond terms, R per state.  FP64: the reference's operations and order
// (HDiag, src/Hamiltonian.h:344-360), so that adding Bz*SzT later reproduces HDiag bit for bit.
template <typename R>
__global__ void __launch_bounds__(256) k_diag(const __grid_constant__ DevModel m, R* __restrict__ diag, long long D) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < D; k += stride) {
        const unsigned long long uk = (unsigned long long)k;
        if constexpr (sizeof(R) == 4) {
            float d = 0.0f;
            for (int b = 0; b < m.nd; b++) d += (__popcll(uk & m.d[b].mask) == 1) ? -m.dqf[b] : m.dqf[b];
            diag[k] = d;
        } else {
            double d = 0.0;
            for (int b = 0; b < m.nd; b++) {
                const double q = 0.25 * m.d[b].dz;
                d += (__popcll(uk & m.d[b].mask) == 1) ? -q : q;
            }
            diag[k] = d;
        }
    }
}

// Fast pass: 512 threads, c = 3, thread t owns the E tile states t + 512 j (j < E), so a state's
// tile-local index splits into thread bits (< 9) and j bits (>= 9).  Term parameters are read once
// per thread per term; the parity of a term's mask over the j bits is a host-precomputed bit mask
// (bjpar / fjbit), the thread-bit part one POPC.  Diagonal read from the precomputed vector.
// Columns: per tile, every active column of `cols` (own vectors at in + c ld, own field); with
// cols.dotp, the alpha partials sum conj(in) out per column and CTA (accumulated in double).
template <typename R, int E>
__global__ void __launch_bounds__(TILE_THREADS) k_hv_pass_fast(const __grid_constant__ DevModel m,
                                                                const __grid_constant__ DevPass p,
                                                                const __grid_constant__ DevCols cols,
                                                                const R* __restrict__ diag,
                                                                const typename V2T<R>::T* __restrict__ in,
                                                                typename V2T<R>::T* __restrict__ out,
                                                                long long ntiles, const int* __restrict__ active) {
    typedef typename V2T<R>::T C;
    unsigned cmask = 0;
    for (int c = 0; c < cols.ncols; c++)
        if (!active || active[c]) cmask |= 1u << c;
    if (!cmask) return;
    constexpr bool F32 = sizeof(R) == 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tile = reinterpret_cast<C*>(smem_raw);
    __shared__ unsigned long long hi_off[E];
    __shared__ double dsm[MAX_COLS][TILE_THREADS / 32][2];
    const int tid = threadIdx.x;
    if (tid < E) hi_off[tid] = p.tabHi[tid];
    if (cols.dotp)
        for (int i = tid; i < MAX_COLS * (TILE_THREADS / 32) * 2; i += TILE_THREADS) (&dsm[0][0][0])[i] = 0.0;
    const unsigned long long lo = p.tabLo[tid >> 3] | (unsigned long long)(tid & 7);
    __syncthreads();
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned long long base = lo;
        for (int q = 0; q < p.nrest; q++) base |= (((unsigned long long)t >> q) & 1ull) << p.rest[q];
        for (unsigned cm = cmask; cm; cm &= cm - 1) {
            const int c = __ffs((int)cm) - 1;
            const C* inc = in + c * cols.ld;
            C* outc = out + c * cols.ld;
            const R fx = F32 ? (R)cols.f.fxf[c] : (R)cols.f.fx[c], fy = F32 ? (R)cols.f.fyf[c] : (R)cols.f.fy[c];
            const R fz = F32 ? (R)cols.f.fzf[c] : (R)cols.f.fz[c];
#pragma unroll
            for (int j = 0; j < E; j++) tile[tid + TILE_THREADS * j] = inc[base | hi_off[j]];
            __syncthreads();
            R ar[E], ai[E];
            if (p.diag) {
#pragma unroll
                for (int j = 0; j < E; j++) {
                    const unsigned long long k = base | hi_off[j];
                    const R d = diag[k];
                    const R nz = (R)(m.N - 2 * __popcll(k));
                    R dg;
                    if constexpr (F32) dg = fmaf(fz, nz, d);
                    else dg = __dadd_rn(d, __dmul_rn(fz, nz));    // HDiag += Bzz*SzT (src/Hamiltonian.h:374)
                    const C v = tile[tid + TILE_THREADS * j];
                    ar[j] = dg * v.x;
                    ai[j] = dg * v.y;
                }
            } else if (p.accumulate) {
#pragma unroll
                for (int j = 0; j < E; j++) {
                    const C o = outc[base | hi_off[j]];
                    ar[j] = o.x;
                    ai[j] = o.y;
                }
            } else {
#pragma unroll
                for (int j = 0; j < E; j++) ar[j] = ai[j] = (R)0;
            }
            for (int b = 0; b < p.nbond; b++) {
                const unsigned int lm = p.blm[b];
                const unsigned int jp = p.bjpar[b];
                const unsigned int pb = __popc((unsigned)tid & lm) & 1u;
                R c0, c1;
                if constexpr (F32) { c0 = p.ceqf[b]; c1 = p.cdifff[b]; }
                else { c0 = p.ceq[b]; c1 = p.cdiff[b]; }
#pragma unroll
                for (int j = 0; j < E; j++) {
                    const R cc = (pb ^ ((jp >> j) & 1u)) ? c1 : c0;
                    const C w = tile[(tid + TILE_THREADS * j) ^ lm];
                    ar[j] = fma(cc, w.x, ar[j]);
                    ai[j] = fma(cc, w.y, ai[j]);
                }
            }
            for (int f = 0; f < p.nfield; f++) {
                const unsigned int lm = p.flm[f];
                const unsigned int jb = p.fjbit[f];
                const bool tb = ((unsigned)tid & lm) != 0u;
#pragma unroll
                for (int j = 0; j < E; j++) {
                    // (Bx/2 + i By/2 (bit ? +1 : -1)) v[k ^ 2^s]
                    const R sfy = (tb || ((jb >> j) & 1u)) ? fy : -fy;
                    const C w = tile[(tid + TILE_THREADS * j) ^ lm];
                    ar[j] = fma(fx, w.x, ar[j]); ar[j] = fma(-sfy, w.y, ar[j]);
                    ai[j] = fma(fx, w.y, ai[j]); ai[j] = fma(sfy, w.x, ai[j]);
                }
            }
            double dre = 0.0, dim = 0.0;
#pragma unroll
            for (int j = 0; j < E; j++) {
                C o;
                o.x = ar[j];
                o.y = ai[j];
                outc[base | hi_off[j]] = o;
                if (cols.dotp) {
                    const C v = tile[tid + TILE_THREADS * j];
                    dre += (double)v.x * (double)o.x + (double)v.y * (double)o.y;
                    dim += (double)v.x * (double)o.y - (double)v.y * (double)o.x;
                }
            }
            if (cols.dotp) {
                for (int o = 16; o > 0; o >>= 1) {
                    dre += __shfl_xor_sync(0xffffffffu, dre, o);
                    dim += __shfl_xor_sync(0xffffffffu, dim, o);
                }
                if ((tid & 31) == 0) { dsm[c][tid >> 5][0] += dre; dsm[c][tid >> 5][1] += dim; }
            }
            __syncthreads();
        }
    }
    if (cols.dotp) {
        __syncthreads();
        if (tid < MAX_COLS && ((cmask >> tid) & 1u)) {
            double re = 0.0, im = 0.0;
            for (int w = 0; w < TILE_THREADS / 32; w++) { re += dsm[tid][w][0]; im += dsm[tid][w][1]; }
            cols.dotp[((size_t)(cols.col0 + tid) * gridDim.x + blockIdx.x) * 2] = re;
            cols.dotp[((size_t)(cols.col0 + tid) * gridDim.x + blockIdx.x) * 2 + 1] = im;
        }
    }
}

// Alpha partials of launches without an epilogue of their own: sum conj(in) out per column over a
// fixed grid of DOT_GRID blocks (layout of DevCols::dotp).
constexpr int DOT_GRID = 608;
template <typename R>
__global__ void __launch_bounds__(256) k_dot_cols(const typename V2T<R>::T* __restrict__ in,
                                                  const typename V2T<R>::T* __restrict__ out, long long ld, long long D,
                                                  const int* __restrict__ active, double* __restrict__ dotp, int col0) {
    const int c = blockIdx.y;
    if (active && !active[c]) return;
    double re = 0.0, im = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += stride) {
        const typename V2T<R>::T v = in[c * ld + i], o = out[c * ld + i];
        re += (double)v.x * (double)o.x + (double)v.y * (double)o.y;
        im += (double)v.x * (double)o.y - (double)v.y * (double)o.x;
    }
    __shared__ double sm[2][8];
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = re; sm[1][threadIdx.x >> 5] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < 8; w++) { a += sm[0][w]; b += sm[1][w]; }
        dotp[((size_t)(col0 + c) * gridDim.x + blockIdx.x) * 2] = a;
        dotp[((size_t)(col0 + c) * gridDim.x + blockIdx.x) * 2 + 1] = b;
    }
}

// Complex64 pass, v2.  Same ownership as k_hv_pass_fast (thread t owns states t + 512 j), but each
// term is dispatched on the high part of its tile-local mask (bits >= 9, LMH < E): the partner of
// state t + 512 j is (t ^ lm_lo) + 512 (j ^ LMH) and the j part of the bond parity is
// popcount(j & LMH), both compile-time after unrolling.  Per state and term this leaves one shared
// load and one packed FFMA2 (bond) or one FFMA2 + one FADD2 (field: acc += fx w, G += +-w; the
// i*By/2*G part is added once at the end).
template <int E, int LMH>
__device__ __forceinline__ void bond_f32(const float2* __restrict__ tile, int tid, unsigned lm_lo, float cA, float cB,
                                         float2 (&acc)[E]) {
    const float2* src = tile + (tid ^ (int)lm_lo);
    const float2 vA = make_float2(cA, cA), vB = make_float2(cB, cB);
#pragma unroll
    for (int j = 0; j < E; j++) {
        const float2 w = src[TILE_THREADS * (j ^ LMH)];
        acc[j] = __ffma2_rn((__builtin_popcount(j & LMH) & 1) ? vB : vA, w, acc[j]);
    }
}
template <int E, int FB>
__device__ __forceinline__ void field_f32(const float2* __restrict__ tile, int tid, unsigned lm_lo, bool tb,
                                          float2 vfx, float2 (&acc)[E], float2 (&G)[E]) {
    const float2* src = tile + (tid ^ (int)lm_lo);
#pragma unroll
    for (int j = 0; j < E; j++) {
        const int jj = FB < 0 ? j : (j ^ (1 << FB));
        const float2 w = src[TILE_THREADS * jj];
        const bool bit = FB < 0 ? tb : ((j >> FB) & 1);
        acc[j] = __ffma2_rn(vfx, w, acc[j]);
        G[j] = bit ? __fadd2_rn(G[j], w) : __fadd2_rn(G[j], make_float2(-w.x, -w.y));
    }
}

template <int E, int L = 0>
__device__ __forceinline__ void bond_dispatch(int lmh, const float2* tile, int tid, unsigned lm_lo, float cA, float cB,
                                              float2 (&acc)[E]) {
    if constexpr (L < E) {
        if (lmh == L) bond_f32<E, L>(tile, tid, lm_lo, cA, cB, acc);
        else bond_dispatch<E, L + 1>(lmh, tile, tid, lm_lo, cA, cB, acc);
    }
}
template <int E, int FB = -1>
__device__ __forceinline__ void field_dispatch(int fb, const float2* tile, int tid, unsigned lm_lo, bool tb, float2 vfx,
                                               float2 (&acc)[E], float2 (&G)[E]) {
    if constexpr ((1 << (FB < 0 ? 0 : FB)) < E || FB < 0) {
        if (fb == FB) field_f32<E, FB>(tile, tid, lm_lo, tb, vfx, acc, G);
        else if constexpr ((2 << (FB < 0 ? -1 + 1 : FB)) < E || FB < 0) field_dispatch<E, FB + 1>(fb, tile, tid, lm_lo, tb, vfx, acc, G);
    }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory"); }

template <int E>
__device__ __forceinline__ unsigned long long tile_bits_of(const DevPass& p, long long t) {
    unsigned long long b = 0;
    for (int q = 0; q < p.nrest; q++) b |= (((unsigned long long)t >> q) & 1ull) << p.rest[q];
    return b;
}

// Double-buffered: tile t+G is copied into the other buffer (cp.async, 16 B per copy) while tile t
// is computed; the diagonal / partial-sum loads of tile t are issued before the term loops and
// consumed after them.
template <int E>
__global__ void __launch_bounds__(TILE_THREADS, 2) k_hv_pass_f32(const __grid_constant__ DevModel m,
                                                               const __grid_constant__ DevPass p,
                                                               const float* __restrict__ diag,
                                                               const float2* __restrict__ in,
                                                               float2* __restrict__ out, long long ntiles,
                                                               const int* __restrict__ active) {
    if (active && *active == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);   // 2 x (512 E) states
    __shared__ unsigned long long hi_off[E];
    const int tid = threadIdx.x;
    if (tid < E) hi_off[tid] = p.tabHi[tid];
    const unsigned long long lo = p.tabLo[tid >> 3] | (unsigned long long)(tid & 7);
    // 16-byte copies: thread t moves states 2t' and 2t'+1, t' = t + 512 i (runs of 8 never split)
    const unsigned long long lo2 = p.tabLo[(tid >> 2) & 63] | (unsigned long long)((2 * tid) & 7);
    const int hi2 = tid >> 8;
    const float2 vfx = make_float2(m.fxf, m.fxf);
    const float fy = m.fyf, fz = m.fzf;
    __syncthreads();
    auto issue = [&](long long t, float2* dst) {
        const unsigned long long b2 = tile_bits_of<E>(p, t) | lo2;
#pragma unroll
        for (int i = 0; i < E / 2; i++)
            cp_async16(dst + 2 * (tid + TILE_THREADS * i), in + (b2 | hi_off[hi2 + 2 * i]));
        cp_async_commit();
    };
    long long t = blockIdx.x;
    int cur = 0;
    if (t < ntiles) issue(t, bufs);
    for (; t < ntiles; t += gridDim.x, cur ^= 1) {
        float2* tile = bufs + cur * (TILE_THREADS * E);
        const long long tn = t + gridDim.x;
        if (tn < ntiles) {
            issue(tn, bufs + (cur ^ 1) * (TILE_THREADS * E));
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const unsigned long long base = tile_bits_of<E>(p, t) | lo;
        float2 acc[E], G[E], pre[E];
        float dpre[E];
#pragma unroll
        for (int j = 0; j < E; j++) {
            acc[j] = make_float2(0.f, 0.f);
            G[j] = make_float2(0.f, 0.f);
            if (p.diag) dpre[j] = diag[base | hi_off[j]];
            else if (p.accumulate) pre[j] = out[base | hi_off[j]];
        }
        for (int b = 0; b < p.nbond; b++) {
            const unsigned int lm = p.blm[b];
            const bool pb = __popc((unsigned)tid & lm & (TILE_THREADS - 1)) & 1;
            const float cA = pb ? p.cdifff[b] : p.ceqf[b], cB = pb ? p.ceqf[b] : p.cdifff[b];
            bond_dispatch<E>((int)(lm >> 9), tile, tid, lm & (TILE_THREADS - 1), cA, cB, acc);
        }
        for (int f = 0; f < p.nfield; f++) {
            const unsigned int lm = p.flm[f];
            const unsigned int lo9 = lm & (TILE_THREADS - 1);
            const bool tb = ((unsigned)tid & lo9) != 0u;
            const int fb = lo9 ? -1 : (31 - __clz((int)(lm >> 9)));
            field_dispatch<E>(fb, tile, tid, lo9, tb, vfx, acc, G);
        }
#pragma unroll
        for (int j = 0; j < E; j++) {
            const unsigned long long k = base | hi_off[j];
            float2 o = acc[j];
            o.x = fmaf(-fy, G[j].y, o.x);      // + i fy G
            o.y = fmaf(fy, G[j].x, o.y);
            if (p.diag) {
                const float dg = fmaf(fz, (float)(m.N - 2 * __popcll(k)), dpre[j]);
                const float2 v = tile[tid + TILE_THREADS * j];
                o.x = fmaf(dg, v.x, o.x);
                o.y = fmaf(dg, v.y, o.y);
            } else if (p.accumulate) {
                o.x += pre[j].x;
                o.y += pre[j].y;
            }
            out[k] = o;
        }
        __syncthreads();   // buffer `cur` is refilled by the next iteration's prefetch
    }
}

// ---------------------------------------------------------------------------------------------
// Register-grouped complex64 pass (device code in hv_pass_device.cuh).  This ahead-of-time
// instance reads the term groups from the pass table; hv_jit.cu compiles the same pass body
// with the groups of one Hamiltonian written out as straight-line code.
// ---------------------------------------------------------------------------------------------
template <int E>
__device__ __forceinline__ void gbond_switch(int lmh, const float2 (&P)[E], float2 vA, float2 vB, float2 (&acc)[E]) {
#define ESC_GB(k)                                                    \
    case k:                                                          \
        if constexpr ((k) < E) escdev::gbond<E, (k)>(P, vA, vB, acc); \
        break;
    switch (lmh) {
        ESC_GB(0) ESC_GB(1) ESC_GB(2) ESC_GB(3) ESC_GB(4) ESC_GB(5) ESC_GB(6) ESC_GB(7)
        ESC_GB(8) ESC_GB(9) ESC_GB(10) ESC_GB(11) ESC_GB(12) ESC_GB(13) ESC_GB(14) ESC_GB(15)
        ESC_GB(16) ESC_GB(17) ESC_GB(18) ESC_GB(19) ESC_GB(20) ESC_GB(21) ESC_GB(22) ESC_GB(23)
        ESC_GB(24) ESC_GB(25) ESC_GB(26) ESC_GB(27) ESC_GB(28) ESC_GB(29) ESC_GB(30) ESC_GB(31)
        default: break;
    }
#undef ESC_GB
}
template <int E, int FB = -1>
__device__ __forceinline__ void gfield_dispatch(int fb, const float2 (&P)[E], float2 vfx, float fy, float sf,
                                                float2 (&acc)[E]) {
    if constexpr ((1 << (FB + 1)) <= E) {
        if (fb == FB) escdev::gfield<E, FB>(P, vfx, fy, sf, acc);
        else gfield_dispatch<E, FB + 1>(fb, P, vfx, fy, sf, acc);
    }
}

template <int E, int TB>
struct RuntimeTerms {
    const DevPass& p;
    __device__ __forceinline__ void operator()(const float2* tile, int tid, float2 vfx, float fy, float2 (&acc)[E]) const {
        int q = 0;
        for (int g = 0; g < p.ngroup; g++) {
            const unsigned int glo = p.glo[g];
            float2 P[E];
            escdev::load_group<E, TB>(tile, tid, glo, P);
            const bool par = __popc((unsigned)tid & glo) & 1;
            const float sf = ((unsigned)tid & glo) ? fy : -fy;
            const int qe = q + p.gnt[g];
            for (; q < qe; q++) {
                const int code = p.gk[q];
                if (code < 32) {
                    const float a = p.ga[q], b = p.gb[q];
                    const float2 vA = par ? make_float2(b, b) : make_float2(a, a);
                    const float2 vB = par ? make_float2(a, a) : make_float2(b, b);
                    gbond_switch<E>(code, P, vA, vB, acc);
                } else {
                    gfield_dispatch<E>(code - 33, P, vfx, fy, sf, acc);
                }
            }
        }
    }
};

// Two CTAs per SM for 4096-state tiles; one for 8192-state tiles (2 x 64 KB ring, 128 registers
// for each of 512 threads).
template <int E, int NS, int TB>
__global__ void __launch_bounds__(TB, TB * E >= 8192 ? 1 : 2) k_hv_pass_f32g(const __grid_constant__ escdev::PassTab pt,
                                                      const __grid_constant__ DevPass p,
                                                      const float* __restrict__ diag,
                                                      const float2* __restrict__ in,
                                                      float2* __restrict__ out, long long ntiles,
                                                      const int* __restrict__ active) {
    escdev::pass_body<E, NS, RuntimeTerms<E, TB>, TB>(pt, RuntimeTerms<E, TB>{p}, diag, in, out, ntiles, active);
}

// Slab pair of two grouped passes (hv_pass_device.cuh: pair_body), ahead of time: 2 tile buffers,
// one CTA per SM for 8192-state tiles, two for 4096.  Launched cooperatively.
template <int E, int TB>
__global__ void __launch_bounds__(TB, TB * E >= 8192 ? 1 : 2) k_hv_pair_f32g(const __grid_constant__ escdev::PassTab pa,
                                                      const __grid_constant__ escdev::PassTab pb,
                                                      const __grid_constant__ escdev::PairTab st,
                                                      const __grid_constant__ DevPass a,
                                                      const __grid_constant__ DevPass b,
                                                      const float* __restrict__ diag,
                                                      const float2* __restrict__ in,
                                                      float2* __restrict__ out, const int* __restrict__ active) {
    escdev::pair_body<E, TB>(pa, pb, st, RuntimeTerms<E, TB>{a}, RuntimeTerms<E, TB>{b}, diag, in, out, active);
}

escdev::PairTab make_pair_tab(const DevPass& a, const DevPass& b, int N, unsigned* sync) {
    escdev::PairTab t;
    std::memset(&t, 0, sizeof(t));
    const unsigned long long all = N >= 64 ? ~0ull : (1ull << N) - 1ull;
    unsigned long long ra = 0, rb = 0;
    for (int q = 0; q < a.nrest; q++) ra |= 1ull << a.rest[q];
    for (int q = 0; q < b.nrest; q++) rb |= 1ull << b.rest[q];
    const unsigned long long ta = all & ~ra, tb = all & ~rb, u = ta | tb;
    const int U = __builtin_popcountll(u);
    if (a.Tp != b.Tp || a.nrest != b.nrest || a.nrest > 30 || U >= N || U - a.Tp > 30)
        throw std::invalid_argument("passes cannot form a slab pair");
    t.nrest = a.nrest;
    t.inner = U - a.Tp;
    t.nslab = 1ll << (N - U);
    // tile number: slab-internal bits (the other pass's tile bits) first, then the slab bits
    const unsigned long long inner[2] = {tb & ~ta, ta & ~tb};
    for (int x = 0; x < 2; x++) {
        int n = 0;
        for (int q = 0; q < N; q++)
            if ((inner[x] >> q) & 1ull) t.rest[x][n++] = (unsigned char)q;
        for (int q = 0; q < N; q++)
            if (!((u >> q) & 1ull)) t.rest[x][n++] = (unsigned char)q;
    }
    t.err = sync;
    t.cnt = sync + SLAB_CNT0;
    t.need = 1u << t.inner;
    // test hook: a count that is never reached, so that every wait of the launch gives up
    if (const char* e = std::getenv("ESC_TEST_SLAB_STALL"))
        if (std::atoi(e) > 0) t.need += 1;
    return t;
}

escdev::PassTab make_pass_tab(const DevPass& p, const DevModel& m, const DevCols* cols, double* dotp) {
    escdev::PassTab t;
    std::memset(&t, 0, sizeof(t));
    std::memcpy(t.tabLo, p.tabLo, sizeof(t.tabLo));
    std::memcpy(t.tabHi, p.tabHi, sizeof(t.tabHi));
    std::memcpy(t.rest, p.rest, sizeof(t.rest));
    t.nrest = p.nrest;
    t.rmask = 0;
    for (int q = 0; q < p.nrest; q++) t.rmask |= 1ull << p.rest[q];
    t.diag = p.diag;
    t.accumulate = p.accumulate;
    t.N = m.N;
    if (cols) {
        t.ld = cols->ld;
        t.ncols = cols->ncols;
        t.dcol0 = cols->col0;
        for (int c = 0; c < cols->ncols; c++) {
            t.fx[c] = cols->f.fxf[c];
            t.fy[c] = cols->f.fyf[c];
            t.fz[c] = cols->f.fzf[c];
        }
    } else {
        t.ncols = 1;
        t.fx[0] = m.fxf;
        t.fy[0] = m.fyf;
        t.fz[0] = m.fzf;
    }
    t.dotp = dotp;
    return t;
}

DevCols single_column(const DevModel& m) {
    DevCols c;
    c.ncols = 1;
    c.f.fx[0] = m.fx; c.f.fy[0] = m.fy; c.f.fz[0] = m.fz;
    c.f.fxf[0] = m.fxf; c.f.fyf[0] = m.fyf; c.f.fzf[0] = m.fzf;
    return c;
}

// FP64 energy sweep: sum over one pass of conj(v[k]) (H_pass v)[k], computed in FP64 from a
// complex64 or complex128 vector, without writing H v.  The passes of a plan add up to
// <v|H|v>.  One (re, im) partial per CTA (fixed grid: deterministic).
template <typename S>
__global__ void __launch_bounds__(TILE_THREADS) k_energy_pass(const __grid_constant__ DevModel m,
                                                               const __grid_constant__ DevPass p,
                                                               const typename V2T<S>::T* __restrict__ in,
                                                               double* __restrict__ partials, long long ntiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2* tile = reinterpret_cast<double2*>(smem_raw);
    const int Tn = 1 << p.Tp;
    const int cm = (1 << p.c) - 1;
    double er = 0.0, ei = 0.0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        unsigned long long base = 0;
        for (int q = 0; q < p.nrest; q++) base |= (((unsigned long long)t >> q) & 1ull) << p.rest[q];
        for (int e = threadIdx.x; e < Tn; e += blockDim.x) {
            const int r = e >> p.c;
            const unsigned long long k = base | p.tabLo[r & 63] | p.tabHi[r >> 6] | (unsigned long long)(e & cm);
            const typename V2T<S>::T x = in[k];
            tile[e] = make_double2((double)x.x, (double)x.y);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < Tn; e += blockDim.x) {
            const int r = e >> p.c;
            const unsigned long long k = base | p.tabLo[r & 63] | p.tabHi[r >> 6] | (unsigned long long)(e & cm);
            const double2 v = tile[e];
            double ar = 0.0, ai = 0.0;
            if (p.diag) {
                double d = 0.0;
                for (int b = 0; b < m.nd; b++) {
                    const double q = 0.25 * m.d[b].dz;
                    d += (__popcll(k & m.d[b].mask) == 1) ? -q : q;
                }
                d = __dadd_rn(d, __dmul_rn(m.fz, (double)(m.N - 2 * __popcll(k))));
                ar = d * v.x;
                ai = d * v.y;
            }
            for (int b = 0; b < p.nbond; b++) {
                const unsigned int lm = p.blm[b];
                const double c = (__popc((unsigned)e & lm) == 1) ? p.cdiff[b] : p.ceq[b];
                const double2 w = tile[e ^ lm];
                ar = fma(c, w.x, ar);
                ai = fma(c, w.y, ai);
            }
            for (int f = 0; f < p.nfield; f++) {
                const unsigned int lm = p.flm[f];
                const double2 w = tile[e ^ lm];
                const double sfy = ((unsigned)e & lm) ? m.fy : -m.fy;
                ar = fma(m.fx, w.x, ar); ar = fma(-sfy, w.y, ar);
                ai = fma(m.fx, w.y, ai); ai = fma(sfy, w.x, ai);
            }
            er += v.x * ar + v.y * ai;
            ei += v.x * ai - v.y * ar;
        }
        __syncthreads();
    }
    __shared__ double red[2][TILE_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        er += __shfl_xor_sync(0xffffffffu, er, o);
        ei += __shfl_xor_sync(0xffffffffu, ei, o);
    }
    if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = er; red[1][threadIdx.x >> 5] = ei; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < TILE_THREADS / 32; w++) { a += red[0][w]; b += red[1][w]; }
        partials[2 * blockIdx.x] = a;
        partials[2 * blockIdx.x + 1] = b;
    }
}

template <typename S>
void launch_energy(const DevModel& m, const std::vector<DevPass>& passes, const void* in, int64_t D,
                   double* partials, int max_blocks, std::vector<double>& host_sum, cudaStream_t s) {
    typedef typename V2T<S>::T C;
    host_sum.assign(2, 0.0);
    for (const DevPass& p : passes) {
        const size_t smem = (size_t(1) << p.Tp) * sizeof(double2);
        if (smem > 48 * 1024)
            ESC_CUDA(cudaFuncSetAttribute(k_energy_pass<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const long long ntiles = (long long)(D >> p.Tp);
        const int g = (int)std::min<long long>(ntiles, max_blocks);
        k_energy_pass<S><<<g, TILE_THREADS, smem, s>>>(m, p, (const C*)in, partials, ntiles);
        ESC_CUDA(cudaGetLastError());
        std::vector<double> h(2 * (size_t)g);
        ESC_CUDA(cudaMemcpyAsync(h.data(), partials, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        ESC_CUDA(cudaStreamSynchronize(s));
        for (int i = 0; i < g; i++) { host_sum[0] += h[2 * i]; host_sum[1] += h[2 * i + 1]; }
    }
}
template void launch_energy<float>(const DevModel&, const std::vector<DevPass>&, const void*, int64_t, double*, int,
                                   std::vector<double>&, cudaStream_t);
template void launch_energy<double>(const DevModel&, const std::vector<DevPass>&, const void*, int64_t, double*, int,
                                    std::vector<double>&, cudaStream_t);

std::vector<DevPass> make_passes(const Plan& P, const DevModel& m, int balance_opt, int stages, int tb_bits) {
    if (tb_bits < 5 || tb_bits > 10) {
        const char* e = std::getenv("ESC_TB_BITS");
        tb_bits = e && std::atoi(e) >= 7 && std::atoi(e) <= 10 ? std::atoi(e) : 9;
    }
    const int np = (int)P.tiles.size();
    std::vector<DevPass> out(np);
    const bool field = m.fx != 0.0 || m.fy != 0.0;
    // Term -> pass assignment (balance_opt, or ESC_PASS_BALANCE).  0: a bond or field goes to the
    // first pass whose tile holds it.  1: most constrained term first, each to the eligible pass
    // with the fewest terms so far.  2: first-fit, then the fewest register groups (below).
    std::vector<unsigned long long> tm(np, 0);
    for (int pi = 0; pi < np; pi++)
        for (int b : P.tiles[pi]) tm[pi] |= 1ull << b;
    std::vector<std::vector<int>> passb(np), passf(np);
    {
        struct Term { unsigned long long mask; int id; bool bond; };
        std::vector<Term> terms;
        for (int b = 0; b < m.nb; b++) terms.push_back({m.b[b].mask, b, true});
        if (field)
            for (int s = 0; s < P.N; s++) terms.push_back({1ull << s, s, false});
        auto elig = [&](unsigned long long mk) {
            std::vector<int> e;
            for (int pi = 0; pi < np; pi++) if (!(mk & ~tm[pi])) e.push_back(pi);
            return e;
        };
        const char* be = std::getenv("ESC_PASS_BALANCE");
        const int mode = balance_opt >= 0 ? balance_opt : (be ? std::atoi(be) : 0);
        const bool balance = mode == 1;
        std::vector<int> order(terms.size()), load(np, 0), asg(terms.size(), -1);
        for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
        if (balance)
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return elig(terms[a].mask).size() < elig(terms[b].mask).size();
            });
        for (int i : order) {
            const std::vector<int> e = elig(terms[i].mask);
            if (e.empty()) {
                if (terms[i].bond) throw std::invalid_argument("plan leaves a bond outside every tile");
                continue;
            }
            int pick = e[0];
            if (balance)
                for (int pi : e) if (load[pi] < load[pick]) pick = pi;
            load[pick]++;
            asg[i] = pick;
        }
        if (mode == 2) {
            // ESC_PASS_BALANCE=2: local search from first-fit that moves single terms between
            // eligible passes while the total number of register groups (shared-memory loads per
            // state) decreases; a pass's groups are counted with its best register sites, as below.
            // The groups are counted for 512 threads per tile whatever tb_bits is, so that every
            // kernel variant of a plan assigns the same terms to the same pass (the self-tuner
            // combines passes of different variants into one H.v).
            constexpr int ASSIGN_TB_BITS = 9;
            auto pass_cost = [&](int pi, int add, int drop) {
                std::vector<unsigned long long> gm;
                for (size_t i = 0; i < terms.size(); i++)
                    if (((int)i != drop && asg[i] == pi) || (int)i == add) gm.push_back(terms[i].mask);
                const std::vector<int>& B = P.tiles[pi];
                const int c = std::min(P.c, (int)B.size());
                const int nf = (int)B.size() - c, r = std::max(0, (int)B.size() - ASSIGN_TB_BITS);
                int best = 1 << 30;
                for (unsigned sel = 0; sel < (1u << nf); sel++) {
                    if (__builtin_popcount(sel) != std::min(r, nf)) continue;
                    unsigned long long regm = 0;
                    for (int q = 0; q < nf; q++)
                        if ((sel >> q) & 1u) regm |= 1ull << B[c + q];
                    std::vector<unsigned long long> g{0ull};
                    for (unsigned long long x : gm)
                        if (std::find(g.begin(), g.end(), x & ~regm) == g.end()) g.push_back(x & ~regm);
                    best = std::min(best, (int)g.size());
                }
                return best;
            };
            std::vector<int> cost(np);
            for (int pi = 0; pi < np; pi++) cost[pi] = pass_cost(pi, -1, -1);
            for (int sweep = 0; sweep < 20; sweep++) {
                bool moved = false;
                for (size_t i = 0; i < terms.size(); i++) {
                    if (asg[i] < 0) continue;
                    for (int q : elig(terms[i].mask)) {
                        const int p = asg[i];
                        if (q == p) continue;
                        const int cp = pass_cost(p, -1, (int)i), cq = pass_cost(q, (int)i, -1);
                        if (cp + cq < cost[p] + cost[q]) {
                            asg[i] = q;
                            cost[p] = cp;
                            cost[q] = cq;
                            moved = true;
                        }
                    }
                }
                if (!moved) break;
            }
        }
        for (size_t i = 0; i < terms.size(); i++)
            if (asg[i] >= 0) (terms[i].bond ? passb : passf)[asg[i]].push_back(terms[i].id);
        for (int pi = 0; pi < np; pi++) {
            std::sort(passb[pi].begin(), passb[pi].end());
            std::sort(passf[pi].begin(), passf[pi].end());
        }
    }
    for (int pi = 0; pi < np; pi++) {
        DevPass& d = out[pi];
        std::memset(&d, 0, sizeof(d));
        d.jit = -1;
        d.stages = stages >= 2 && stages <= 5 ? stages : pass_stages();
        d.tb_bits = tb_bits;
        std::vector<int> B = P.tiles[pi];
        d.Tp = (int)B.size();
        d.c = std::min(P.c, d.Tp);
        if (d.Tp - d.c > 12) throw std::invalid_argument("tile too large for the run-offset tables");
        unsigned long long tmask = 0;
        for (int q = 0; q < d.Tp; q++) tmask |= 1ull << B[q];
        for (int q = 0; q < d.c; q++)
            if (B[q] != q) throw std::invalid_argument("tile must contain the lowest c bits");
        const std::vector<int>& pb = passb[pi];
        const std::vector<int>& pf = passf[pi];
        if ((int)pb.size() > MAX_PTERMS) throw std::invalid_argument("too many bonds in one pass");
        // Register sites: the tile has 2^Tp states over 2^tb_bits threads, so the top
        // r = Tp - tb_bits local bits index a thread's registers.  Pick the r non-shared sites that
        // leave the fewest distinct thread-bit masks (each costs one shared-memory load per state)
        // and put them last.
        const int r = std::max(0, d.Tp - tb_bits);
        if (r > 0 && d.Tp - d.c >= r) {
            const int nf = d.Tp - d.c;   // free positions c..Tp-1
            std::vector<int> freeb(B.begin() + d.c, B.end());
            std::vector<unsigned long long> gm;
            for (int b : pb) gm.push_back(m.b[b].mask);
            for (int s : pf) gm.push_back(1ull << s);
            int best = 1 << 30;
            unsigned bestsel = 0;
            for (unsigned sel = 0; sel < (1u << nf); sel++) {
                if (__builtin_popcount(sel) != r) continue;
                // local numbering: register sites -> bits Tp-r.., others keep their order
                unsigned long long regm = 0;
                for (int q = 0; q < nf; q++)
                    if ((sel >> q) & 1u) regm |= 1ull << freeb[q];
                // distinct masks of the non-register part (global masks suffice)
                std::vector<unsigned long long> g{0ull};
                for (unsigned long long x : gm) {
                    const unsigned long long lo = x & ~regm;
                    if (std::find(g.begin(), g.end(), lo) == g.end()) g.push_back(lo);
                }
                if ((int)g.size() < best) { best = (int)g.size(); bestsel = sel; }
            }
            std::vector<int> lane, reg;
            for (int q = 0; q < nf; q++) (((bestsel >> q) & 1u) ? reg : lane).push_back(freeb[q]);
            B.resize(d.c);
            B.insert(B.end(), lane.begin(), lane.end());
            B.insert(B.end(), reg.begin(), reg.end());
        }
        int local_of[64];
        for (int q = 0; q < 64; q++) local_of[q] = -1;
        for (int q = 0; q < d.Tp; q++) local_of[B[q]] = q;
        for (int rr = 0; rr < 64; rr++) {
            unsigned long long lo = 0, hi = 0;
            for (int q = 0; q < 6; q++) {
                if (d.c + q < d.Tp && ((rr >> q) & 1)) lo |= 1ull << B[d.c + q];
                if (d.c + 6 + q < d.Tp && ((rr >> q) & 1)) hi |= 1ull << B[d.c + 6 + q];
            }
            d.tabLo[rr] = lo; d.tabHi[rr] = hi;
        }
        d.nrest = 0;
        for (int q = 0; q < P.N; q++) if (!((tmask >> q) & 1ull)) d.rest[d.nrest++] = (unsigned char)q;
        auto local = [&](unsigned long long gm) {
            unsigned int lm = 0;
            for (int q = 0; q < P.N; q++) if ((gm >> q) & 1ull) lm |= 1u << local_of[q];
            return lm;
        };
        d.diag = (pi == 0);
        d.accumulate = (pi > 0);
        for (int b : pb) {
            d.blm[d.nbond] = local(m.b[b].mask);
            d.ceq[d.nbond] = m.b[b].ceq;
            d.cdiff[d.nbond] = m.b[b].cdiff;
            d.ceqf[d.nbond] = (float)m.b[b].ceq;
            d.cdifff[d.nbond] = (float)m.b[b].cdiff;
            for (int j = 0; j < 32; j++)
                d.bjpar[d.nbond] |= (unsigned)(__builtin_popcount(((unsigned)j << 9) & d.blm[d.nbond]) & 1) << j;
            d.nbond++;
        }
        for (int s : pf) {
            d.flm[d.nfield] = local(1ull << s);
            for (int j = 0; j < 32; j++)
                d.fjbit[d.nfield] |= (unsigned)((((unsigned)j << 9) & d.flm[d.nfield]) != 0u) << j;
            d.nfield++;
        }
        // register groups: thread-bit mask = local bits below tb_bits
        const unsigned lanes = (1u << std::min(d.Tp, tb_bits)) - 1u;
        std::vector<unsigned> keys;
        for (int b = 0; b < d.nbond; b++) keys.push_back(d.blm[b] & lanes);
        for (int f = 0; f < d.nfield; f++) keys.push_back(d.flm[f] & lanes);
        std::vector<unsigned> order;
        for (unsigned k : keys)
            if (std::find(order.begin(), order.end(), k) == order.end()) order.push_back(k);
        d.ngroup = 0;
        d.nterm = 0;
        for (unsigned g : order) {
            int n = 0;
            for (int b = 0; b < d.nbond; b++)
                if ((d.blm[b] & lanes) == g) {
                    d.gk[d.nterm] = (unsigned char)(d.blm[b] >> tb_bits);
                    d.ga[d.nterm] = d.ceqf[b];
                    d.gb[d.nterm] = d.cdifff[b];
                    d.nterm++; n++;
                }
            for (int f = 0; f < d.nfield; f++)
                if ((d.flm[f] & lanes) == g) {
                    const unsigned hi = d.flm[f] >> tb_bits;
                    d.gk[d.nterm] = (unsigned char)(hi ? 33 + (31 - __builtin_clz(hi)) : 32);
                    d.nterm++; n++;
                }
            d.glo[d.ngroup] = (unsigned short)g;
            d.gnt[d.ngroup] = (unsigned char)n;
            d.ngroup++;
        }
        d.jit_pair = -1;
    }
    if (slab_pairs_env() == 1) mark_pairs(out, P.N);
    return out;
}

void mark_pairs(std::vector<DevPass>& ps, int N) {
    const unsigned long long all = N >= 64 ? ~0ull : (1ull << N) - 1ull;
    std::vector<unsigned long long> tm(ps.size(), all);
    for (size_t i = 0; i < ps.size(); i++) {
        ps[i].pair = 0;
        ps[i].slab_bits = 0;
        for (int q = 0; q < ps[i].nrest; q++) tm[i] &= ~(1ull << ps[i].rest[q]);
    }
    for (size_t pi = 0; pi + 1 < ps.size();) {
        const int ub = __builtin_popcountll(tm[pi] | tm[pi + 1]);
        if (ub <= SLAB_MAX_BITS && ub < N && ps[pi].Tp == ps[pi + 1].Tp && ps[pi].c == 3 && ps[pi + 1].c == 3) {
            ps[pi].pair = 1;
            ps[pi].slab_bits = ub;
            pi += 2;
        } else {
            pi++;
        }
    }
}

template <typename R>
void launch_diag(const DevModel& m, void* diag, int64_t D, cudaStream_t s) {
    long long g = (D + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_diag<R><<<(unsigned)g, 256, 0, s>>>(m, (R*)diag, (long long)D);
    ESC_CUDA(cudaGetLastError());
}

template <typename R, int E>
static int run_fast(const DevModel& m, const DevPass& p, const DevCols& cols, const void* diag, const void* in, void* out,
                    int64_t D, int sms, cudaStream_t s, const int* active) {
    typedef typename V2T<R>::T C;
    const size_t smem = (size_t)TILE_THREADS * E * sizeof(C);
    if (smem > 48 * 1024)
        ESC_CUDA(cudaFuncSetAttribute(k_hv_pass_fast<R, E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ESC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_pass_fast<R, E>, TILE_THREADS, smem));
    const long long ntiles = (long long)(D >> p.Tp);
    const long long g = std::min<long long>(ntiles, (long long)sms * std::max(per_sm, 1));
    k_hv_pass_fast<R, E><<<(unsigned)g, TILE_THREADS, smem, s>>>(m, p, cols, (const R*)diag, (const C*)in, (C*)out,
                                                                 ntiles, active);
    ESC_CUDA(cudaGetLastError());
    return (int)g;
}

template <int E>
static void run_f32(const DevModel& m, const DevPass& p, const void* diag, const void* in, void* out, int64_t D, int sms,
                    cudaStream_t s, const int* active) {
    const size_t smem = 2 * (size_t)TILE_THREADS * E * sizeof(float2);   // double buffer
    if (smem > 48 * 1024)
        ESC_CUDA(cudaFuncSetAttribute(k_hv_pass_f32<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ESC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_pass_f32<E>, TILE_THREADS, smem));
    const long long ntiles = (long long)(D >> p.Tp);
    const long long g = std::min<long long>(ntiles, (long long)sms * std::max(per_sm, 1));
    k_hv_pass_f32<E><<<(unsigned)g, TILE_THREADS, smem, s>>>(m, p, (const float*)diag, (const float2*)in, (float2*)out,
                                                             ntiles, active);
    ESC_CUDA(cudaGetLastError());
}

template <int E, int NS, int TB = TILE_THREADS>
static int run_f32g(const escdev::PassTab& pt, const DevPass& p, const void* diag, const void* in, void* out, int64_t D,
                    int sms, cudaStream_t s, const int* active) {
    // NS-stage ring of tiles (NS = 4, 5: 2 tiles + staging of the epilogue loads)
    const size_t smem = (size_t)(NS >= 4 ? 3 : NS) * TB * E * sizeof(float2);
    // always raised: dynamic + static shared memory may pass 48 KB even when the ring alone does not
    ESC_CUDA(cudaFuncSetAttribute(k_hv_pass_f32g<E, NS, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ESC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_pass_f32g<E, NS, TB>, TB, smem));
    const long long ntiles = (long long)(D >> p.Tp);
    const long long g = std::min<long long>(ntiles, (long long)sms * std::max(per_sm, 1));
    k_hv_pass_f32g<E, NS, TB><<<(unsigned)g, TB, smem, s>>>(pt, p, (const float*)diag, (const float2*)in, (float2*)out,
                                                            ntiles, active);
    ESC_CUDA(cudaGetLastError());
    return (int)g;
}

int pass_stages() {
    const char* e = std::getenv("ESC_STAGES");
    const int x = e ? std::atoi(e) : 2;
    return x >= 2 && x <= 5 ? x : 2;
}

// Grouped complex64 pass (ahead of time): E = 2^(Tp - tb_bits) states per thread; returns the grid,
// or 0 when no instance fits the pass's shape.
static int run_grouped(const escdev::PassTab& pt, const DevPass& p, const void* diag, const void* in, void* out, int64_t D,
                       int sms, cudaStream_t s, const int* active) {
    if (!(p.c == 3 && ((p.Tp == 11 || p.Tp == 12) ? p.tb_bits >= 7 && p.tb_bits <= 9
                                                   : p.Tp == 13 && (p.tb_bits == 9 || p.tb_bits == 10))))
        return 0;
    switch ((p.tb_bits == 8 ? 100 : p.tb_bits == 7 ? 200 : p.tb_bits == 10 ? 300 : 0) + (p.Tp == 11 ? 10 : p.Tp == 12 ? 20 : 30) +
            p.stages) {
        case 335: return run_f32g<8, 5, 1024>(pt, p, diag, in, out, D, sms, s, active);
        case 35: return run_f32g<16, 5, 512>(pt, p, diag, in, out, D, sms, s, active);
        case 215: return run_f32g<16, 5, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 225: return run_f32g<32, 5, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 15: return run_f32g<4, 5>(pt, p, diag, in, out, D, sms, s, active);
        case 25: return run_f32g<8, 5>(pt, p, diag, in, out, D, sms, s, active);
        case 115: return run_f32g<8, 5, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 125: return run_f32g<16, 5, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 332: return run_f32g<8, 2, 1024>(pt, p, diag, in, out, D, sms, s, active);
        case 333: return run_f32g<8, 3, 1024>(pt, p, diag, in, out, D, sms, s, active);
        case 334: return run_f32g<8, 4, 1024>(pt, p, diag, in, out, D, sms, s, active);
        case 32: return run_f32g<16, 2, 512>(pt, p, diag, in, out, D, sms, s, active);
        case 33: return run_f32g<16, 3, 512>(pt, p, diag, in, out, D, sms, s, active);
        case 34: return run_f32g<16, 4, 512>(pt, p, diag, in, out, D, sms, s, active);
        case 212: return run_f32g<16, 2, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 213: return run_f32g<16, 3, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 214: return run_f32g<16, 4, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 222: return run_f32g<32, 2, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 223: return run_f32g<32, 3, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 224: return run_f32g<32, 4, 128>(pt, p, diag, in, out, D, sms, s, active);
        case 12: return run_f32g<4, 2>(pt, p, diag, in, out, D, sms, s, active);
        case 13: return run_f32g<4, 3>(pt, p, diag, in, out, D, sms, s, active);
        case 14: return run_f32g<4, 4>(pt, p, diag, in, out, D, sms, s, active);
        case 23: return run_f32g<8, 3>(pt, p, diag, in, out, D, sms, s, active);
        case 24: return run_f32g<8, 4>(pt, p, diag, in, out, D, sms, s, active);
        case 112: return run_f32g<8, 2, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 113: return run_f32g<8, 3, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 114: return run_f32g<8, 4, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 122: return run_f32g<16, 2, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 123: return run_f32g<16, 3, 256>(pt, p, diag, in, out, D, sms, s, active);
        case 124: return run_f32g<16, 4, 256>(pt, p, diag, in, out, D, sms, s, active);
        default: return run_f32g<8, 2>(pt, p, diag, in, out, D, sms, s, active);
    }
}

template <int E, int TB>
static int run_pair_aot(const escdev::PassTab& pa, const escdev::PassTab& pb, const escdev::PairTab& st, const DevPass& a,
                        const DevPass& b, const void* diag, const void* in, void* out, int sms, cudaStream_t s,
                        const int* active) {
    const size_t smem = (size_t)2 * TB * E * sizeof(float2);
    ESC_CUDA(cudaFuncSetAttribute(k_hv_pair_f32g<E, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    ESC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_pair_f32g<E, TB>, TB, smem));
    const long long items = (2 * st.nslab) << st.inner;
    const long long g = std::min<long long>(items, (long long)sms * std::max(per_sm, 1));
    const float* dg = (const float*)diag;
    const float2* vin = (const float2*)in;
    float2* vout = (float2*)out;
    void* args[] = {(void*)&pa, (void*)&pb, (void*)&st, (void*)&a, (void*)&b, (void*)&dg, (void*)&vin, (void*)&vout,
                    (void*)&active};
    ESC_CUDA(cudaLaunchCooperativeKernel((const void*)k_hv_pair_f32g<E, TB>, dim3((unsigned)g), dim3(TB), args, smem, s));
    return (int)g;
}

static std::atomic<unsigned long long> g_pair_launches{0};
unsigned long long slab_pair_launches() { return g_pair_launches.load(); }

// Slab pair of passes a (a.pair set) and b on one complex64 column; returns the grid, or 0 when
// no pair kernel exists for their shape (the caller then runs the passes one by one).
static int run_pair(const DevModel& m, const DevPass& a, const DevPass& b, const DevCols& cols, double* dotp,
                    const void* diag, const void* in, void* out, int64_t D, int sms, cudaStream_t s, const int* active) {
    if (!m.slab_sync || !pair_launchable(a, b)) return 0;
    const escdev::PairTab st = make_pair_tab(a, b, m.N, m.slab_sync);
    const escdev::PassTab pa = make_pass_tab(a, m, &cols, nullptr), pb = make_pass_tab(b, m, &cols, dotp);
    ESC_CUDA(cudaMemsetAsync(st.cnt, 0, (size_t)st.nslab * sizeof(unsigned), s));
    g_pair_launches++;
    if (a.jit_pair >= 0) return jit_pair_launch(a, pa, pb, st, diag, in, out, D, sms, s, active);
    if (a.Tp == 13) return run_pair_aot<16, 512>(pa, pb, st, a, b, diag, in, out, sms, s, active);
    return run_pair_aot<8, 512>(pa, pb, st, a, b, diag, in, out, sms, s, active);
}

template <typename R>
int launch_hv_cols(const DevModel& m, const DevCols& cols, const std::vector<DevPass>& passes, const void* in, void* out,
                   int64_t D, const void* diag, cudaStream_t s, const int* active) {
    typedef typename V2T<R>::T C;
    int dev = 0, sms = 0;
    ESC_CUDA(cudaGetDevice(&dev));
    ESC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (cols.ncols < 1 || cols.ncols > MAX_COLS) throw std::invalid_argument("1..16 columns per H.V launch");
    int G = 0;
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const DevPass& p = passes[pi];
        if constexpr (sizeof(R) == 4) {
            if (p.pair && pi + 1 < passes.size() && cols.ncols == 1 && diag) {
                double* dotp2 = pi + 2 == passes.size() ? cols.dotp : nullptr;
                const int g2 = run_pair(m, p, passes[pi + 1], cols, dotp2, diag, in, out, D, sms, s, active);
                if (g2) {
                    if (dotp2) G = g2;
                    pi++;
                    continue;
                }
            }
        }
        double* dotp = pi + 1 == passes.size() ? cols.dotp : nullptr;
        int g = 0;   // grid of a launch that handled every column (and the alpha epilogue)
        if constexpr (sizeof(R) == 4) {
            if (diag) {
                const escdev::PassTab pt = make_pass_tab(p, m, &cols, dotp);
                if (p.jit >= 0) g = jit_launch(p, pt, diag, in, out, D, sms, s, active);
                else g = run_grouped(pt, p, diag, in, out, D, sms, s, active);
            }
        }
        if (!g && diag && p.c == 3 && p.Tp >= 10 && p.Tp <= 13 && (sizeof(R) == 8 || !(p.Tp >= 11))) {
            DevCols cc = cols;
            cc.dotp = dotp;
            switch (p.Tp) {
                case 10: g = run_fast<R, 2>(m, p, cc, diag, in, out, D, sms, s, active); break;
                case 11: g = run_fast<R, 4>(m, p, cc, diag, in, out, D, sms, s, active); break;
                case 12: g = run_fast<R, 8>(m, p, cc, diag, in, out, D, sms, s, active); break;
                default: g = run_fast<R, 16>(m, p, cc, diag, in, out, D, sms, s, active); break;
            }
        }
        if (g) {
            if (dotp) G = g;
            continue;
        }
        // single-column kernels: one launch per column with that column's field
        for (int c = 0; c < cols.ncols; c++) {
            DevModel mc = m;
            mc.fx = cols.f.fx[c]; mc.fy = cols.f.fy[c]; mc.fz = cols.f.fz[c];
            mc.fxf = cols.f.fxf[c]; mc.fyf = cols.f.fyf[c]; mc.fzf = cols.f.fzf[c];
            const C* inc = (const C*)in + c * cols.ld;
            C* outc = (C*)out + c * cols.ld;
            const int* act = active ? active + c : nullptr;
            if (sizeof(R) == 4 && diag && p.c == 3 && p.Tp >= 11 && p.Tp <= 13) {
                switch (p.Tp) {
                    case 11: run_f32<4>(mc, p, diag, inc, outc, D, sms, s, act); break;
                    case 12: run_f32<8>(mc, p, diag, inc, outc, D, sms, s, act); break;
                    default: run_f32<16>(mc, p, diag, inc, outc, D, sms, s, act); break;
                }
                continue;
            }
            const size_t smem = (size_t(1) << p.Tp) * sizeof(C);
            if (smem > 48 * 1024)
                ESC_CUDA(cudaFuncSetAttribute(k_hv_pass<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int per_sm = 0;
            ESC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hv_pass<R>, TILE_THREADS, smem));
            const long long ntiles = (long long)(D >> p.Tp);
            const long long gg = std::min<long long>(ntiles, (long long)sms * std::max(per_sm, 1));
            k_hv_pass<R><<<(unsigned)gg, TILE_THREADS, smem, s>>>(mc, p, inc, outc, ntiles, act);
            ESC_CUDA(cudaGetLastError());
        }
        if (dotp) {
            k_dot_cols<R><<<dim3(DOT_GRID, cols.ncols), 256, 0, s>>>((const C*)in, (const C*)out, cols.ld, D, active, dotp,
                                                                    cols.col0);
            ESC_CUDA(cudaGetLastError());
            G = DOT_GRID;
        }
    }
    return G;
}

template <typename R>
void launch_hv_tiled(const DevModel& m, const std::vector<DevPass>& passes, const void* in, void* out, int64_t D,
                     const void* diag, cudaStream_t s, const int* active) {
    launch_hv_cols<R>(m, single_column(m), passes, in, out, D, diag, s, active);
}

template int launch_hv_cols<double>(const DevModel&, const DevCols&, const std::vector<DevPass>&, const void*, void*,
                                    int64_t, const void*, cudaStream_t, const int*);
template int launch_hv_cols<float>(const DevModel&, const DevCols&, const std::vector<DevPass>&, const void*, void*,
                                   int64_t, const void*, cudaStream_t, const int*);
template void launch_hv_tiled<double>(const DevModel&, const std::vector<DevPass>&, const void*, void*, int64_t,
                                      const void*, cudaStream_t, const int*);
template void launch_hv_tiled<float>(const DevModel&, const std::vector<DevPass>&, const void*, void*, int64_t,
                                     const void*, cudaStream_t, const int*);
template void launch_diag<double>(const DevModel&, void*, int64_t, cudaStream_t);
template void launch_diag<float>(const DevModel&, void*, int64_t, cudaStream_t);

}  // namespace esc

// =============================================================================================
// Allocation-free Rayleigh quotient.
//
// For callers that cannot allocate device memory themselves or through this library: code that
// runs inside another framework's memory pool, under a memory cap, or in a process that must not
// grow its device footprint after start-up.  The scratch of this entry point (one partial energy
// per tile, the norm-reduction partials and the result) is the file-scope array below, which
// every GPU that loads the library holds until the process exits.
// =============================================================================================
namespace esc {
namespace {
constexpr int NOALLOC_TILE_BITS = 12;
constexpr int NOALLOC_MAX_TILES = 1 << 13;                 // 2^13 tiles of 2^12 states: N <= 25
constexpr int NOALLOC_SCRATCH = 2 * NOALLOC_MAX_TILES      // per-tile (re, im) energy partials
                                + 2 * RED_MAX_BLOCKS       // norm-reduction partials
                                + 8;                       // reduction result
constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
// Per device: the array's device address and the unique id of the CUDA context it was looked up
// in.  A context rebuilt after cudaDeviceReset loads the module again, possibly at another
// address; its new id triggers a fresh lookup.
struct NoallocSlot {
    unsigned long long ctx_id = 0;
    void* ptr = nullptr;
};
NoallocSlot g_noalloc_slot[NOALLOC_MAX_DEVICES];

// cuCtxGetCurrent / cuCtxGetId through the runtime (the library links no libcuda)
typedef int (*PFN_ctx_current)(void**);
typedef int (*PFN_ctx_id)(void*, unsigned long long*);
bool current_context_id(unsigned long long& id) {
    static PFN_ctx_current cur = nullptr;
    static PFN_ctx_id gid = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess) {
            cur = (PFN_ctx_current)a;
            gid = (PFN_ctx_id)b;
        }
        (void)cudaGetLastError();
    }
    void* ctx = nullptr;
    return cur && gid && cur(&ctx) == 0 && ctx && gid(ctx, &id) == 0;
}

// Plans of the allocation-free path, kept per process (host memory only): a repeated call with the
// same model does not repeat the covering search.
std::map<std::string, Plan> g_noalloc_plans;
}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH];

}  // namespace esc

extern "C" esc_status esc_rayleigh_noalloc(const esc_params* p, const void* v, esc_dtype dt, void* stream, double* E) {
    using namespace esc;
    auto fail = [&](esc_status st, const std::string& m) { set_last_error(m); return st; };
    if (!p || !v || !E) return fail(ESC_ERR_PARAM, "null argument");
    try {
        cudaStream_t s = (cudaStream_t)stream;
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
            (void)cudaGetLastError();
            return fail(ESC_ERR_CUDA, "no usable CUDA device");
        }
        if (dt != ESC_C128 && dt != ESC_C64) return fail(ESC_ERR_PARAM, "esc_rayleigh_noalloc: dt must be ESC_C128 or ESC_C64");
        double* scratch = nullptr;
        {
            // set-up once per device (and context), with that device current: the device address of
            // the static array; host code must not pass the array's host-side name to a kernel
            std::lock_guard<std::mutex> lk(g_noalloc_mu);
            unsigned long long id = 0;
            const bool have_id = current_context_id(id);
            NoallocSlot& slot = g_noalloc_slot[dev];
            if (!slot.ptr || !have_id || slot.ctx_id != id) {
                void* ptr = nullptr;
                const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
                if (rc != cudaSuccess || !ptr) {
                    (void)cudaGetLastError();
                    slot = NoallocSlot{};
                    return fail(ESC_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(rc));
                }
                slot.ptr = ptr;
                slot.ctx_id = have_id ? id : 0;
            }
            scratch = (double*)slot.ptr;
        }
        Lattice L;
        std::vector<Bond> bonds;
        build_lattice(*p, L);
        build_bonds(*p, L, bonds);
        const int N = L.N;
        const int64_t D = int64_t(1) << N;
        if (N - NOALLOC_TILE_BITS > 13)
            return fail(ESC_ERR_PARAM, "esc_rayleigh_noalloc: at most 25 sites (2^25 states); the static scratch holds "
                                       "8192 tile partials");
        std::vector<std::pair<int, int>> pairs;
        for (const auto& b : bonds)
            if (b.kx - b.ky != 0.0 || b.kx + b.ky != 0.0) pairs.push_back({b.i, b.j});
        std::string key = std::to_string(N) + ":";
        for (const auto& pr : pairs) key += std::to_string(pr.first) + "," + std::to_string(pr.second) + ";";
        Plan P;
        {
            std::lock_guard<std::mutex> lk(g_noalloc_mu);
            auto it = g_noalloc_plans.find(key);
            if (it == g_noalloc_plans.end())
                it = g_noalloc_plans.emplace(key, make_plan_reference_order(N, pairs, NOALLOC_TILE_BITS, 3, 200)).first;
            P = it->second;
        }
        const DevModel m = make_dev_model(*p, L, bonds, p->Bxx, p->Byy, p->Bzz);
        const std::vector<DevPass> passes = make_passes(P, m);
        double* part = scratch;                                // [2 * tiles]
        double* red = scratch + 2 * NOALLOC_MAX_TILES;         // [2 * RED_MAX_BLOCKS]
        double* res = red + 2 * RED_MAX_BLOCKS;                // [2]
        double num = 0.0;
        for (const DevPass& ps : passes) {
            const long long ntiles = (long long)(D >> ps.Tp);
            const size_t smem = (size_t(1) << ps.Tp) * sizeof(double2);
            // one CTA per tile: every partial the host reads below is written by this launch
            if (dt == ESC_C64) {
                if (smem > 48 * 1024) ESC_CUDA(cudaFuncSetAttribute(k_energy_pass<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                k_energy_pass<float><<<(unsigned)ntiles, TILE_THREADS, smem, s>>>(m, ps, (const float2*)v, part, ntiles);
            } else {
                if (smem > 48 * 1024) ESC_CUDA(cudaFuncSetAttribute(k_energy_pass<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                k_energy_pass<double><<<(unsigned)ntiles, TILE_THREADS, smem, s>>>(m, ps, (const double2*)v, part, ntiles);
            }
            ESC_CUDA(cudaGetLastError());
            std::vector<double> h(2 * (size_t)ntiles);
            ESC_CUDA(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
            ESC_CUDA(cudaStreamSynchronize(s));
            for (long long i = 0; i < ntiles; i++) num += h[2 * i];
        }
        if (dt == ESC_C64) launch_dot<float>(v, v, D, red, res, s);
        else launch_dot<double>(v, v, D, red, res, s);
        double nn[2];
        ESC_CUDA(cudaMemcpyAsync(nn, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
        ESC_CUDA(cudaStreamSynchronize(s));
        *E = num / nn[0];
        return ESC_OK;
    } catch (std::invalid_argument& e) {
        return fail(ESC_ERR_PARAM, e.what());
    } catch (std::exception& e) {
        return fail(ESC_ERR_CUDA, e.what());
    }
}
