// hv_pass_device.cuh -- device code of the register-grouped complex64 H.v pass.
//
// Shared by the ahead-of-time kernel in hv_tiled.cu (terms read from the pass table at run time)
// and by the kernels specialised per Hamiltonian at run time in hv_jit.cu (terms compiled in as
// straight-line code).  It includes nothing, because it is also handed verbatim to NVRTC.
//
// A CTA of TB threads (1024, 512, 256 or 128: more register states per thread) owns one tile of TB E
// basis states at a time: thread t holds the states t + TB j (j < E), i.e. tile-local bits
// 0..log2(TB)-1 are thread bits and the bits above are register bits.
// Tiles are copied global -> shared with cp.async (16 B per copy, runs of 8 consecutive states),
// double buffered: tile n+1 is in flight while tile n is computed.  Terms come in groups of equal
// thread-bit mask: a thread loads the E partner states of a group from shared memory once and
// applies every term of the group from registers.
//
// Columns: one launch can apply the pass to up to MAXC vectors (column c at in + c ld, out + c ld,
// with its own field).  A CTA takes its tiles in turn and, per tile, every active column: the tile
// offsets and the term groups are decoded once for all columns, and the copy ring runs over the
// (tile, column) items.  Columns whose flag is 0 are skipped (recurrences that have stopped).
//
// Alpha epilogue (the last pass of a Lanczos step): with dotp set, each CTA also sums
// conj(in[k]) out[k] over the states it wrote, per column, in float-float (Dekker/Knuth error-free
// products and sums: no FP64 arithmetic per state), and writes one (re, im) double pair per column.
// The grid and the order of the additions are fixed, so the partials are bit-reproducible.
#pragma once

namespace escdev {

constexpr int TPB = 512;
constexpr int MAXC = 16;   // columns of one launch

// Per-pass tables (kernel parameter).  tabLo / tabHi map the tile-local bits c.. (6 at a time)
// to global index offsets; rest lists the global bits of the tile number.
struct PassTab {
    unsigned long long tabLo[64];
    unsigned long long tabHi[16];
    unsigned long long rmask;   // the global bits of the tile number (tile_bits of all ones)
    unsigned char rest[40];
    int nrest, diag, accumulate, N;
    long long ld;               // column stride (states)
    int ncols;
    int dcol0;                  // global index of column 0 in the alpha partials (launches over a column range)
    float fx[MAXC], fy[MAXC], fz[MAXC];   // Bx/2, By/2, Bz/2 per column
    double* dotp;               // alpha partials: (re, im) at dotp[((dcol0 + c) * gridDim.x + blockIdx.x) * 2]; NULL: none
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int NPEND>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(NPEND) : "memory"); }

// Float-float accumulation: (hi, lo) += a b exactly up to the final rounding of lo.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}
__device__ __forceinline__ void ff_addprod(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    ff_add(hi, lo, p);
    lo += e;
}
// (hi, lo) += (h2, l2)
__device__ __forceinline__ void ff_add2(float& hi, float& lo, float h2, float l2) {
    ff_add(hi, lo, h2);
    lo += l2;
}

// Active columns of a launch as a bit mask (active == NULL: all ncols columns)
__device__ __forceinline__ unsigned column_mask(const PassTab& p, const int* active) {
    unsigned m = 0;
    for (int c = 0; c < p.ncols; c++)
        if (!active || active[c]) m |= 1u << c;
    return m;
}
// next set bit of m above c, or -1
__device__ __forceinline__ int next_column(unsigned m, int c) {
    const unsigned r = m & ~((2u << c) - 1u);
    return r ? __ffs((int)r) - 1 : -1;
}

// Alpha epilogue accumulators: one float-float (re, im) per column and warp in shared memory.
struct DotAcc {
    float (*s)[32][4];   // [MAXC][warp (at most 32 of 1024 threads)][hi re, lo re, hi im, lo im]
    __device__ __forceinline__ void clear(int tid, int nthreads) {
        for (int i = tid; i < MAXC * 32 * 4; i += nthreads) (&s[0][0][0])[i] = 0.f;
    }
    // adds the thread's (re, im) float-float sums of one column: warp butterfly, lane 0 accumulates
    __device__ __forceinline__ void add(int c, int tid, float rh, float rl, float ih, float il) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a = __shfl_xor_sync(0xffffffffu, rh, o), b = __shfl_xor_sync(0xffffffffu, rl, o);
            const float x = __shfl_xor_sync(0xffffffffu, ih, o), y = __shfl_xor_sync(0xffffffffu, il, o);
            ff_add2(rh, rl, a, b);
            ff_add2(ih, il, x, y);
        }
        if ((tid & 31) == 0) {
            float* q = s[c][tid >> 5];
            ff_add2(q[0], q[1], rh, rl);
            ff_add2(q[2], q[3], ih, il);
        }
    }
    // per column: warps summed in order in double, written by one thread per column
    __device__ __forceinline__ void store(const PassTab& p, unsigned mask, int tid, int nwarps) {
        __syncthreads();
        if (tid < MAXC && ((mask >> tid) & 1u)) {
            double re = 0.0, im = 0.0;
            for (int w = 0; w < nwarps; w++) {
                re += (double)s[tid][w][0] + (double)s[tid][w][1];
                im += (double)s[tid][w][2] + (double)s[tid][w][3];
            }
            p.dotp[((unsigned long long)(p.dcol0 + tid) * gridDim.x + blockIdx.x) * 2] = re;
            p.dotp[((unsigned long long)(p.dcol0 + tid) * gridDim.x + blockIdx.x) * 2 + 1] = im;
        }
    }
};

__device__ __forceinline__ unsigned long long tile_bits(const PassTab& p, long long t) {
    unsigned long long b = 0;
    for (int q = 0; q < p.nrest; q++) b |= (((unsigned long long)t >> q) & 1ull) << p.rest[q];
    return b;
}
// tile_bits(a + b) from x = tile_bits(a) and y = tile_bits(b): the bits outside the mask are set to
// one so that carries run across them, then cleared (bits carried past the top are dropped, which
// only happens for tile numbers past the last tile)
__device__ __forceinline__ unsigned long long deposit_add(unsigned long long x, unsigned long long y, unsigned long long m) {
    return ((x | ~m) + y) & m;
}

// Partners of a group: P[j] = state (t ^ lo) + TB j of the tile (TB threads per tile).
template <int E, int TB = TPB>
__device__ __forceinline__ void load_group(const float2* tile, int tid, unsigned lo, float2 (&P)[E]) {
    const float2* src = tile + (tid ^ (int)lo);
#pragma unroll
    for (int j = 0; j < E; j++) P[j] = src[TB * j];
}

// parity of the low 5 bits of x
__host__ __device__ constexpr int par4(int x) { return (x ^ (x >> 1) ^ (x >> 2) ^ (x >> 3) ^ (x >> 4)) & 1; }

// Bond term with register mask LMH: acc[j] += c * P[j ^ LMH], c = vA or vB by the parity of the
// register bits under the mask (vA / vB already swapped for the thread-bit parity).
template <int E, int LMH>
__device__ __forceinline__ void gbond(const float2 (&P)[E], float2 vA, float2 vB, float2 (&acc)[E]) {
#pragma unroll
    for (int j = 0; j < E; j++) acc[j] = __ffma2_rn(par4(j & LMH) ? vB : vA, P[j ^ LMH], acc[j]);
}

// Field term on register bit FB (FB < 0: on a thread bit, sign sf = bit ? By/2 : -By/2 of the
// thread): acc[j] += (Bx/2 + i s) w, s = bit ? By/2 : -By/2.
template <int E, int FB>
__device__ __forceinline__ void gfield(const float2 (&P)[E], float2 vfx, float fy, float sf, float2 (&acc)[E]) {
#pragma unroll
    for (int j = 0; j < E; j++) {
        const float2 w = P[FB < 0 ? j : (j ^ (1 << FB))];
        const float sg = FB < 0 ? sf : (((j >> FB) & 1) ? fy : -fy);
        acc[j] = __ffma2_rn(vfx, w, acc[j]);
        // the i s part crosses the components: two scalar FMAs (no swapped register pair)
        acc[j].x = fmaf(-sg, w.y, acc[j].x);
        acc[j].y = fmaf(sg, w.x, acc[j].y);
    }
}

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}

// Per-CTA set-up shared by both pass bodies: register-index offsets hi_off[j] (global offset of
// tile state TB j), the thread's own offset `lo`, and the copy offsets.  Tile state s has its
// local bits 3..8 in tabLo[(s >> 3) & 63] and bits 9.. in tabHi[s >> 9].
template <int E, int TB>
__device__ __forceinline__ void tile_offsets(const PassTab& p, int tid, unsigned long long* hi_off,
                                             unsigned long long& lo, unsigned long long (&lo2)[2]) {
    if (tid < E) hi_off[tid] = p.tabLo[((TB * tid) >> 3) & 63] | p.tabHi[(TB * tid) >> 9];
    lo = p.tabLo[(tid >> 3) & 63] | p.tabHi[tid >> 9] | (unsigned long long)(tid & 7);   // tabHi: 1024 threads
    // 16-byte copies: copy c = tid + TB i moves tile states 2c and 2c+1 (runs of 8 never split);
    // (c >> 2) & 63 depends on i only for TB = 128 (through bit 5: i odd)
    lo2[0] = p.tabLo[(tid >> 2) & 63] | (unsigned long long)((2 * tid) & 7);
    lo2[1] = p.tabLo[((tid >> 2) + 32) & 63] | (unsigned long long)((2 * tid) & 7);
}
// copies tile b (b = tile_bits of its number) into dst
template <int E, int TB>
__device__ __forceinline__ void issue_tile(const PassTab& p, const float2* __restrict__ in, float2* dst,
                                           unsigned long long b, int tid, const unsigned long long (&lo2)[2]) {
#pragma unroll
    for (int i = 0; i < E / 2; i++) {
        const unsigned long long l = (TB == 128 && (i & 1)) ? lo2[1] : lo2[0];
        cp_async16(dst + 2 * (tid + TB * i), in + (b | l | p.tabHi[(tid + TB * i) >> 8]));
    }
}

// copies the float tile b (4 states per 16-byte copy: half a run of 8) of x into dst (tile layout)
template <int E, int TB>
__device__ __forceinline__ void issue_tile_f32(const PassTab& p, const float* __restrict__ x, float* dst,
                                               unsigned long long b, int tid) {
#pragma unroll
    for (int i = 0; i < E / 4; i++) {
        const int q = tid + TB * i;
        cp_async16(dst + 4 * q, x + (b | p.tabLo[(q >> 1) & 63] | p.tabHi[q >> 7] | (unsigned long long)((q & 1) << 2)));
    }
}

// Sums conj(v) o over a thread's E states of one item in float-float and adds them to the
// column's accumulators (alpha epilogue).
template <int E, int TB>
__device__ __forceinline__ void dot_item(DotAcc& da, int c, int tid, const float2* tile, const float2 (&o)[E]) {
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll
    for (int j = 0; j < E; j++) {
        const float2 v = tile[tid + TB * j];
        ff_addprod(rh, rl, v.x, o[j].x);
        ff_addprod(rh, rl, v.y, o[j].y);
        ff_addprod(ih, il, v.x, o[j].y);
        ff_addprod(ih, il, -v.y, o[j].x);
    }
    da.add(c, tid, rh, rl, ih, il);
}

// 2-stage tile ring + staged epilogue loads (see pass_body, NS = 4).
template <int E, int TB, class Terms>
__device__ __forceinline__ void pass_body_staged(const PassTab& p, const Terms& terms, const float* __restrict__ diag,
                                                 const float2* __restrict__ in, float2* __restrict__ out,
                                                 long long ntiles, const int* __restrict__ active) {
    const unsigned cmask = column_mask(p, active);
    if (!cmask) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);   // 2 x (TB E) states
    float2* stage = bufs + 2 * TB * E;                     // TB E partials (or diagonal entries)
    __shared__ unsigned long long hi_off[E];
    __shared__ float dsm[MAXC][32][4];
    DotAcc da{dsm};
    const int tid = threadIdx.x;
    unsigned long long lo, lo2[2];
    tile_offsets<E, TB>(p, tid, hi_off, lo, lo2);
    if (p.dotp) da.clear(tid, TB);
    __syncthreads();
    const long long g = gridDim.x;
    const long long ld = p.ld;
    const int c0 = __ffs((int)cmask) - 1;
    const unsigned long long dg = tile_bits(p, g);
    // current item (t, c) and the next one (tn, cn)
    long long t = blockIdx.x;
    int c = c0;
    unsigned long long bt = tile_bits(p, t);
    long long tn = t;
    int cn = c;
    unsigned long long bn = bt;
    auto advance = [&](long long& tt, int& cc, unsigned long long& bb) {
        const int nx = next_column(cmask, cc);
        if (nx >= 0) {
            cc = nx;
        } else {
            cc = c0;
            tt += g;
            bb = deposit_add(bb, dg, p.rmask);
        }
    };
    advance(tn, cn, bn);
    if (t < ntiles) issue_tile<E, TB>(p, in + c * ld, bufs, bt, tid, lo2);
    cp_async_commit();
    for (int cur = 0; t < ntiles; cur ^= 1) {
        const unsigned long long base = bt | lo;
        float2* outc = out + c * ld;
        // [partials of item t]: thread-private staging slots, read back by the same thread
#pragma unroll
        for (int j = 0; j < E; j++) {
            if (p.diag) cp_async4(reinterpret_cast<float*>(stage) + tid + TB * j, diag + (base | hi_off[j]));
            else if (p.accumulate) cp_async8(stage + tid + TB * j, outc + (base | hi_off[j]));
        }
        cp_async_commit();
        if (tn < ntiles) issue_tile<E, TB>(p, in + cn * ld, bufs + (cur ^ 1) * (TB * E), bn, tid, lo2);   // [item t+1]
        cp_async_commit();
        cp_async_wait<2>();         // tile of the item has landed
        __syncthreads();
        float2* tile = bufs + cur * (TB * E);
        const float2 vfx = make_float2(p.fx[c], p.fx[c]);
        const float fy = p.fy[c], fz = p.fz[c];
        float2 acc[E];
#pragma unroll
        for (int j = 0; j < E; j++) acc[j] = make_float2(0.f, 0.f);
        terms(tile, tid, vfx, fy, acc);
        cp_async_wait<1>();         // partials of the item have landed (the next tile may be in flight)
#pragma unroll
        for (int j = 0; j < E; j++) {
            const unsigned long long k = base | hi_off[j];
            float2 o = acc[j];
            if (p.diag) {
                const float dgv = fmaf(fz, (float)(p.N - 2 * __popcll(k)), reinterpret_cast<const float*>(stage)[tid + TB * j]);
                const float2 v = tile[tid + TB * j];
                o.x = fmaf(dgv, v.x, o.x);
                o.y = fmaf(dgv, v.y, o.y);
            } else if (p.accumulate) {
                const float2 pr = stage[tid + TB * j];
                o.x += pr.x;
                o.y += pr.y;
            }
            outc[k] = o;
            acc[j] = o;
        }
        if (p.dotp) dot_item<E, TB>(da, c, tid, tile, acc);
        __syncthreads();   // buffer `cur` is refilled two items later; staging reused next item
        t = tn; c = cn; bt = bn;
        advance(tn, cn, bn);
    }
    cp_async_wait<0>();
    if (p.dotp) da.store(p, cmask, tid, TB / 32);
}

// 2-stage tile ring + staging area, one item ahead (see pass_body, NS = 5).
template <int E, int TB, class Terms>
__device__ __forceinline__ void pass_body_ahead(const PassTab& p, const Terms& terms, const float* __restrict__ diag,
                                                const float2* __restrict__ in, float2* __restrict__ out,
                                                long long ntiles, const int* __restrict__ active) {
    const unsigned cmask = column_mask(p, active);
    if (!cmask) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);   // 2 x (TB E) states
    float2* stage = bufs + 2 * TB * E;                     // TB E partials (or diagonal entries)
    __shared__ unsigned long long hi_off[E];
    __shared__ float dsm[MAXC][32][4];
    DotAcc da{dsm};
    const int tid = threadIdx.x;
    unsigned long long lo, lo2[2];
    tile_offsets<E, TB>(p, tid, hi_off, lo, lo2);
    if (p.dotp) da.clear(tid, TB);
    __syncthreads();
    const long long g = gridDim.x;
    const long long ld = p.ld;
    const int c0 = __ffs((int)cmask) - 1;
    const unsigned long long dg = tile_bits(p, g);
    auto advance = [&](long long& tt, int& cc, unsigned long long& bb) {
        const int nx = next_column(cmask, cc);
        if (nx >= 0) {
            cc = nx;
        } else {
            cc = c0;
            tt += g;
            bb = deposit_add(bb, dg, p.rmask);
        }
    };
    // copies of item (tt, cc): its tile into buffer `slot`, the same tile of the partial result (or
    // of the diagonal) into the staging area, in tile layout
    auto issue = [&](long long tt, int cc, unsigned long long bb, int slot) {
        if (tt < ntiles) {
            issue_tile<E, TB>(p, in + cc * ld, bufs + slot * (TB * E), bb, tid, lo2);
            if (p.diag) issue_tile_f32<E, TB>(p, diag, reinterpret_cast<float*>(stage), bb, tid);
            else if (p.accumulate) issue_tile<E, TB>(p, out + cc * ld, stage, bb, tid, lo2);
        }
        cp_async_commit();
    };
    long long t = blockIdx.x;
    int c = c0;
    unsigned long long bt = tile_bits(p, t);
    issue(t, c, bt, 0);
    long long tn = t;
    int cn = c;
    unsigned long long bn = bt;
    advance(tn, cn, bn);
    for (int cur = 0; t < ntiles; cur ^= 1) {
        cp_async_wait<0>();
        __syncthreads();   // item t's tile (every thread's copies) has landed; buffer cur^1 is free
        float2 pre[E];
        float dpre[E];
#pragma unroll
        for (int j = 0; j < E; j++) {
            if (p.diag) dpre[j] = reinterpret_cast<const float*>(stage)[tid + TB * j];
            else if (p.accumulate) pre[j] = stage[tid + TB * j];
        }
        __syncthreads();   // every thread's staging reads are performed before the area is refilled
        issue(tn, cn, bn, cur ^ 1);   // [item t+1]
        float2* tile = bufs + cur * (TB * E);
        float2* outc = out + c * ld;
        const unsigned long long base = bt | lo;
        const float2 vfx = make_float2(p.fx[c], p.fx[c]);
        const float fy = p.fy[c], fz = p.fz[c];
        float2 acc[E];
#pragma unroll
        for (int j = 0; j < E; j++) acc[j] = make_float2(0.f, 0.f);
        terms(tile, tid, vfx, fy, acc);
#pragma unroll
        for (int j = 0; j < E; j++) {
            const unsigned long long k = base | hi_off[j];
            float2 o = acc[j];
            if (p.diag) {
                const float dgv = fmaf(fz, (float)(p.N - 2 * __popcll(k)), dpre[j]);
                const float2 v = tile[tid + TB * j];
                o.x = fmaf(dgv, v.x, o.x);
                o.y = fmaf(dgv, v.y, o.y);
            } else if (p.accumulate) {
                o.x += pre[j].x;
                o.y += pre[j].y;
            }
            outc[k] = o;
            acc[j] = o;
        }
        if (p.dotp) dot_item<E, TB>(da, c, tid, tile, acc);
        t = tn; c = cn; bt = bn;
        advance(tn, cn, bn);
    }
    cp_async_wait<0>();
    if (p.dotp) da.store(p, cmask, tid, TB / 32);
}

// One pass over all tiles.  Terms: functor terms(tile, tid, vfx, fy, acc) adding the off-diagonal
// terms of the pass for the thread's E states.  diag (pass 1): bond part of the diagonal per state.
// NS-stage ring of tile buffers: the next NS-1 items are in flight while one is computed; every
// iteration commits exactly one cp.async group (possibly empty), so wait_group<NS-1> always means
// "the current item's tile has landed".
//
// NS = 4 is a 2-stage ring plus a staging area for the per-state loads of the epilogue (the
// partial result of the earlier passes, or the bond diagonal in pass 1): they are copied with
// cp.async as well, so no register holds them while the terms are applied and the compiler cannot
// sink them next to their use.  Commit order per iteration: [partials of item i] [tile of item i+1].
//
// NS = 5 runs the same two tile buffers and staging area one item ahead, with the partials (or the
// diagonal) copied as a tile, in 16-byte runs like the input: at the top of item i each thread
// moves its states' staged partials into registers, and then the copies of item i+1's tile and
// partials are issued, so they are in flight while item i is computed and stored, and neither the
// terms nor the epilogue of an item waits for DRAM.
template <int E, int NS, class Terms, int TB = TPB>
__device__ __forceinline__ void pass_body(const PassTab& p, const Terms& terms, const float* __restrict__ diag,
                                          const float2* __restrict__ in, float2* __restrict__ out, long long ntiles,
                                          const int* __restrict__ active) {
    if constexpr (NS == 4) {
        pass_body_staged<E, TB>(p, terms, diag, in, out, ntiles, active);
        return;
    }
    if constexpr (NS == 5) {
        pass_body_ahead<E, TB>(p, terms, diag, in, out, ntiles, active);
        return;
    }
    const unsigned cmask = column_mask(p, active);
    if (!cmask) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);   // NS x (TB E) states
    __shared__ unsigned long long hi_off[E];
    __shared__ float dsm[MAXC][32][4];
    DotAcc da{dsm};
    const int tid = threadIdx.x;
    unsigned long long lo, lo2[2];
    tile_offsets<E, TB>(p, tid, hi_off, lo, lo2);
    if (p.dotp) da.clear(tid, TB);
    __syncthreads();
    const long long g = gridDim.x;
    const long long ld = p.ld;
    const int c0 = __ffs((int)cmask) - 1;
    const unsigned long long dg = tile_bits(p, g);
    auto advance = [&](long long& tt, int& cc, unsigned long long& bb) {
        const int nx = next_column(cmask, cc);
        if (nx >= 0) {
            cc = nx;
        } else {
            cc = c0;
            tt += g;
            bb = deposit_add(bb, dg, p.rmask);
        }
    };
    // issue cursor: the next item to copy
    long long ti = blockIdx.x;
    int ci = c0;
    unsigned long long bi = tile_bits(p, ti);
    auto issue = [&](int slot) {
        if (ti < ntiles) issue_tile<E, TB>(p, in + ci * ld, bufs + slot * (TB * E), bi, tid, lo2);
        cp_async_commit();
        advance(ti, ci, bi);
    };
#pragma unroll
    for (int s = 0; s < NS - 1; s++) issue(s);
    long long t = blockIdx.x;
    int c = c0;
    unsigned long long bt = tile_bits(p, t);
    for (int cur = 0; t < ntiles; cur = (cur + 1 == NS ? 0 : cur + 1), advance(t, c, bt)) {
        issue(cur == 0 ? NS - 1 : cur - 1);
        cp_async_wait<NS - 1>();
        __syncthreads();
        float2* tile = bufs + cur * (TB * E);
        float2* outc = out + c * ld;
        const unsigned long long base = bt | lo;
        const float2 vfx = make_float2(p.fx[c], p.fx[c]);
        const float fy = p.fy[c], fz = p.fz[c];
        float2 acc[E], pre[E];
        float dpre[E];
#pragma unroll
        for (int j = 0; j < E; j++) {
            acc[j] = make_float2(0.f, 0.f);
            if (p.diag) dpre[j] = diag[base | hi_off[j]];
            else if (p.accumulate) pre[j] = outc[base | hi_off[j]];
        }
        terms(tile, tid, vfx, fy, acc);
#pragma unroll
        for (int j = 0; j < E; j++) {
            const unsigned long long k = base | hi_off[j];
            float2 o = acc[j];
            if (p.diag) {
                const float dgv = fmaf(fz, (float)(p.N - 2 * __popcll(k)), dpre[j]);
                const float2 v = tile[tid + TB * j];
                o.x = fmaf(dgv, v.x, o.x);
                o.y = fmaf(dgv, v.y, o.y);
            } else if (p.accumulate) {
                o.x += pre[j].x;
                o.y += pre[j].y;
            }
            outc[k] = o;
            acc[j] = o;
        }
        if (p.dotp) dot_item<E, TB>(da, c, tid, tile, acc);
        __syncthreads();   // buffer `cur` is refilled by a later iteration's prefetch
    }
    cp_async_wait<0>();
    if (p.dotp) da.store(p, cmask, tid, TB / 32);
}

// ---------------------------------------------------------------------------------------------
// Slab pairs.  Two passes A and B whose tiles together span U bits run in one launch over slabs of
// 2^U states (the states that agree on the other N - U bits): a slab's tiles of A, then its tiles
// of B, which read the partial result that A wrote into the slab.  At U = 21 a slab is 16 MB of
// complex64 states, so B finds the slab's input and A's partial result in the L2 cache: for the two
// passes, DRAM sees one read of the input, one read of the earlier partial (or the diagonal) and
// one write of the result, as for a single pass.
//
// Items (one tile of one pass each) are dealt round-robin to the CTAs in the order
//     A(0) | A(1) B(0) | A(2) B(1) | ... | A(S-1) B(S-2) | B(S-1)
// (A(s): the 2^(U-T) tiles of A in slab s), so B(s) begins one slab after A(s).  Before computing
// a tile of B(s), a CTA waits until every tile of A(s) has been written (a per-slab counter,
// raised after a tile's stores with a fence).  The launch is cooperative, so all CTAs are
// resident, and every tile that a wait depends on comes earlier in the order and waits for
// nothing itself: the waits end.  Each wait still gives up after about a second, sets *err and
// lets the launch finish (with a wrong result, which the host reports).
struct PairTab {
    unsigned char rest[2][40];   // per pass: global bits of the tile number, slab-internal bits first
    int nrest;                   // N - T
    int inner;                   // U - T: log2 of the tiles of one pass in one slab
    long long nslab;             // 2^(N - U)
    unsigned* cnt;               // [nslab] tiles of A written, per slab (zero at launch)
    unsigned* err;               // set to 1 by a wait that gave up
    unsigned need;               // tiles of A per slab: 2^inner
};

// item k -> pass (sec = 0: A, 1: B), slab s and tile number t = s 2^inner + (tile in slab)
__host__ __device__ __forceinline__ void pair_item(const PairTab& st, long long k, int& sec, long long& s, long long& t) {
    const long long q = k >> st.inner;
    if (q == 0) {
        sec = 0; s = 0;
    } else if (q == 2 * st.nslab - 1) {
        sec = 1; s = st.nslab - 1;
    } else if (q & 1) {
        sec = 0; s = (q + 1) >> 1;
    } else {
        sec = 1; s = (q >> 1) - 1;
    }
    t = (s << st.inner) | (k & ((1ll << st.inner) - 1));
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}
// Waits until *cnt >= need.  Gives up after about one second (and after 2^24 polls whatever the
// timer says), setting *err; returns at once once an earlier wait of the launch has given up.
static __device__ __noinline__ void wait_slab(const unsigned* cnt, unsigned need, unsigned* err) {
    if (ld_acquire_u32(cnt) >= need) return;
    const unsigned long long t0 = globaltimer_ns();
    for (unsigned it = 0; it < (1u << 24); it++) {
        __nanosleep(200);
        if (ld_acquire_u32(cnt) >= need) return;
        if ((it & 63) == 0) {
            if (ld_acquire_u32(err)) return;
            if (globaltimer_ns() - t0 > 1000000000ull) break;
        }
    }
    atomicExch(err, 1u);
}

// One launch of a slab pair (single column, 2 tile buffers).  Per state the same operations in the
// same order as pass_body, so the result is bit-identical to the two passes run one after the other.
// The per-pass tables the items need (tile-number bits, run offsets) are copied to shared memory
// once, so an item's addresses cost a few shared-memory loads.
template <int E, int TB, class TermsA, class TermsB>
__device__ __forceinline__ void pair_body(const PassTab& pa, const PassTab& pb, const PairTab& st, const TermsA& ta,
                                          const TermsB& tb, const float* __restrict__ diag,
                                          const float2* __restrict__ in, float2* __restrict__ out,
                                          const int* __restrict__ active) {
    if (active && !active[0]) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* bufs = reinterpret_cast<float2*>(smem_raw);   // 2 x (TB E) states
    __shared__ unsigned long long hi_off[2][E];
    __shared__ unsigned long long s_lo[2][64], s_hi[2][16];   // PassTab::tabLo / tabHi of A and B
    __shared__ unsigned long long lut[2][5][64];              // tile number, 6 bits at a time -> global bits
    __shared__ float dsm[MAXC][32][4];
    DotAcc da{dsm};
    const int tid = threadIdx.x;
    if (tid < E) {
        hi_off[0][tid] = pa.tabLo[((TB * tid) >> 3) & 63] | pa.tabHi[(TB * tid) >> 9];
        hi_off[1][tid] = pb.tabLo[((TB * tid) >> 3) & 63] | pb.tabHi[(TB * tid) >> 9];
    }
    for (int i = tid; i < 64; i += TB) {
        s_lo[0][i] = pa.tabLo[i];
        s_lo[1][i] = pb.tabLo[i];
    }
    for (int i = tid; i < 16; i += TB) {
        s_hi[0][i] = pa.tabHi[i];
        s_hi[1][i] = pb.tabHi[i];
    }
    for (int i = tid; i < 2 * 5 * 64; i += TB) {
        const int x = i / 320, c = (i / 64) % 5, v = i & 63;
        unsigned long long b = 0;
        for (int q = 0; q < 6; q++)
            if (6 * c + q < st.nrest && ((v >> q) & 1)) b |= 1ull << st.rest[x][6 * c + q];
        lut[x][c][v] = b;
    }
    if (pb.dotp) da.clear(tid, TB);
    __syncthreads();
    auto tile_of = [&](int x, long long t) {
        return lut[x][0][t & 63] | lut[x][1][(t >> 6) & 63] | lut[x][2][(t >> 12) & 63] | lut[x][3][(t >> 18) & 63] |
               lut[x][4][(t >> 24) & 63];
    };
    const long long g = gridDim.x;
    const long long total = (2 * st.nslab) << st.inner;
    long long ki = blockIdx.x;   // issue cursor
    auto issue = [&](int slot) {
        if (ki < total) {
            int sec;
            long long s, t;
            pair_item(st, ki, sec, s, t);
            const unsigned long long b = tile_of(sec, t);
            const unsigned long long l0 = s_lo[sec][(tid >> 2) & 63] | (unsigned long long)((2 * tid) & 7);
            const unsigned long long l1 = s_lo[sec][((tid >> 2) + 32) & 63] | (unsigned long long)((2 * tid) & 7);
            float2* dst = bufs + slot * (TB * E);
#pragma unroll
            for (int i = 0; i < E / 2; i++) {   // as issue_tile
                const unsigned long long l = (TB == 128 && (i & 1)) ? l1 : l0;
                cp_async16(dst + 2 * (tid + TB * i), in + (b | l | s_hi[sec][(tid + TB * i) >> 8]));
            }
        }
        cp_async_commit();
        ki += g;
    };
    const int N = pa.N;
    const float2 vfx = make_float2(pa.fx[0], pa.fx[0]);
    const float fy = pa.fy[0], fz = pa.fz[0];
    issue(0);
    int cur = 0;
    for (long long k = blockIdx.x; k < total; k += g, cur ^= 1) {
        issue(cur ^ 1);
        int sec;
        long long s, t;
        pair_item(st, k, sec, s, t);
        if (sec && tid == 0) wait_slab(st.cnt + s, st.need, st.err);
        cp_async_wait<1>();
        __syncthreads();
        const unsigned long long base =
            tile_of(sec, t) | s_lo[sec][(tid >> 3) & 63] | s_hi[sec][tid >> 9] | (unsigned long long)(tid & 7);
        const unsigned long long* ho = hi_off[sec];
        float2* tile = bufs + cur * (TB * E);
        const int pdiag = sec ? pb.diag : pa.diag, pacc = sec ? pb.accumulate : pa.accumulate;
        float2 acc[E], pre[E];
        float dpre[E];
#pragma unroll
        for (int j = 0; j < E; j++) {
            acc[j] = make_float2(0.f, 0.f);
            if (pdiag) dpre[j] = diag[base | ho[j]];
            else if (pacc) pre[j] = __ldcg(out + (base | ho[j]));
        }
        if (sec) tb(tile, tid, vfx, fy, acc);
        else ta(tile, tid, vfx, fy, acc);
#pragma unroll
        for (int j = 0; j < E; j++) {
            const unsigned long long kk = base | ho[j];
            float2 o = acc[j];
            if (pdiag) {
                const float dgv = fmaf(fz, (float)(N - 2 * __popcll(kk)), dpre[j]);
                const float2 v = tile[tid + TB * j];
                o.x = fmaf(dgv, v.x, o.x);
                o.y = fmaf(dgv, v.y, o.y);
            } else if (pacc) {
                o.x += pre[j].x;
                o.y += pre[j].y;
            }
            out[kk] = o;
            acc[j] = o;
        }
        if (sec && pb.dotp) dot_item<E, TB>(da, 0, tid, tile, acc);
        __syncthreads();   // buffer `cur` is refilled by the next iteration's prefetch
        if (!sec && tid == 0) {
            __threadfence();   // the tile's stores (ordered before by the barrier) before the count
            atomicAdd(st.cnt + s, 1u);
        }
    }
    cp_async_wait<0>();
    if (pb.dotp) da.store(pb, 1u, tid, TB / 32);
}

}  // namespace escdev
