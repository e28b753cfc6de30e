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
template <int E, int NS, class Terms, int TB = TPB>
__device__ __forceinline__ void pass_body(const PassTab& p, const Terms& terms, const float* __restrict__ diag,
                                          const float2* __restrict__ in, float2* __restrict__ out, long long ntiles,
                                          const int* __restrict__ active) {
    if constexpr (NS == 4) {
        pass_body_staged<E, TB>(p, terms, diag, in, out, ntiles, active);
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

}  // namespace escdev
