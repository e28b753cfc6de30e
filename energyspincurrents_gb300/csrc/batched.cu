// batched.cu -- batched continued-fraction Lanczos: independent three-term recurrences on up to
// 16 columns (each column its own start vector and its own field), run in lockstep with all
// recurrence state on the device so that one iteration can be captured in a CUDA graph and
// replayed.  A column stops when beta_k < tol * |phi| or at its own step limit; stopped columns
// skip their work (every kernel checks the column's flag).
//
// Buffers: three sets V[0..2] of ncols vectors (stride D).  At iteration it the roles are
// prev = V[it % 3], cur = V[(it + 1) % 3], w = V[(it + 2) % 3]; a graph holds three unrolled
// iterations (one per rotation), so every kernel parameter is fixed and the iteration counter is
// read from device memory.
//
// One iteration: the tiled H.V passes over all active columns (one launch per pass; the last pass
// also leaves the partial sums of <cur|H cur> per column, so alpha needs no extra sweep over the
// vectors), alpha, the update u_{k+1} (fused with its squared norm), beta and the stop test.
//
// The Lanczos vectors are kept unnormalised: u_k = beta_k v_k with beta_0 = |phi| and beta_k the
// usual off-diagonal, so no pass over the vectors only rescales them.  With w = H u_k:
//   alpha_k   = <u_k|w> / beta_k^2
//   u_{k+1}   = (w - alpha_k u_k) / beta_k - (beta_k / beta_{k-1}) u_{k-1},   beta_{k+1} = |u_{k+1}|
// which is the three-term recurrence of the normalised vectors multiplied through by beta_{k+1}.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "esc_internal.h"

namespace esc {

template <typename R> struct V2B;
template <> struct V2B<double> { typedef double2 T; };
template <> struct V2B<float> { typedef float2 T; };

__device__ __forceinline__ void bff_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}
__device__ __forceinline__ void bff_addprod(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    bff_add(hi, lo, p);
    lo += e;
}

static constexpr int BTPB = 256;
static constexpr int BGRID = CFB_GRID;   // blocks per column for the streaming kernels and reductions
static constexpr int UNR = 4;            // independent elements in flight per thread

__device__ __forceinline__ void block_sum2(double& a, double& b, double* dst) {
    __shared__ double sm[2][BTPB / 32];
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = a; sm[1][threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < BTPB / 32; w++) { x += sm[0][w]; y += sm[1][w]; }
        dst[0] = x;
        dst[1] = y;
    }
    __syncthreads();
}

// Grid-stride loop over [0, D) that hands UNR elements (i, i + stride, ...) to f at once, so
// that each thread keeps UNR independent loads in flight; the visiting order is fixed by the
// grid, which keeps the reductions built on it deterministic.
template <typename F>
__device__ __forceinline__ void stream_loop(long long D, F&& f) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (UNR - 1) * stride < D; i += UNR * stride) f(i, stride, UNR);
    for (; i < D; i += stride) f(i, stride, 1);
}

// alpha_c[it] = (sum of partials) / |u_it|^2 (one block per column)
__global__ void __launch_bounds__(BTPB) kb_alpha(const double* __restrict__ part, int G, const int* __restrict__ it_p,
                                                 const int* __restrict__ active, double* __restrict__ alpha,
                                                 const double* __restrict__ b2, int kmax) {
    const int c = blockIdx.x;
    if (!active[c]) return;
    double re = 0.0, im = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) {
        re += part[((size_t)c * G + i) * 2];
        im += part[((size_t)c * G + i) * 2 + 1];
    }
    __shared__ double out[2];
    block_sum2(re, im, out);
    if (threadIdx.x == 0) {
        const int it = *it_p;
        const double nb2 = b2[(size_t)c * (kmax + 1) + it];   // |u_it|^2 (> 0 while the column is active)
        alpha[((size_t)c * kmax + it) * 2] = out[0] / nb2;
        alpha[((size_t)c * kmax + it) * 2 + 1] = out[1] / nb2;
    }
}

// w <- u_{it+1} (the recurrence above); |u_{it+1}|^2 partials
template <typename R>
__global__ void __launch_bounds__(BTPB) kb_update(typename V2B<R>::T* __restrict__ w,
                                                  const typename V2B<R>::T* __restrict__ cur,
                                                  const typename V2B<R>::T* __restrict__ prev, long long D,
                                                  const int* __restrict__ it_p, const int* __restrict__ active,
                                                  const double* __restrict__ alpha, const double* __restrict__ b2,
                                                  int kmax, double* __restrict__ part) {
    typedef typename V2B<R>::T C;
    const int c = blockIdx.y;
    if (!active[c]) return;
    const int it = *it_p;
    // u_{it+1} = c1 w - (c2r + i c2i) u_it - c3 u_{it-1}
    const double bk = sqrt(b2[(size_t)c * (kmax + 1) + it]);
    const double bp = it > 0 ? sqrt(b2[(size_t)c * (kmax + 1) + it - 1]) : 1.0;
    const R c1 = (R)(1.0 / bk);
    const R ar = (R)(alpha[((size_t)c * kmax + it) * 2] / bk), ai = (R)(alpha[((size_t)c * kmax + it) * 2 + 1] / bk);
    const R be = it > 0 ? (R)(bk / bp) : (R)0;
    C* W = w + (size_t)c * D;
    const C* X = cur + (size_t)c * D;
    const C* P = prev + (size_t)c * D;
    double acc = 0.0, dummy = 0.0;
    float hh = 0.f, ll = 0.f;
    stream_loop(D, [&](long long i, long long st, int n) {
        C a[UNR], x[UNR], p[UNR];
#pragma unroll
        for (int u = 0; u < UNR; u++)
            if (u < n) {
                a[u] = W[i + u * st];
                x[u] = X[i + u * st];
                p[u] = it > 0 ? P[i + u * st] : C{(R)0, (R)0};
            }
#pragma unroll
        for (int u = 0; u < UNR; u++) {
            if (u >= n) break;
            C o = a[u];
            o.x = c1 * o.x - (ar * x[u].x - ai * x[u].y);
            o.y = c1 * o.y - (ar * x[u].y + ai * x[u].x);
            o.x = o.x - be * p[u].x;
            o.y = o.y - be * p[u].y;
            W[i + u * st] = o;
            if constexpr (sizeof(R) == 4) { bff_addprod(hh, ll, o.x, o.x); bff_addprod(hh, ll, o.y, o.y); }
            else acc += (double)o.x * o.x + (double)o.y * o.y;
        }
    });
    if constexpr (sizeof(R) == 4) acc = (double)hh + (double)ll;
    block_sum2(acc, dummy, part + ((size_t)c * gridDim.x + blockIdx.x) * 2);
}

// b2_c[it+1] = |w|^2; stop test; iteration counter advanced by block 0 after all columns
__global__ void __launch_bounds__(BTPB) kb_beta(const double* __restrict__ part, int G, const int* __restrict__ it_p,
                                                int* __restrict__ active, double* __restrict__ b2, int kmax,
                                                const int* __restrict__ steps, double tol) {
    const int c = blockIdx.x;
    if (!active[c]) return;
    double s = 0.0, dummy = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) s += part[((size_t)c * G + i) * 2];
    __shared__ double out[2];
    block_sum2(s, dummy, out);
    if (threadIdx.x == 0) {
        const int it = *it_p;
        b2[(size_t)c * (kmax + 1) + it + 1] = out[0];
        const double b0 = sqrt(b2[(size_t)c * (kmax + 1)]);
        // 2: stops after this iteration (kb_advance clears it)
        if (!(sqrt(out[0]) > tol * b0) || it + 1 >= steps[c]) active[c] = 2;
    }
}

__global__ void kb_advance(int* it_p, int* active, int ncols) {
    for (int c = 0; c < ncols; c++)
        if (active[c] == 2) active[c] = 0;
    *it_p += 1;
}

// |phi_c|^2 -> b2[c][0] (u_0 = phi_c, unnormalised)
template <typename R>
__global__ void __launch_bounds__(BTPB) kb_norm0(const typename V2B<R>::T* __restrict__ v, long long D,
                                                 double* __restrict__ part) {
    const int c = blockIdx.y;
    const typename V2B<R>::T* X = v + (size_t)c * D;
    double acc = 0.0, dummy = 0.0;
    float hh = 0.f, ll = 0.f;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += stride) {
        const typename V2B<R>::T a = X[i];
        if constexpr (sizeof(R) == 4) { bff_addprod(hh, ll, a.x, a.x); bff_addprod(hh, ll, a.y, a.y); }
        else acc += (double)a.x * a.x + (double)a.y * a.y;
    }
    if constexpr (sizeof(R) == 4) acc = (double)hh + (double)ll;
    block_sum2(acc, dummy, part + ((size_t)c * gridDim.x + blockIdx.x) * 2);
}
__global__ void __launch_bounds__(BTPB) kb_norm0_final(const double* __restrict__ part, int G, double* __restrict__ b2,
                                                       int kmax, int* __restrict__ active) {
    const int c = blockIdx.x;
    double s = 0.0, dummy = 0.0;
    for (int i = threadIdx.x; i < G; i += blockDim.x) s += part[((size_t)c * G + i) * 2];
    __shared__ double out[2];
    block_sum2(s, dummy, out);
    if (threadIdx.x == 0) {
        b2[(size_t)c * (kmax + 1)] = out[0];
        active[c] = out[0] > 0.0 ? 1 : 0;
    }
}

// Helpers for the ground-state Lanczos on this recurrence (one column; iteration counter on the
// device, so they can sit inside the captured iterations):
// L[it + 1] = w  (Krylov basis kept for Ritz-mode spectra)
template <typename R>
__global__ void __launch_bounds__(BTPB) kb_store(const typename V2B<R>::T* __restrict__ w, typename V2B<R>::T* __restrict__ L,
                                                 long long D, const int* __restrict__ it_p, const int* __restrict__ active) {
    if (!active[0]) return;
    typename V2B<R>::T* dst = L + (size_t)(*it_p + 1) * D;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += stride) dst[i] = w[i];
}
// gs += zc[it + 1] w  (ground state rebuilt from the regenerated vectors)
template <typename R>
__global__ void __launch_bounds__(BTPB) kb_accum(const typename V2B<R>::T* __restrict__ w, typename V2B<R>::T* __restrict__ gs,
                                                 long long D, const int* __restrict__ it_p, const double* __restrict__ zc,
                                                 const int* __restrict__ active) {
    if (!active[0]) return;
    const R z = (R)zc[*it_p + 1];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += stride) {
        typename V2B<R>::T a = gs[i];
        const typename V2B<R>::T b = w[i];
        a.x = fma(z, b.x, a.x);
        a.y = fma(z, b.y, a.y);
        gs[i] = a;
    }
}
template <typename R>
void launch_store_iter(const void* w, void* L, int64_t D, const int* d_it, const int* d_active, cudaStream_t s) {
    typedef typename V2B<R>::T C;
    kb_store<R><<<BGRID, BTPB, 0, s>>>((const C*)w, (C*)L, D, d_it, d_active);
    ESC_CUDA(cudaGetLastError());
}
template <typename R>
void launch_accum_iter(const void* w, void* gs, int64_t D, const int* d_it, const double* zc, const int* d_active,
                       cudaStream_t s) {
    typedef typename V2B<R>::T C;
    kb_accum<R><<<BGRID, BTPB, 0, s>>>((const C*)w, (C*)gs, D, d_it, zc, d_active);
    ESC_CUDA(cudaGetLastError());
}
template void launch_store_iter<float>(const void*, void*, int64_t, const int*, const int*, cudaStream_t);
template void launch_store_iter<double>(const void*, void*, int64_t, const int*, const int*, cudaStream_t);
template void launch_accum_iter<float>(const void*, void*, int64_t, const int*, const double*, const int*, cudaStream_t);
template void launch_accum_iter<double>(const void*, void*, int64_t, const int*, const double*, const int*, cudaStream_t);

template <typename R>
void CFBatch<R>::run(cudaStream_t s) {
    typedef typename V2B<R>::T C;
    const size_t vs = (size_t)ncols * D;
    C* V[3] = {(C*)bufs, (C*)bufs + vs, (C*)bufs + 2 * vs};
    const dim3 gcol(BGRID, ncols);
    if (start_it == 0) {
        // start: cur = V[1] holds phi
        ESC_CUDA(cudaMemsetAsync(d_it, 0, sizeof(int), s));
        kb_norm0<R><<<gcol, BTPB, 0, s>>>(V[1], D, d_part);
        kb_norm0_final<<<ncols, BTPB, 0, s>>>(d_part, BGRID, d_b2, kmax, d_active);
        ESC_CUDA(cudaGetLastError());
    } else {
        // pageable source: the copy completes before cudaMemcpyAsync returns
        ESC_CUDA(cudaMemcpyAsync(d_it, &start_it, sizeof(int), cudaMemcpyHostToDevice, s));
    }
    auto iteration = [&](int r) {
        C* prev = V[r % 3];
        C* cur = V[(r + 1) % 3];
        C* w = V[(r + 2) % 3];
        const int G = hv_all(cur, w, d_active, d_part, s);   // w = H cur; alpha partials per column
        kb_alpha<<<ncols, BTPB, 0, s>>>(d_part, G, d_it, d_active, d_alpha, d_b2, kmax);
        kb_update<R><<<gcol, BTPB, 0, s>>>(w, cur, prev, D, d_it, d_active, d_alpha, d_b2, kmax, d_part);
        if (after_update) after_update(w, s);
        kb_beta<<<ncols, BTPB, 0, s>>>(d_part, BGRID, d_it, d_active, d_b2, kmax, d_steps, tol);
        kb_advance<<<1, 1, 0, s>>>(d_it, d_active, ncols);
        ESC_CUDA(cudaGetLastError());
    };
    const int rounds = (kmax - start_it + 2) / 3;
    if (use_graph) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        ESC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int r = 0; r < 3; r++) iteration(start_it + r);
        ESC_CUDA(cudaStreamEndCapture(s, &g));
        ESC_CUDA(cudaGraphInstantiate(&ge, g, 0));
        for (int q = 0; q < rounds; q++) ESC_CUDA(cudaGraphLaunch(ge, s));
        ESC_CUDA(cudaStreamSynchronize(s));
        cudaGraphExecDestroy(ge);
        cudaGraphDestroy(g);
    } else {
        for (int q = 0; q < rounds; q++)
            for (int r = 0; r < 3; r++) iteration(start_it + r);
        ESC_CUDA(cudaStreamSynchronize(s));
    }
}

template struct CFBatch<float>;
template struct CFBatch<double>;

}  // namespace esc
