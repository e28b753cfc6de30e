// kernels.cu -- sm_103a kernels of the Lanczos ED library: H.v gathers, operator apply,
// deterministic reductions, Krylov-basis GEMVs.  R = double (complex128 storage and arithmetic)
// or float (complex64 storage and arithmetic, double accumulation in every reduction).
//
// All kernels are pull-style gathers: each output element is written by exactly one thread, so
// there are no atomics and results are bit-reproducible for a given launch geometry.
#include <cuda_runtime.h>

#include "esc_internal.h"

namespace esc {

template <typename R> struct V2;
template <> struct V2<double> { typedef double2 T; };
template <> struct V2<float> { typedef float2 T; };

// Float-float accumulation (Dekker/Knuth error-free transforms): the complex64 path keeps its
// reductions at ~2^-44 relative accuracy without FP64 arithmetic, which GB300 executes at a small
// fraction of the FP32 rate.
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
    const float s = hi + x;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (x - bp);
    hi = s;
    lo += err;
}
__device__ __forceinline__ void ff_addprod(float& hi, float& lo, float a, float b) {
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    ff_add(hi, lo, p);
    lo += e;
}

static inline int grid_for(int64_t n, int tpb, int max_blocks) {
    int64_t g = (n + tpb - 1) / tpb;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return (int)g;
}
static constexpr int SMS = 152;

int red_blocks(int64_t n) {
    // Fixed function of n: identical launch geometry (and so identical rounding) on every call.
    return grid_for(n, 2048, RED_MAX_BLOCKS);
}

// =============================================================================================
// Operator strings (src/Observables.h: single-site ops :429-521, currents :161-470, totals)
// =============================================================================================
template <typename R>
__global__ void __launch_bounds__(256) k_apply(const __grid_constant__ DevOp op,
                                               const typename V2<R>::T* __restrict__ in,
                                               typename V2<R>::T* __restrict__ out, long long D) {
    typedef typename V2<R>::T C;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < D; k += stride) {
        R ar = 0, ai = 0;
        for (int t = 0; t < op.nt; t++) {
            const unsigned long long k0 = (unsigned long long)k ^ op.flip[t];
            const unsigned int fac = op.fac[t];
            const int nf = fac & 3;
            R cr = sizeof(R) == 4 ? (R)op.cref[t] : (R)op.cre[t], ci = sizeof(R) == 4 ? (R)op.cimf[t] : (R)op.cim[t];
            unsigned long long ket = k0;
            for (int q = 0; q < nf; q++) {
                const int s = (fac >> (2 + 8 * q)) & 63;
                const int o = (fac >> (8 + 8 * q)) & 3;
                const R h = ((ket >> s) & 1ull) ? (R)-0.5 : (R)0.5;
                if (o == 1) { cr *= (R)0.5; ci *= (R)0.5; ket ^= 1ull << s; }         // S^x: 1/2, flip
                else if (o == 2) { const R nr = -ci * h, ni = cr * h; cr = nr; ci = ni; ket ^= 1ull << s; }  // S^y: +-i/2
                else { cr *= h; ci *= h; }                                            // S^z: +-1/2
            }
            const C w = in[k0];
            const R r = cr, i = ci;
            ar = fma(r, w.x, ar); ar = fma(-i, w.y, ar);
            ai = fma(r, w.y, ai); ai = fma(i, w.x, ai);
        }
        C o; o.x = ar; o.y = ai;
        out[k] = o;
    }
}

template <typename R>
void launch_apply(const DevOp& op, const void* in, void* out, int64_t D, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_apply<R><<<grid_for(D, 256, SMS * 16), 256, 0, s>>>(op, (const C*)in, (C*)out, (long long)D);
    ESC_CUDA(cudaGetLastError());
}

// =============================================================================================
// Deterministic reductions (double accumulation, fixed grid, fixed butterfly tree)
// =============================================================================================
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double* dst) {
    // 256 threads: warp butterflies, then 8 warp results summed in warp order by warp 0.
    __shared__ double sm[8][NV];
#pragma unroll
    for (int q = 0; q < NV; q++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0)
#pragma unroll
        for (int q = 0; q < NV; q++) sm[w][q] = v[q];
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += sm[i][threadIdx.x];
        dst[threadIdx.x] = s;
    }
    __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(256) k_dot_partial(const typename V2<R>::T* __restrict__ a,
                                                     const typename V2<R>::T* __restrict__ b, long long n,
                                                     double* __restrict__ partials) {
    double v[2] = {0.0, 0.0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    if constexpr (sizeof(R) == 4) {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float2 x = a[i], y = b[i];
            ff_addprod(rh, rl, x.x, y.x); ff_addprod(rh, rl, x.y, y.y);
            ff_addprod(ih, il, x.x, y.y); ff_addprod(ih, il, -x.y, y.x);
        }
        v[0] = (double)rh + (double)rl;
        v[1] = (double)ih + (double)il;
    } else {
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const double xr = a[i].x, xi = a[i].y, yr = b[i].x, yi = b[i].y;
            v[0] += xr * yr + xi * yi;
            v[1] += xr * yi - xi * yr;
        }
    }
    block_reduce_store<2>(v, partials + 2 * blockIdx.x);
}

template <typename R>
__global__ void __launch_bounds__(256) k_nrm2_partial(const typename V2<R>::T* __restrict__ a, long long n,
                                                      double* __restrict__ partials) {
    double v[1] = {0.0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    if constexpr (sizeof(R) == 4) {
        float hh = 0.f, ll = 0.f;
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const float2 x = a[i];
            ff_addprod(hh, ll, x.x, x.x); ff_addprod(hh, ll, x.y, x.y);
        }
        v[0] = (double)hh + (double)ll;
    } else {
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const double xr = a[i].x, xi = a[i].y;
            v[0] += xr * xr + xi * xi;
        }
    }
    block_reduce_store<1>(v, partials + blockIdx.x);
}

// Sum NV-vectors of nparts partials (stride NV) in a fixed order into dst[NV].
template <int NV>
__global__ void __launch_bounds__(256) k_finalize(const double* __restrict__ partials, int nparts,
                                                  double* __restrict__ dst) {
    double v[NV];
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
#pragma unroll
        for (int q = 0; q < NV; q++) v[q] += partials[(size_t)i * NV + q];
    block_reduce_store<NV>(v, dst);
}

template <typename R>
void launch_dot(const void* a, const void* b, int64_t n, double* partials, double* dst, cudaStream_t s) {
    typedef typename V2<R>::T C;
    const int g = red_blocks(n);
    k_dot_partial<R><<<g, 256, 0, s>>>((const C*)a, (const C*)b, n, partials);
    k_finalize<2><<<1, 256, 0, s>>>(partials, g, dst);
    ESC_CUDA(cudaGetLastError());
}

template <typename R>
void launch_nrm2(const void* a, int64_t n, double* partials, double* dst, cudaStream_t s) {
    typedef typename V2<R>::T C;
    const int g = red_blocks(n);
    k_nrm2_partial<R><<<g, 256, 0, s>>>((const C*)a, n, partials);
    k_finalize<1><<<1, 256, 0, s>>>(partials, g, dst);
    ESC_CUDA(cudaGetLastError());
}

// w = (w - alpha v) - beta u ; |w|^2 partials.  Mirrors V2 - alpha*V1 - beta*V0
// (src/DynLanczosSolver.h:96) with complex alpha and real beta.
template <typename R>
__global__ void __launch_bounds__(256) k_lanczos_update(typename V2<R>::T* __restrict__ w,
                                                        const typename V2<R>::T* __restrict__ v,
                                                        const typename V2<R>::T* __restrict__ u,
                                                        const double* __restrict__ d_alpha,
                                                        const double* __restrict__ d_beta2, long long n,
                                                        double* __restrict__ partials) {
    typedef typename V2<R>::T C;
    const R are = (R)d_alpha[0], aim = (R)d_alpha[1];
    const R be = d_beta2 ? (R)sqrt(d_beta2[0]) : (R)0;   // beta = |w_prev| = sqrt(|w_prev|^2)
    double acc[1] = {0.0};
    float hh = 0.f, ll = 0.f;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        C x = w[i];
        const C y = v[i];
        x.x = x.x - (are * y.x - aim * y.y);
        x.y = x.y - (are * y.y + aim * y.x);
        if (u) {
            const C z = u[i];
            x.x = x.x - be * z.x;
            x.y = x.y - be * z.y;
        }
        w[i] = x;
        if constexpr (sizeof(R) == 4) { ff_addprod(hh, ll, x.x, x.x); ff_addprod(hh, ll, x.y, x.y); }
        else acc[0] += (double)x.x * (double)x.x + (double)x.y * (double)x.y;
    }
    if constexpr (sizeof(R) == 4) acc[0] = (double)hh + (double)ll;
    block_reduce_store<1>(acc, partials + blockIdx.x);
}

template <typename R>
void launch_lanczos_update(void* w, const void* v, const void* u, const double* d_alpha, const double* d_beta2,
                           int64_t n, double* partials, double* dst, cudaStream_t s) {
    typedef typename V2<R>::T C;
    const int g = red_blocks(n);
    k_lanczos_update<R><<<g, 256, 0, s>>>((C*)w, (const C*)v, (const C*)u, d_alpha, d_beta2, n, partials);
    k_finalize<1><<<1, 256, 0, s>>>(partials, g, dst);
    ESC_CUDA(cudaGetLastError());
}

template <typename R>
__global__ void __launch_bounds__(256) k_scale_rsqrt(const typename V2<R>::T* in, typename V2<R>::T* out,
                                                     const double* __restrict__ d_nrm2, long long n) {
    typedef typename V2<R>::T C;
    // |w| = 0 (Krylov space exhausted) leaves a zero vector instead of NaNs; the host reports it.
    const double nrm = sqrt(d_nrm2[0]);
    const double inv_ok = nrm > 0.0 ? 1.0 : 0.0;
    const double den = nrm > 0.0 ? nrm : 1.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    if constexpr (sizeof(R) == 4) {
        const float inv = (float)(inv_ok / den);
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const C x = in[i];
            C y;
            y.x = x.x * inv;
            y.y = x.y * inv;
            out[i] = y;
        }
    } else {
        // Eigen's normalize() divides by the norm (src/DynLanczosSolver.h:100)
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            const C x = in[i];
            C y;
            y.x = (R)(inv_ok * ((double)x.x / den));
            y.y = (R)(inv_ok * ((double)x.y / den));
            out[i] = y;
        }
    }
}

template <typename R>
void launch_scale_rsqrt(const void* in, void* out, const double* d_nrm2, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_scale_rsqrt<R><<<grid_for(n, 256, SMS * 16), 256, 0, s>>>((const C*)in, (C*)out, d_nrm2, n);
    ESC_CUDA(cudaGetLastError());
}

template <typename R>
__global__ void __launch_bounds__(256) k_axpby(const typename V2<R>::T* x, const typename V2<R>::T* y,
                                               typename V2<R>::T* out, double ar, double ai, double br, double bi,
                                               long long n) {
    typedef typename V2<R>::T C;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const C p = x[i], q = y[i];
        const R a_r = (R)ar, a_i = (R)ai, b_r = (R)br, b_i = (R)bi;
        C o;
        o.x = a_r * p.x - a_i * p.y + b_r * q.x - b_i * q.y;
        o.y = a_r * p.y + a_i * p.x + b_r * q.y + b_i * q.x;
        out[i] = o;
    }
}

template <typename R>
void launch_axpby(const void* x, const void* y, void* out, cplx a, cplx b, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_axpby<R><<<grid_for(n, 256, SMS * 16), 256, 0, s>>>((const C*)x, (const C*)y, (C*)out, a.real(), a.imag(),
                                                         b.real(), b.imag(), n);
    ESC_CUDA(cudaGetLastError());
}

// r[j] = sum_k conj(L_j[k]) w[k] for j < m, in groups of JB columns; partials [m][G][2].
template <typename R, int JB>
__global__ void __launch_bounds__(256) k_gemv_h(const typename V2<R>::T* __restrict__ L, long long ld, int m,
                                                const typename V2<R>::T* __restrict__ w, long long n,
                                                double* __restrict__ partials) {
    const int G = gridDim.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (int j0 = 0; j0 < m; j0 += JB) {
        double v[2 * JB];
#pragma unroll
        for (int q = 0; q < 2 * JB; q++) v[q] = 0.0;
        if constexpr (sizeof(R) == 4) {
            float hv[2 * JB], lv[2 * JB];
#pragma unroll
            for (int q = 0; q < 2 * JB; q++) hv[q] = lv[q] = 0.f;
            for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
                const float2 y = w[i];
#pragma unroll
                for (int q = 0; q < JB; q++)
                    if (j0 + q < m) {
                        const float2 x = L[(long long)(j0 + q) * ld + i];
                        ff_addprod(hv[2 * q], lv[2 * q], x.x, y.x); ff_addprod(hv[2 * q], lv[2 * q], x.y, y.y);
                        ff_addprod(hv[2 * q + 1], lv[2 * q + 1], x.x, y.y); ff_addprod(hv[2 * q + 1], lv[2 * q + 1], -x.y, y.x);
                    }
            }
#pragma unroll
            for (int q = 0; q < 2 * JB; q++) v[q] = (double)hv[q] + (double)lv[q];
        } else {
            for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
                const double yr = w[i].x, yi = w[i].y;
#pragma unroll
                for (int q = 0; q < JB; q++)
                    if (j0 + q < m) {
                        const typename V2<R>::T x = L[(long long)(j0 + q) * ld + i];
                        v[2 * q] += (double)x.x * yr + (double)x.y * yi;
                        v[2 * q + 1] += (double)x.x * yi - (double)x.y * yr;
                    }
            }
        }
        __shared__ double out[2 * JB];
        block_reduce_store<2 * JB>(v, out);
        if (threadIdx.x < 2 * JB && j0 + (int)threadIdx.x / 2 < m)
            partials[((size_t)(j0 + threadIdx.x / 2) * G + blockIdx.x) * 2 + (threadIdx.x & 1)] = out[threadIdx.x];
    }
}

__global__ void __launch_bounds__(256) k_finalize_rows(const double* __restrict__ partials, int G, int m,
                                                       double* __restrict__ r) {
    // one block per row j
    const int j = blockIdx.x;
    double v[2] = {0.0, 0.0};
    for (int i = threadIdx.x; i < G; i += blockDim.x) {
        v[0] += partials[((size_t)j * G + i) * 2];
        v[1] += partials[((size_t)j * G + i) * 2 + 1];
    }
    block_reduce_store<2>(v, r + 2 * j);
}

template <typename R>
void launch_gemv_h(const void* L, int64_t ld, int m, const void* w, int64_t n, double* partials,
                   int64_t partials_cap, double* r, cudaStream_t s) {
    typedef typename V2<R>::T C;
    if (m <= 0) return;
    int g = red_blocks(n);
    while ((int64_t)m * g * 2 > partials_cap && g > 1) g = (g + 1) / 2;
    k_gemv_h<R, 4><<<g, 256, 0, s>>>((const C*)L, ld, m, (const C*)w, n, partials);
    k_finalize_rows<<<m, 256, 0, s>>>(partials, g, m, r);
    ESC_CUDA(cudaGetLastError());
}

// w[k] -= sum_j L_j[k] r_j (complex r, double accumulation)
template <typename R>
__global__ void __launch_bounds__(256) k_gemv_sub(const typename V2<R>::T* __restrict__ L, long long ld, int m,
                                                  const double* __restrict__ r, typename V2<R>::T* __restrict__ w,
                                                  long long n) {
    extern __shared__ double rs[];
    for (int q = threadIdx.x; q < 2 * m; q += blockDim.x) rs[q] = r[q];
    __syncthreads();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename V2<R>::T y = w[i];
        if constexpr (sizeof(R) == 4) {
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int j = 0; j < m; j++) {
                const float2 x = L[(long long)j * ld + i];
                const float cr = (float)rs[2 * j], ci = (float)rs[2 * j + 1];
                ff_addprod(rh, rl, x.x, cr); ff_addprod(rh, rl, -x.y, ci);
                ff_addprod(ih, il, x.x, ci); ff_addprod(ih, il, x.y, cr);
            }
            y.x = y.x - (rh + rl);
            y.y = y.y - (ih + il);
        } else {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < m; j++) {
                const typename V2<R>::T x = L[(long long)j * ld + i];
                const double cr = rs[2 * j], ci = rs[2 * j + 1];
                sr += (double)x.x * cr - (double)x.y * ci;
                si += (double)x.x * ci + (double)x.y * cr;
            }
            y.x = (R)((double)y.x - sr);
            y.y = (R)((double)y.y - si);
        }
        w[i] = y;
    }
}

template <typename R>
void launch_gemv_sub(const void* L, int64_t ld, int m, const double* r, void* w, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    if (m <= 0) return;
    k_gemv_sub<R><<<grid_for(n, 256, SMS * 16), 256, 2 * m * sizeof(double), s>>>((const C*)L, ld, m, r, (C*)w, n);
    ESC_CUDA(cudaGetLastError());
}

template <typename R>
__global__ void __launch_bounds__(256) k_lincomb(const typename V2<R>::T* __restrict__ L, long long ld, int m,
                                                 const double* __restrict__ z, typename V2<R>::T* __restrict__ out,
                                                 long long n) {
    extern __shared__ double zs[];
    for (int q = threadIdx.x; q < m; q += blockDim.x) zs[q] = z[q];
    __syncthreads();
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename V2<R>::T y;
        if constexpr (sizeof(R) == 4) {
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int j = 0; j < m; j++) {
                const float2 x = L[(long long)j * ld + i];
                const float z = (float)zs[j];
                ff_addprod(rh, rl, x.x, z);
                ff_addprod(ih, il, x.y, z);
            }
            y.x = rh + rl;
            y.y = ih + il;
        } else {
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < m; j++) {
                const typename V2<R>::T x = L[(long long)j * ld + i];
                sr += (double)x.x * zs[j];
                si += (double)x.y * zs[j];
            }
            y.x = (R)sr;
            y.y = (R)si;
        }
        out[i] = y;
    }
}

template <typename R>
void launch_lincomb(const void* L, int64_t ld, int m, const double* z, void* out, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_lincomb<R><<<grid_for(n, 256, SMS * 16), 256, m * sizeof(double), s>>>((const C*)L, ld, m, z, (C*)out, n);
    ESC_CUDA(cudaGetLastError());
}

template <typename R>
__global__ void __launch_bounds__(256) k_axpy_dev(const typename V2<R>::T* __restrict__ x, typename V2<R>::T* __restrict__ y,
                                                  const double* __restrict__ d_coef, long long n) {
    const R c = (R)d_coef[0];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename V2<R>::T a = y[i];
        const typename V2<R>::T b = x[i];
        a.x = fma(c, b.x, a.x);
        a.y = fma(c, b.y, a.y);
        y[i] = a;
    }
}
template <typename R>
void launch_axpy_dev(const void* x, void* y, const double* d_coef, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_axpy_dev<R><<<grid_for(n, 256, SMS * 16), 256, 0, s>>>((const C*)x, (C*)y, d_coef, n);
    ESC_CUDA(cudaGetLastError());
}
template void launch_axpy_dev<double>(const void*, void*, const double*, int64_t, cudaStream_t);
template void launch_axpy_dev<float>(const void*, void*, const double*, int64_t, cudaStream_t);

__global__ void k_c128_to_c64(const double2* in, float2* out, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = make_float2((float)in[i].x, (float)in[i].y);
}
__global__ void k_c64_to_c128(const float2* in, double2* out, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = make_double2((double)in[i].x, (double)in[i].y);
}
void launch_convert_c128_to_c64(const void* in, void* out, int64_t n, cudaStream_t s) {
    k_c128_to_c64<<<grid_for(n, 256, SMS * 16), 256, 0, s>>>((const double2*)in, (float2*)out, n);
    ESC_CUDA(cudaGetLastError());
}
void launch_convert_c64_to_c128(const void* in, void* out, int64_t n, cudaStream_t s) {
    k_c64_to_c128<<<grid_for(n, 256, SMS * 16), 256, 0, s>>>((const float2*)in, (double2*)out, n);
    ESC_CUDA(cudaGetLastError());
}

// Counter-based complex normal start vector: SplitMix64 (Steele, Lea & Flood 2014) hashes of
// (seed, 2k) and (seed, 2k+1) -> two uniforms -> Box-Muller.  Not normalised here.
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
template <typename R>
__global__ void k_start_normal(unsigned long long seed, typename V2<R>::T* out, long long n) {
    const unsigned long long base = splitmix64(seed);
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long h1 = splitmix64(base ^ (2ull * (unsigned long long)i));
        const unsigned long long h2 = splitmix64(base ^ (2ull * (unsigned long long)i + 1ull));
        typename V2<R>::T o;
        if constexpr (sizeof(R) == 4) {
            const float u1 = (float)((h1 >> 40) + 1ull) * 0x1.0p-24f;   // (0, 1]
            const float u2 = (float)(h2 >> 40) * 0x1.0p-24f;            // [0, 1)
            const float r = sqrtf(-2.0f * logf(u1));
            float sn, cs;
            sincospif(2.0f * u2, &sn, &cs);
            o.x = r * cs;
            o.y = r * sn;
        } else {
            const double u1 = (double)((h1 >> 11) + 1ull) * 0x1.0p-53;   // (0, 1]
            const double u2 = (double)(h2 >> 11) * 0x1.0p-53;            // [0, 1)
            const double r = sqrt(-2.0 * log(u1));
            double sn, cs;
            sincospi(2.0 * u2, &sn, &cs);
            o.x = (R)(r * cs);
            o.y = (R)(r * sn);
        }
        out[i] = o;
    }
}
template <typename R>
void launch_start_normal(uint64_t seed, void* out, int64_t n, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_start_normal<R><<<grid_for(n, 256, SMS * 16), 256, 0, s>>>(seed, (C*)out, n);
    ESC_CUDA(cudaGetLastError());
}

// out[c][i] = (i == j0 + c) for c < ncols: unit vectors e_{j0} .. e_{j0+ncols-1}, stride D
template <typename R>
__global__ void __launch_bounds__(256) k_unit_columns(typename V2<R>::T* __restrict__ out, long long D, long long j0,
                                                      int ncols) {
    const long long n = (long long)ncols * D;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        typename V2<R>::T v;
        v.x = (i % D == j0 + i / D) ? (R)1 : (R)0;
        v.y = (R)0;
        out[i] = v;
    }
}
template <typename R>
void launch_unit_columns(void* out, int64_t D, int64_t j0, int ncols, cudaStream_t s) {
    typedef typename V2<R>::T C;
    k_unit_columns<R><<<grid_for((int64_t)ncols * D, 256, SMS * 16), 256, 0, s>>>((C*)out, D, j0, ncols);
    ESC_CUDA(cudaGetLastError());
}
template void launch_unit_columns<double>(void*, int64_t, int64_t, int, cudaStream_t);
template void launch_unit_columns<float>(void*, int64_t, int64_t, int, cudaStream_t);

// explicit instantiations
#define ESC_INST(R)                                                                                        \
    template void launch_apply<R>(const DevOp&, const void*, void*, int64_t, cudaStream_t);                \
    template void launch_dot<R>(const void*, const void*, int64_t, double*, double*, cudaStream_t);        \
    template void launch_nrm2<R>(const void*, int64_t, double*, double*, cudaStream_t);                    \
    template void launch_lanczos_update<R>(void*, const void*, const void*, const double*, const double*,  \
                                           int64_t, double*, double*, cudaStream_t);                       \
    template void launch_scale_rsqrt<R>(const void*, void*, const double*, int64_t, cudaStream_t);         \
    template void launch_axpby<R>(const void*, const void*, void*, cplx, cplx, int64_t, cudaStream_t);      \
    template void launch_gemv_h<R>(const void*, int64_t, int, const void*, int64_t, double*, int64_t,      \
                                   double*, cudaStream_t);                                                 \
    template void launch_gemv_sub<R>(const void*, int64_t, int, const double*, void*, int64_t, cudaStream_t); \
    template void launch_lincomb<R>(const void*, int64_t, int, const double*, void*, int64_t, cudaStream_t); \
    template void launch_start_normal<R>(uint64_t, void*, int64_t, cudaStream_t);
ESC_INST(double)
ESC_INST(float)

}  // namespace esc
