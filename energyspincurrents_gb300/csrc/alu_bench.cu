// alu_bench.cu -- arithmetic ceilings of the current device: FP32 FMA, packed f32x2 FMA and FP64
// FMA throughput, for placing the H.v passes (FP32 on complex64, FP64 on complex128) against the
// ALU roofline as well as the memory one.
//
// Each thread runs CH independent FMA chains for `iters` rounds (enough independent work per warp
// to fill the pipes); the result is stored only under a condition the host makes false, so the
// chains stay live.  Timed with CUDA events around one launch after a warm-up launch.
#include <cuda_runtime.h>

#include "esc_internal.h"

namespace esc {
namespace {

constexpr int CH = 8;
constexpr int TPB_ALU = 256;

__global__ void __launch_bounds__(TPB_ALU) k_ffma(int iters, float b, float c, float* sink, int flag) {
    float a[CH];
#pragma unroll
    for (int i = 0; i < CH; i++) a[i] = (float)(threadIdx.x + i);
    for (int n = 0; n < iters; n++)
#pragma unroll
        for (int i = 0; i < CH; i++) a[i] = fmaf(a[i], b, c);
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < CH; i++) s += a[i];
    if (flag == 12345) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(TPB_ALU) k_ffma2(int iters, float b, float c, float* sink, int flag) {
    float2 a[CH];
    const float2 bb = make_float2(b, b), cc = make_float2(c, c);
#pragma unroll
    for (int i = 0; i < CH; i++) a[i] = make_float2((float)(threadIdx.x + i), (float)(threadIdx.x - i));
    for (int n = 0; n < iters; n++)
#pragma unroll
        for (int i = 0; i < CH; i++) a[i] = __ffma2_rn(a[i], bb, cc);
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < CH; i++) s += a[i].x + a[i].y;
    if (flag == 12345) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(TPB_ALU) k_dfma(int iters, double b, double c, double* sink, int flag) {
    double a[CH];
#pragma unroll
    for (int i = 0; i < CH; i++) a[i] = (double)(threadIdx.x + i);
    for (int n = 0; n < iters; n++)
#pragma unroll
        for (int i = 0; i < CH; i++) a[i] = fma(a[i], b, c);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < CH; i++) s += a[i];
    if (flag == 12345) sink[threadIdx.x] = s;
}

}  // namespace
}  // namespace esc

// out[0..2]: FP32 FMA, packed f32x2 FMA, FP64 FMA throughput in TFLOP/s (an FMA = 2 flops, a
// packed FMA = 4); out[3..5]: the kernel times in ms.
extern "C" esc_status esc_alu_peaks(double* out) {
    using namespace esc;
    if (!out) return ESC_ERR_PARAM;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        (void)cudaGetLastError();
        set_last_error("no usable CUDA device");
        return ESC_ERR_CUDA;
    }
    void* sink = nullptr;
    if (cudaMalloc(&sink, TPB_ALU * sizeof(double)) != cudaSuccess) {
        (void)cudaGetLastError();
        set_last_error("device allocation failed");
        return ESC_ERR_MEMORY;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int grid = sms * 8;   // 8 x 256 threads per SM
    const double threads = (double)grid * TPB_ALU;
    const int it32 = 1 << 14, it64 = 1 << 8;   // about a second each at the nominal rates
    auto timed = [&](auto launch) {
        launch();
        cudaEventRecord(e0);
        launch();
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        return (double)ms;
    };
    const double t0 = timed([&] { k_ffma<<<grid, TPB_ALU>>>(it32, 0.999f, 1e-3f, (float*)sink, 0); });
    const double t1 = timed([&] { k_ffma2<<<grid, TPB_ALU>>>(it32, 0.999f, 1e-3f, (float*)sink, 0); });
    const double t2 = timed([&] { k_dfma<<<grid, TPB_ALU>>>(it64, 0.999, 1e-3, (double*)sink, 0); });
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return ESC_ERR_CUDA;
    }
    out[0] = threads * it32 * CH * 2.0 / (t0 * 1e-3) / 1e12;
    out[1] = threads * it32 * CH * 4.0 / (t1 * 1e-3) / 1e12;
    out[2] = threads * it64 * CH * 2.0 / (t2 * 1e-3) / 1e12;
    out[3] = t0;
    out[4] = t1;
    out[5] = t2;
    return ESC_OK;
}
