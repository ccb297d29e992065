// so4_peak.cu -- FMA throughput loops, the CUDA-core denominators of the roofline.
//
// The kernels of this library are bound by the FP32 (and, for the plain path, FP64)
// FMA pipes, not by HBM or tensor cores.  cuBLAS SGEMM / DGEMM rates stand in for
// those peaks in the benchmark; these loops measure the pipes directly: every thread
// runs NCH independent FMA chains for `iters` iterations (packed FP32 pairs,
// fma.rn.f32x2; scalar FP32; or FP64), enough warps per SM to hide the FMA latency,
// and writes one value per thread so nothing is optimised away.  No counterpart in
// the reference (measurement only).
#include "so4_common.cuh"

namespace {

constexpr int PEAK_THREADS = 256;
constexpr int PEAK_NCH = 8;  // independent chains per thread

__global__ void __launch_bounds__(PEAK_THREADS) k_peak_ffma2(int iters, float seed, float *out) {
    float2 acc[PEAK_NCH];
    const float2 m = make_float2(0.999999f, 1.000001f), a = make_float2(1e-7f, -1e-7f);
#pragma unroll
    for (int c = 0; c < PEAK_NCH; ++c) acc[c] = make_float2(seed + c, seed - c);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PEAK_NCH; ++c) acc[c] = __ffma2_rn(acc[c], m, a);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < PEAK_NCH; ++c) s += acc[c].x + acc[c].y;
    out[(size_t)blockIdx.x * PEAK_THREADS + threadIdx.x] = s;
}

__global__ void __launch_bounds__(PEAK_THREADS) k_peak_ffma(int iters, float seed, float *out) {
    float acc[2 * PEAK_NCH];
#pragma unroll
    for (int c = 0; c < 2 * PEAK_NCH; ++c) acc[c] = seed + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < 2 * PEAK_NCH; ++c) acc[c] = fmaf(acc[c], 0.999999f, 1e-7f);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 2 * PEAK_NCH; ++c) s += acc[c];
    out[(size_t)blockIdx.x * PEAK_THREADS + threadIdx.x] = s;
}

__global__ void __launch_bounds__(PEAK_THREADS) k_peak_dfma(int iters, float seed, float *out) {
    double acc[PEAK_NCH];
#pragma unroll
    for (int c = 0; c < PEAK_NCH; ++c) acc[c] = (double)seed + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < PEAK_NCH; ++c) acc[c] = fma(acc[c], 0.999999999, 1e-12);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < PEAK_NCH; ++c) s += acc[c];
    out[(size_t)blockIdx.x * PEAK_THREADS + threadIdx.x] = (float)s;
}

}  // namespace

extern "C" int so4_peak_fma(int kind, int iters, int blocks, float *d_out, double *h_flop, void *stream) {
    if (iters <= 0 || blocks <= 0 || !d_out || !h_flop) return SO4_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const double threads = (double)blocks * PEAK_THREADS;
    switch (kind) {
        case 0:
            k_peak_ffma2<<<blocks, PEAK_THREADS, 0, st>>>(iters, 1.f, d_out);
            *h_flop = threads * iters * PEAK_NCH * 4.0;  // 2 FMAs of 2 flops per fma.rn.f32x2
            break;
        case 1:
            k_peak_ffma<<<blocks, PEAK_THREADS, 0, st>>>(iters, 1.f, d_out);
            *h_flop = threads * iters * 2 * PEAK_NCH * 2.0;
            break;
        case 2:
            k_peak_dfma<<<blocks, PEAK_THREADS, 0, st>>>(iters, 1.f, d_out);
            *h_flop = threads * iters * PEAK_NCH * 2.0;
            break;
        default:
            return SO4_ERR_ARG;
    }
    so4_count_launch();
    return cudaGetLastError() == cudaSuccess ? SO4_OK : SO4_ERR_CUDA;
}
