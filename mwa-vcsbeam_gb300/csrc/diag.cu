// Diagnostics: the FP32 FMA throughput of this GPU, measured by the library
// itself, as the compute denominator for the fused PFB + beamformer (whose
// arithmetic is FP32 on the CUDA cores). No reference counterpart.
#include "vgb_launch.cuh"

namespace vgb {

// Each thread runs 16 independent FMA chains (8 packed pairs, or 16 scalar),
// `iters` times, on values the compiler cannot fold (a, b from the host).
template <bool kPacked> __global__ void __launch_bounds__(256) fma_peak_kernel(float *out, int iters, float a, float b)
{
    const float seed = (float)(threadIdx.x + blockIdx.x) * 1e-7f;
    if (kPacked) {
        float2 acc[8];
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] = make_float2(seed + k, seed - k);
        const float2 A = make_float2(a, a), B = make_float2(b, b);
        for (int i = 0; i < iters; i++)
#pragma unroll
            for (int k = 0; k < 8; k++) acc[k] = __ffma2_rn(acc[k], A, B);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) s += acc[k].x + acc[k].y;
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    } else {
        float acc[16];
#pragma unroll
        for (int k = 0; k < 16; k++) acc[k] = seed + k;
        for (int i = 0; i < iters; i++)
#pragma unroll
            for (int k = 0; k < 16; k++) acc[k] = fmaf(acc[k], a, b);
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 16; k++) s += acc[k];
        out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

} // namespace vgb

using namespace vgb;

// FP32 throughput in TFLOP/s (2 flops per FMA) of `iters` x 16 FMAs per
// thread over 8 blocks of 256 threads per SM, timed with CUDA events on
// `stream` (best of three launches after one warm-up). packed != 0 issues
// them as FFMA2 (two FMAs per instruction), else as scalar FFMA.
extern "C" int vgb_fp32_peak(int packed, int iters, double *tflops, void *stream)
{
    if (!tflops || iters <= 0) return set_error(VGB_ERR_INVALID, "fp32_peak: bad argument");
    int dev = 0, sms = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (!rc) rc = check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
    if (rc) return rc;
    const int blocks = 8 * sms, threads = 256;
    float *out = nullptr;
    rc = check_cuda(cudaMalloc(reinterpret_cast<void **>(&out), sizeof(float) * blocks * threads), "cudaMalloc");
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    rc = check_cuda(cudaEventCreate(&e0), "event");
    if (!rc) rc = check_cuda(cudaEventCreate(&e1), "event");
    float best = 0.f;
    for (int r = 0; r < 4 && !rc; r++) {
        rc = check_cuda(cudaEventRecord(e0, st), "event");
        if (packed)
            fma_peak_kernel<true><<<blocks, threads, 0, st>>>(out, iters, 0.999999f, 1e-6f);
        else
            fma_peak_kernel<false><<<blocks, threads, 0, st>>>(out, iters, 0.999999f, 1e-6f);
        if (!rc) rc = check_launch("fma_peak_kernel");
        if (!rc) rc = check_cuda(cudaEventRecord(e1, st), "event");
        if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "event");
        float ms = 0.f;
        if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "event");
        if (!rc && r > 0 && (best == 0.f || ms < best)) best = ms;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (rc) return rc;
    const double flops = 2.0 * 16.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return VGB_SUCCESS;
}
