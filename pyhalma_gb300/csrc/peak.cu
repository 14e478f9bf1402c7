// FP32 FMA rate of this GPU, measured with a kernel of independent FMA chains: the roofline
// denominator of the pair kernels (a CUDA-core workload whose peak is not the tensor-core or
// copy figure).  Scalar fma.rn.f32 or packed fma.rn.f32x2 (two lanes per instruction, the
// form the pair kernels use); an FMA counts as two flops.
#include "common.cuh"
#include "pair_math.cuh"

namespace halma {
namespace {

constexpr int kPeakThreads = 256;
constexpr int kChains = 8;

template <bool Packed>
__global__ void __launch_bounds__(kPeakThreads) fma_rate_kernel(int iters, float a, float b, float *sink) {
    const float s0 = 1e-3f * (float)(threadIdx.x & 63);
    if (Packed) {
        f2x v[kChains];
#pragma unroll
        for (int k = 0; k < kChains; ++k) v[k] = pack2(s0 + (float)k, s0 - (float)k);
        const f2x A = pack2(a, a), B = pack2(b, b);
        for (int i = 0; i < iters; ++i)
#pragma unroll
            for (int k = 0; k < kChains; ++k) v[k] = fma2(v[k], A, B);
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            float lo, hi;
            unpack2(v[k], lo, hi);
            acc += lo + hi;
        }
        if (acc == -1.0f) sink[0] = acc;   // keeps the chains alive; never true for these inputs
    } else {
        float v[2 * kChains];
#pragma unroll
        for (int k = 0; k < 2 * kChains; ++k) v[k] = s0 + (float)k;
        for (int i = 0; i < iters; ++i)
#pragma unroll
            for (int k = 0; k < 2 * kChains; ++k) v[k] = fmaf(v[k], a, b);
        float acc = 0.f;
#pragma unroll
        for (int k = 0; k < 2 * kChains; ++k) acc += v[k];
        if (acc == -1.0f) sink[0] = acc;
    }
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_measure_fp32_fma_rate(int32_t packed, int32_t iters, double *tflops, double *ms,
                                           halma_stream_t stream) {
    if (iters < 1 || !tflops) return fail(HALMA_ERR_INVALID, "iters must be >= 1 and tflops non-NULL");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    void *base = nullptr;
    HALMA_TRY(workspace(256, &base, st));
    float *sink = at<float>(base, 0);
    int bps = 0;
    if (packed)
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fma_rate_kernel<true>, kPeakThreads, 0));
    else
        HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fma_rate_kernel<false>, kPeakThreads, 0));
    const int grid = device_sm_count() * std::max(bps, 1);
    cudaEvent_t e0, e1;
    HALMA_CUDA(cudaEventCreate(&e0));
    HALMA_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {   // the first launch warms the clocks up; the fastest counts
        HALMA_CUDA(cudaEventRecord(e0, st));
        if (packed) HALMA_LAUNCH(fma_rate_kernel<true>, grid, kPeakThreads, 0, st, iters, 0.999f, 1e-3f, sink);
        else HALMA_LAUNCH(fma_rate_kernel<false>, grid, kPeakThreads, 0, st, iters, 0.999f, 1e-3f, sink);
        HALMA_CUDA(cudaEventRecord(e1, st));
        HALMA_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        HALMA_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep > 0) best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double fmas = (double)grid * kPeakThreads * iters * (2.0 * kChains);
    *tflops = 2.0 * fmas / (best * 1e-3) / 1e12;
    if (ms) *ms = best;
    return HALMA_OK;
}
