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

// The pair kernels' arithmetic alone, at the occupancy its registers allow: per pair of
// particles 3 sub + 3 fma (r^2 + eps^2) + 2 fma (one term for each particle) as f32x2
// instructions, two pairs per instruction, and one rsqrt per pair on the special-function
// unit -- the FP32 pipe and the special-function unit are both loaded to exactly their
// throughput (8 lane-operations at 128 per SM-cycle, one rsqrt at 16 per SM-cycle), so neither
// peak alone is reachable by this mix.  Sources come from shared memory as in the block
// kernel, 8 targets per lane; no reductions, no bookkeeping.  The measured rate is the ceiling
// the symmetric block kernel is compared against.
constexpr int kMixT = 8;

__device__ __forceinline__ f2x vsub2(f2x a, f2x b) {
    f2x d;
    asm volatile("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x vfma2(f2x a, f2x b, f2x c) {
    f2x d;
    asm volatile("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ float vrsqrt(float x) {
    float y;
    asm volatile("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__global__ void __launch_bounds__(kPeakThreads) pair_mix_kernel(int iters, float eps2, float *sink) {
    __shared__ float4 src[32];   // 16 source pairs: {x, x', y, y'}, {z, z', m, m'}
    if (threadIdx.x < 32) {
        const float u = 0.01f * (float)threadIdx.x;
        src[threadIdx.x] = (threadIdx.x & 1) ? make_float4(0.25f - u, u, 1.f, 1.f) : make_float4(u, -u, 0.5f * u, 1.f - u);
    }
    __syncthreads();
    const float s0 = 1e-3f * (float)(threadIdx.x & 63);
    f2x tx[kMixT], ty[kMixT], tz[kMixT], tm[kMixT], acc[kMixT], sacc[8];
#pragma unroll
    for (int t = 0; t < kMixT; ++t) {
        tx[t] = pack2(s0 + 0.1f * t, s0 + 0.1f * t);
        ty[t] = pack2(s0 - 0.1f * t, s0 - 0.1f * t);
        tz[t] = pack2(0.3f * t, 0.3f * t);
        tm[t] = pack2(1.f, 1.f);
        acc[t] = pack2(0.f, 0.f);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) sacc[k] = pack2(0.f, 0.f);
    const f2x e2 = pack2(eps2, eps2);
    for (int i = 0; i < iters; ++i) {
        const int half = i & 1;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float4 a = src[half * 16 + 2 * k], b = src[half * 16 + 2 * k + 1];
            const f2x X = pack2(a.x, a.y), Y = pack2(a.z, a.w), Z = pack2(b.x, b.y), M = pack2(b.z, b.w);
#pragma unroll
            for (int t = 0; t < kMixT; ++t) {
                const f2x dx = vsub2(X, tx[t]), dy = vsub2(Y, ty[t]), dz = vsub2(Z, tz[t]);
                f2x r2 = vfma2(dz, dz, e2);
                r2 = vfma2(dy, dy, r2);
                r2 = vfma2(dx, dx, r2);
                float r0, r1;
                unpack2(r2, r0, r1);
                const f2x ri = pack2(vrsqrt(r0), vrsqrt(r1));
                acc[t] = vfma2(M, ri, acc[t]);
                sacc[k] = vfma2(tm[t], ri, sacc[k]);
            }
        }
    }
    float v = 0.f;
#pragma unroll
    for (int t = 0; t < kMixT; ++t) {
        float lo, hi;
        unpack2(acc[t], lo, hi);
        v += lo + hi;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float lo, hi;
        unpack2(sacc[k], lo, hi);
        v += lo + hi;
    }
    if (v == -1.0f) sink[0] = v;   // keeps the sums alive; never true for these inputs
}

// The tile kernel's arithmetic alone (incremental passes and small haloes): per pair term
// 3 sub + 3 fma + 1 fma as f32x2 and one rsqrt, 4 targets per lane, sources from shared
// memory, the target sums only.  7 lane-operations a term keep the FP32 pipe just under the
// special-function unit's one rsqrt a term.
constexpr int kTermT = 4;

__global__ void __launch_bounds__(kPeakThreads) term_mix_kernel(int iters, float eps2, float *sink) {
    __shared__ float4 src[32];
    if (threadIdx.x < 32) {
        const float u = 0.01f * (float)threadIdx.x;
        src[threadIdx.x] = (threadIdx.x & 1) ? make_float4(0.25f - u, u, 1.f, 1.f) : make_float4(u, -u, 0.5f * u, 1.f - u);
    }
    __syncthreads();
    const float s0 = 1e-3f * (float)(threadIdx.x & 63);
    f2x tx[kTermT], ty[kTermT], tz[kTermT], acc[kTermT];
#pragma unroll
    for (int t = 0; t < kTermT; ++t) {
        tx[t] = pack2(s0 + 0.1f * t, s0 + 0.1f * t);
        ty[t] = pack2(s0 - 0.1f * t, s0 - 0.1f * t);
        tz[t] = pack2(0.3f * t, 0.3f * t);
        acc[t] = pack2(0.f, 0.f);
    }
    const f2x e2 = pack2(eps2, eps2);
    for (int i = 0; i < iters; ++i) {
        const int half = i & 1;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const float4 a = src[half * 16 + 2 * k], b = src[half * 16 + 2 * k + 1];
            const f2x X = pack2(a.x, a.y), Y = pack2(a.z, a.w), Z = pack2(b.x, b.y), M = pack2(b.z, b.w);
#pragma unroll
            for (int t = 0; t < kTermT; ++t) {
                const f2x dx = vsub2(X, tx[t]), dy = vsub2(Y, ty[t]), dz = vsub2(Z, tz[t]);
                f2x r2 = vfma2(dz, dz, e2);
                r2 = vfma2(dy, dy, r2);
                r2 = vfma2(dx, dx, r2);
                float r0, r1;
                unpack2(r2, r0, r1);
                acc[t] = vfma2(M, pack2(vrsqrt(r0), vrsqrt(r1)), acc[t]);
            }
        }
    }
    float v = 0.f;
#pragma unroll
    for (int t = 0; t < kTermT; ++t) {
        float lo, hi;
        unpack2(acc[t], lo, hi);
        v += lo + hi;
    }
    if (v == -1.0f) sink[0] = v;   // keeps the sums alive; never true for these inputs
}

// Fastest of three timed launches (after one warm-up) of a peak kernel on its full-occupancy grid.
template <class K>
int time_peak_kernel(K kernel, int iters, cudaStream_t st, float *best_ms, int *grid_out) {
    void *base = nullptr;
    HALMA_TRY(workspace(256, &base, st));
    float *sink = at<float>(base, 0);
    int bps = 0;
    HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, kPeakThreads, 0));
    const int grid = device_sm_count() * std::max(bps, 1);
    cudaEvent_t e0, e1;
    HALMA_CUDA(cudaEventCreate(&e0));
    HALMA_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        HALMA_CUDA(cudaEventRecord(e0, st));
        HALMA_LAUNCH(kernel, grid, kPeakThreads, 0, st, iters, 1e-8f, sink);
        HALMA_CUDA(cudaEventRecord(e1, st));
        HALMA_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        HALMA_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep > 0) best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *best_ms = best;
    *grid_out = grid;
    return HALMA_OK;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_measure_term_rate(int32_t iters, double *terms_per_s, double *ms, halma_stream_t stream) {
    if (iters < 1 || !terms_per_s) return fail(HALMA_ERR_INVALID, "iters must be >= 1 and terms_per_s non-NULL");
    std::lock_guard<std::mutex> guard(api_mutex());
    float best = 0.f;
    int grid = 0;
    HALMA_TRY(time_peak_kernel(term_mix_kernel, iters, (cudaStream_t)stream, &best, &grid));
    // per iteration and thread: 8 source pairs x kTermT targets x 2 terms
    const double terms = (double)grid * kPeakThreads * iters * 8.0 * kTermT * 2.0;
    *terms_per_s = terms / (best * 1e-3);
    if (ms) *ms = best;
    return HALMA_OK;
}

extern "C" int halma_measure_pair_rate(int32_t iters, double *pairs_per_s, double *ms, halma_stream_t stream) {
    if (iters < 1 || !pairs_per_s) return fail(HALMA_ERR_INVALID, "iters must be >= 1 and pairs_per_s non-NULL");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    void *base = nullptr;
    HALMA_TRY(workspace(256, &base, st));
    float *sink = at<float>(base, 0);
    int bps = 0;
    HALMA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pair_mix_kernel, kPeakThreads, 0));
    const int grid = device_sm_count() * std::max(bps, 1);
    cudaEvent_t e0, e1;
    HALMA_CUDA(cudaEventCreate(&e0));
    HALMA_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {   // the first launch warms the clocks up; the fastest counts
        HALMA_CUDA(cudaEventRecord(e0, st));
        HALMA_LAUNCH(pair_mix_kernel, grid, kPeakThreads, 0, st, iters, 1e-8f, sink);
        HALMA_CUDA(cudaEventRecord(e1, st));
        HALMA_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        HALMA_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep > 0) best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // per iteration and thread: 8 source pairs x kMixT targets x 2 (two sources per f32x2)
    const double pairs = (double)grid * kPeakThreads * iters * 8.0 * kMixT * 2.0;
    *pairs_per_s = pairs / (best * 1e-3);
    if (ms) *ms = best;
    return HALMA_OK;
}

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
