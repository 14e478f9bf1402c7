// halma_sequential_sum_f64: the left-to-right FP64 sum of every segment, rounded after each
// addition exactly as a scalar loop would, with the warp-wide integer-ulp adds of seqsum.cuh.
// It is the building block of the cleaning's per-cell sums (a numba loop in the reference,
// python_scripts/halo_properties.py:120-157) and lets the tests pin that building block against
// numpy's sequential accumulation on any values.
#include <string.h>

#include <vector>

#include "common.cuh"
#include "seqsum.cuh"

namespace halma {
namespace {

__global__ void seq_sum_kernel(int64_t nseg, const int64_t *__restrict__ off, const double *__restrict__ v,
                               double *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < nseg; s += warps) {
        const int64_t b = off[s], e = off[s + 1];
        SeqSum q;
        seq_init(q);
        for (int64_t k0 = b; k0 < e; k0 += 32) {
            const int64_t k = k0 + lane;
            const double a = k < e ? v[k] : 0.0;
            seq_add_warp(q, a, e - k0 < 32 ? (int)(e - k0) : 32, lane);
        }
        if (lane == 0) out[s] = seq_value(q);
    }
}

int seq_sum_device(int64_t nseg, const int64_t *off, const double *v, double *out, cudaStream_t st) {
    HALMA_LAUNCH(seq_sum_kernel, grid_for(nseg * 32, 256, device_sm_count() * 16), 256, 0, st, nseg, off, v, out);
    return HALMA_OK;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_sequential_sum_f64(int64_t n, const double *values, int64_t n_segments, const int64_t *offsets,
                                        double *out, halma_stream_t stream) {
    if (n < 0 || n_segments < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n_segments == 0) return HALMA_OK;
    if (!offsets || !out || (n > 0 && !values)) return fail(HALMA_ERR_INVALID, "null pointer");
    // the offsets must run from 0 to n without decreasing (checked on the host)
    std::vector<int64_t> hoff(n_segments + 1);
    if (is_device_pointer(offsets)) {
        HALMA_CUDA(cudaMemcpy(hoff.data(), offsets, 8ull * (n_segments + 1), cudaMemcpyDeviceToHost));
    } else {
        memcpy(hoff.data(), offsets, 8ull * (n_segments + 1));
    }
    if (hoff[0] != 0 || hoff[n_segments] != n) return fail(HALMA_ERR_INVALID, "segment offsets must run from 0 to n");
    for (int64_t s = 0; s < n_segments; ++s)
        if (hoff[s + 1] < hoff[s]) return fail(HALMA_ERR_INVALID, "segment offsets must not decrease");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dv = nullptr;
    const int64_t *doff = nullptr;
    double *dout = nullptr;
    sg.add(values, n, true, false, &dv);
    sg.add(offsets, n_segments + 1, true, false, &doff);
    sg.add((const double *)out, n_segments, false, true, &dout);
    void *stage = nullptr;
    if (sg.any_host) {
        Layout L;
        sg.plan(L);
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
    }
    int s = sg.bind_and_upload(stage, st);
    if (s == HALMA_OK) s = seq_sum_device(n_segments, doff, dv, dout, st);
    if (s == HALMA_OK) s = sg.download(st);
    if (stage) {
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
    }
    return s;
}
