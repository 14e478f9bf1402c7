// Radix sorts and scans (CUB device primitives) used by FoF, groups and reductions.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cuda/functional>

#include "sort.cuh"

namespace halma {

size_t sort_pairs_u64_i32_bytes(int n, int end_bit) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                    (const int32_t *)nullptr, (int32_t *)nullptr, n, 0, end_bit);
    return b;
}

int sort_pairs_u64_i32(void *tmp, size_t tmp_bytes, const uint64_t *kin, uint64_t *kout,
                       const int32_t *vin, int32_t *vout, int n, int end_bit, cudaStream_t s) {
    HALMA_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kin, kout, vin, vout, n, 0, end_bit, s));
    return HALMA_OK;
}

size_t sort_pairs_u32_i32_bytes(int n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t *)nullptr, (uint32_t *)nullptr,
                                    (const int32_t *)nullptr, (int32_t *)nullptr, n, 0, 32);
    return b;
}

int sort_pairs_u32_i32(void *tmp, size_t tmp_bytes, const uint32_t *kin, uint32_t *kout,
                       const int32_t *vin, int32_t *vout, int n, int end_bit, cudaStream_t s) {
    HALMA_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kin, kout, vin, vout, n, 0, end_bit, s));
    return HALMA_OK;
}

size_t sort_keys_u64_bytes(int n, int end_bit) {
    size_t b = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, b, (const uint64_t *)nullptr, (uint64_t *)nullptr, n, 0, end_bit);
    return b;
}

int sort_keys_u64(void *tmp, size_t tmp_bytes, const uint64_t *kin, uint64_t *kout, int n, int end_bit,
                  cudaStream_t s) {
    HALMA_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes, kin, kout, n, 0, end_bit, s));
    return HALMA_OK;
}

size_t exclusive_sum_i64_bytes(int n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (const int64_t *)nullptr, (int64_t *)nullptr, n);
    return b;
}

int exclusive_sum_i64(void *tmp, size_t tmp_bytes, const int64_t *in, int64_t *out, int n, cudaStream_t s) {
    HALMA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, n, s));
    return HALMA_OK;
}

size_t inclusive_max_i32_bytes(int n) {
    size_t b = 0;
    cub::DeviceScan::InclusiveScan(nullptr, b, (const int32_t *)nullptr, (int32_t *)nullptr, cuda::maximum<>{}, n);
    return b;
}

int inclusive_max_i32(void *tmp, size_t tmp_bytes, const int32_t *in, int32_t *out, int n, cudaStream_t s) {
    HALMA_CUDA(cub::DeviceScan::InclusiveScan(tmp, tmp_bytes, in, out, cuda::maximum<>{}, n, s));
    return HALMA_OK;
}

namespace {
struct Int3Sum {
    __device__ __forceinline__ int4 operator()(const int4 &a, const int4 &b) const {
        return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, 0);
    }
};
}  // namespace

size_t exclusive_sum_int3_bytes(int n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveScan(nullptr, b, (const int4 *)nullptr, (int4 *)nullptr, Int3Sum{},
                                   make_int4(0, 0, 0, 0), n);
    return b;
}

int exclusive_sum_int3(void *tmp, size_t tmp_bytes, const int4 *in, int4 *out, int n, cudaStream_t s) {
    HALMA_CUDA(cub::DeviceScan::ExclusiveScan(tmp, tmp_bytes, in, out, Int3Sum{}, make_int4(0, 0, 0, 0), n, s));
    return HALMA_OK;
}

size_t exclusive_sum_i32_bytes(int n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (const int32_t *)nullptr, (int32_t *)nullptr, n);
    return b;
}

int exclusive_sum_i32(void *tmp, size_t tmp_bytes, const int32_t *in, int32_t *out, int n,
                      cudaStream_t s) {
    HALMA_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, in, out, n, s));
    return HALMA_OK;
}

}  // namespace halma
