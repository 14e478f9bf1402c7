// Radix sort / scan wrappers (implemented with CUB in sort.cu so that only one translation
// unit pays the template compile time).
#pragma once
#include "common.cuh"

namespace halma {

size_t sort_pairs_u64_i32_bytes(int n, int end_bit);
int sort_pairs_u64_i32(void *tmp, size_t tmp_bytes, const uint64_t *kin, uint64_t *kout,
                       const int32_t *vin, int32_t *vout, int n, int end_bit, cudaStream_t s);
size_t sort_pairs_u32_i32_bytes(int n);
int sort_pairs_u32_i32(void *tmp, size_t tmp_bytes, const uint32_t *kin, uint32_t *kout,
                       const int32_t *vin, int32_t *vout, int n, int end_bit, cudaStream_t s);
size_t sort_keys_u64_bytes(int n, int end_bit);
int sort_keys_u64(void *tmp, size_t tmp_bytes, const uint64_t *kin, uint64_t *kout, int n, int end_bit,
                  cudaStream_t s);
size_t exclusive_sum_i64_bytes(int n);
int exclusive_sum_i64(void *tmp, size_t tmp_bytes, const int64_t *in, int64_t *out, int n, cudaStream_t s);
size_t inclusive_max_i32_bytes(int n);
int inclusive_max_i32(void *tmp, size_t tmp_bytes, const int32_t *in, int32_t *out, int n, cudaStream_t s);
// Exclusive prefix sums of the x, y and z fields of int4 values at once (w is ignored, set to 0).
size_t exclusive_sum_int3_bytes(int n);
int exclusive_sum_int3(void *tmp, size_t tmp_bytes, const int4 *in, int4 *out, int n, cudaStream_t s);
size_t exclusive_sum_i32_bytes(int n);
int exclusive_sum_i32(void *tmp, size_t tmp_bytes, const int32_t *in, int32_t *out, int n,
                      cudaStream_t s);

}  // namespace halma
