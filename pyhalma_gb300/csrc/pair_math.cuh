// Per-pair arithmetic shared by the potential, unbinding and gradient kernels.
#pragma once
#include <cuda_runtime.h>

namespace halma {

// ---- packed FP32 pairs (sm_100+ f32x2 instructions: two FP32 lanes per instruction) -------
typedef unsigned long long f2x;   // {lo, hi} float pair in one 64-bit register

__device__ __forceinline__ f2x pack2(float lo, float hi) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(f2x r, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r));
}
__device__ __forceinline__ f2x sub2(f2x a, f2x b) {
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x add2(f2x a, f2x b) {
    f2x d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x mul2(f2x a, f2x b) {
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c) {
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Hardware reciprocal square root, subnormal inputs and outputs flushed to zero (the
// softened r^2 >= eps^2 is never subnormal); one special-function instruction.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Error-free transformation of s + v (Knuth's TwoSum); the rounding error goes into c.
// Six additions, no fused operations, valid for any magnitudes.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float v) {
    float t = s + v;
    float bp = t - s;
    float err = (s - (t - bp)) + (v - bp);
    s = t;
    c += err;
}

// Double-float numbers: a value held as the unevaluated sum hi + lo of two FP32 numbers
// (float2 {hi, lo}), about 48 significant bits, computed with FP32 operations only -- on a GPU
// whose FP64 rate is a small fraction of its FP32 rate, this carries FP64-like accuracy
// through per-particle code.  Error-free transformations of Knuth (TwoSum) and Dekker
// (FastTwoSum, |a| >= |b|); neither contains a product, so FMA contraction cannot alter them.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = a + b;
    const float bp = s - a;
    return make_float2(s, (a - (s - bp)) + (b - bp));
}

__device__ __forceinline__ float2 df_fast_two_sum(float a, float b) {
    const float s = a + b;
    return make_float2(s, b - (s - a));
}

// The accurate double-float sum (both parts added with TwoSum, renormalised twice), valid
// under cancellation, as in an incremental update phi - delta with delta close to phi.
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float2 s = df_two_sum(a.x, b.x);
    const float2 t = df_two_sum(a.y, b.y);
    s = df_fast_two_sum(s.x, s.y + t.x);
    return df_fast_two_sum(s.x, s.y + t.y);
}

__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, make_float2(-b.x, -b.y)); }

// A compensated FP32 accumulator (sum s, accumulated rounding errors c, |c| << |s|) as a
// normalised double-float.
__device__ __forceinline__ float2 df_from_acc(float s, float c) { return df_fast_two_sum(s, c); }

__device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// One softened pair term m / sqrt(r^2 + eps2) with the FP32 special-function rsqrt.
__device__ __forceinline__ float pair_term_fast(float4 q, float px, float py, float pz, float eps2,
                                                float acc) {
    float dx = q.x - px;
    float dy = q.y - py;
    float dz = q.z - pz;
    float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    return fmaf(q.w, rsqrtf(r2), acc);
}

// Same, with the reference's pair mask: the term counts only when the source's x, y and z
// all differ from the target's (particle_subroutines.f90:499-501).
__device__ __forceinline__ float pair_term_fast_masked(float4 q, float px, float py, float pz,
                                                       float eps2, float acc) {
    float dx = q.x - px;
    float dy = q.y - py;
    float dz = q.z - pz;
    float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    float ri = rsqrtf(r2);
    bool keep = (q.x != px) & (q.y != py) & (q.z != pz);
    return fmaf(q.w, keep ? ri : 0.0f, acc);
}

// The reference's float32 statement, each operation rounded on its own (no FMA):
//   r = sqrt((xj-xi)**2 + (yj-yi)**2 + (zj-zi)**2); phi = phi + m / r
// (particle_subroutines.f90:502-505), guarded by the mask of f90:499-501.
__device__ __forceinline__ float pair_term_reference(float4 q, float px, float py, float pz,
                                                     float acc) {
    if (q.x != px && q.y != py && q.z != pz) {
        float dx = __fsub_rn(q.x, px);
        float dy = __fsub_rn(q.y, py);
        float dz = __fsub_rn(q.z, pz);
        float s = __fmul_rn(dx, dx);
        s = __fadd_rn(s, __fmul_rn(dy, dy));
        s = __fadd_rn(s, __fmul_rn(dz, dz));
        float r = __fsqrt_rn(s);
        acc = __fadd_rn(acc, __fdiv_rn(q.w, r));
    }
    return acc;
}

}  // namespace halma
