// Adjoint of the softened potential  phi_i = sum_j m_j (|s_j - t_i|^2 + eps2)^-1/2.
//
// For an upstream gradient g_i = dL/dphi_i the derivatives are two all-pairs sums of the same
// shape, so one kernel serves both:
//   over targets a = t_i, partners b = s_j, weights w_b = m_j:
//       V_a = sum_b w_b (p_b - p_a) r^-3            -> dL/dt_i = g_i * V_a
//   over sources a = s_j, partners b = t_i, weights w_b = g_i:
//       S_a = sum_b w_b r^-1,  V_a = sum_b w_b (p_b - p_a) r^-3
//                                                   -> dL/dm_j = S_a, dL/ds_j = m_j * V_a
// with r^2 = |p_b - p_a|^2 + eps2.  FP32 pair terms (rsqrt) as f32x2 instructions (two partners
// per instruction), per-chunk FP32 partials folded into TwoSum-compensated accumulators.  The
// self pair (b == a + self_offset) is skipped when the mask asks for it.
#include <math.h>
#include <string.h>

#include "common.cuh"
#include "pair_math.cuh"

namespace halma {
namespace {

constexpr int kGWarps = 8;
constexpr float kFarG = 3.0e30f;

__device__ __forceinline__ float4 load_b(const float *__restrict__ x, const float *__restrict__ y,
                                         const float *__restrict__ z, const float *__restrict__ w, int64_t j,
                                         int64_t n) {
    if (j < n) return make_float4(x[j], y[j], z[j], w[j]);
    return make_float4(kFarG, kFarG, kFarG, 0.f);
}

// 32 partners of the staged chunk against the lane's T particles, two partners per f32x2
// instruction: sa[kp] = {x_2kp, x_2kp+1, y_2kp, y_2kp+1}, sb[kp] = {z.., z.., w.., w..}.  Per
// pair: r^-1 and w r^-3 (p_b - p_a); the chunk's partials are {even, odd} pairs.  SELF: the
// pair whose partner index (j0 + slot) equals self[t] is skipped.
template <int T, bool WANT_S, bool SELF>
__device__ __forceinline__ void adjoint_chunk(const float4 *sa, const float4 *sb, const f2x (&px)[T],
                                              const f2x (&py)[T], const f2x (&pz)[T], f2x e2, int64_t j0,
                                              const int64_t (&self)[T], f2x (&ps)[T], f2x (&pvx)[T],
                                              f2x (&pvy)[T], f2x (&pvz)[T]) {
#pragma unroll 4
    for (int kp = 0; kp < 16; ++kp) {
        const float4 qa = sa[kp], qb = sb[kp];
        const f2x X = pack2(qa.x, qa.y), Y = pack2(qa.z, qa.w), Z = pack2(qb.x, qb.y), W = pack2(qb.z, qb.w);
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const f2x dx = sub2(X, px[t]), dy = sub2(Y, py[t]), dz = sub2(Z, pz[t]);
            f2x r2 = fma2(dz, dz, e2);
            r2 = fma2(dy, dy, r2);
            r2 = fma2(dx, dx, r2);
            float r0, r1;
            unpack2(r2, r0, r1);
            float i0 = rsqrt_ftz(r0), i1 = rsqrt_ftz(r1);
            if (SELF) {
                if (j0 + 2 * kp == self[t]) i0 = 0.f;
                if (j0 + 2 * kp + 1 == self[t]) i1 = 0.f;
            }
            const f2x ri = pack2(i0, i1);
            const f2x wr = mul2(W, ri);
            const f2x wr3 = mul2(mul2(wr, ri), ri);
            if (WANT_S) ps[t] = add2(ps[t], wr);
            pvx[t] = fma2(wr3, dx, pvx[t]);
            pvy[t] = fma2(wr3, dy, pvy[t]);
            pvz[t] = fma2(wr3, dz, pvz[t]);
        }
    }
}

__device__ __forceinline__ void fold2(float &s, float &c, f2x v) {
    float lo, hi;
    unpack2(v, lo, hi);
    two_sum_acc(s, c, lo + hi);
}

// One warp per tile of 32*T particles a against all partners b, streamed in chunks of 32
// through a per-warp shared buffer; chunk partials folded into TwoSum-compensated sums.
template <int T, bool WANT_S>
__global__ void __launch_bounds__(256, 3) adjoint_kernel(
    const float *__restrict__ bx, const float *__restrict__ by, const float *__restrict__ bz,
    const float *__restrict__ bw, int64_t nb, const float *__restrict__ ax, const float *__restrict__ ay,
    const float *__restrict__ az, int64_t na, float eps2, int self_mask, int64_t self_off,
    const float *__restrict__ vscale, float *__restrict__ out_s, float *__restrict__ out_v) {
    __shared__ float4 buf[kGWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float *sa = reinterpret_cast<float *>(buf[w]);        // 16 float4: x/y pairs
    float *sb = reinterpret_cast<float *>(buf[w] + 16);   // 16 float4: z/w pairs
    const int kp = lane >> 1, hf = lane & 1;
    const f2x e2 = pack2(eps2, eps2);
    const int64_t ntiles = (na + 32 * T - 1) / (32 * T);
    for (int64_t tile = (int64_t)blockIdx.x * kGWarps + w; tile < ntiles; tile += (int64_t)gridDim.x * kGWarps) {
        f2x px[T], py[T], pz[T];
        float ss[T], sc[T], vxs[T], vxc[T], vys[T], vyc[T], vzs[T], vzc[T];
        int64_t self[T];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int64_t a = tile * 32 * T + t * 32 + lane;
            const bool v = a < na;
            const float x = v ? ax[a] : kFarG, y = v ? ay[a] : kFarG, z = v ? az[a] : kFarG;
            px[t] = pack2(x, x);
            py[t] = pack2(y, y);
            pz[t] = pack2(z, z);
            self[t] = (v && self_mask) ? a + self_off : -1;
            ss[t] = sc[t] = vxs[t] = vxc[t] = vys[t] = vyc[t] = vzs[t] = vzc[t] = 0.f;
        }
        // partner indices self[t] lie in [lo_self, lo_self + 32 * T) for this tile
        const int64_t lo_self = tile * 32 * T + self_off;
        float4 nxt = load_b(bx, by, bz, bw, lane, nb);
        for (int64_t j0 = 0; j0 < nb; j0 += 32) {
            __syncwarp();
            sa[kp * 4 + hf] = nxt.x;
            sa[kp * 4 + 2 + hf] = nxt.y;
            sb[kp * 4 + hf] = nxt.z;
            sb[kp * 4 + 2 + hf] = nxt.w;
            __syncwarp();
            nxt = load_b(bx, by, bz, bw, j0 + 32 + lane, nb);
            f2x ps[T], pvx[T], pvy[T], pvz[T];
#pragma unroll
            for (int t = 0; t < T; ++t) ps[t] = pvx[t] = pvy[t] = pvz[t] = pack2(0.f, 0.f);
            const bool self_chunk = self_mask && j0 + 32 > lo_self && j0 < lo_self + 32 * T;
            if (self_chunk)
                adjoint_chunk<T, WANT_S, true>(buf[w], buf[w] + 16, px, py, pz, e2, j0, self, ps, pvx, pvy, pvz);
            else
                adjoint_chunk<T, WANT_S, false>(buf[w], buf[w] + 16, px, py, pz, e2, j0, self, ps, pvx, pvy, pvz);
#pragma unroll
            for (int t = 0; t < T; ++t) {
                if (WANT_S) fold2(ss[t], sc[t], ps[t]);
                fold2(vxs[t], vxc[t], pvx[t]);
                fold2(vys[t], vyc[t], pvy[t]);
                fold2(vzs[t], vzc[t], pvz[t]);
            }
        }
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int64_t a = tile * 32 * T + t * 32 + lane;
            if (a >= na) continue;
            if (WANT_S && out_s) out_s[a] = ss[t] + sc[t];
            if (out_v) {
                const float sc_ = vscale[a];
                out_v[3 * a + 0] = sc_ * (vxs[t] + vxc[t]);
                out_v[3 * a + 1] = sc_ * (vys[t] + vyc[t]);
                out_v[3 * a + 2] = sc_ * (vzs[t] + vzc[t]);
            }
        }
    }
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_potential_grad_f32(int64_t ns, const float *m_, const float *sx_, const float *sy_,
                                        const float *sz_, int64_t nt, const float *tx_, const float *ty_,
                                        const float *tz_, const float *g_, double eps2, int32_t mask,
                                        int64_t self_offset, float *grad_m, float *grad_src, float *grad_tgt,
                                        halma_stream_t stream) {
    if (ns < 0 || nt < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (mask != HALMA_MASK_SELF && mask != HALMA_MASK_NONE)
        return fail(HALMA_ERR_INVALID, "gradient supports the SELF and NONE masks only");
    if (!(eps2 >= 0.0) || !isfinite(eps2)) return fail(HALMA_ERR_INVALID, "eps2 must be finite and >= 0");
    if ((ns > 0 && (!m_ || !sx_ || !sy_ || !sz_)) || (nt > 0 && (!tx_ || !ty_ || !tz_ || !g_)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    if (ns == 0 || nt == 0) {
        // empty sums: every requested gradient is zero
        std::lock_guard<std::mutex> guard(api_mutex());
        cudaStream_t st = (cudaStream_t)stream;
        float *outs[3] = {grad_m, grad_src, grad_tgt};
        const int64_t cnt[3] = {ns, 3 * ns, 3 * nt};
        for (int q = 0; q < 3; ++q) {
            if (!outs[q] || cnt[q] == 0) continue;
            if (is_device_pointer(outs[q])) HALMA_CUDA(cudaMemsetAsync(outs[q], 0, 4 * cnt[q], st));
            else memset(outs[q], 0, 4 * cnt[q]);
        }
        return HALMA_OK;
    }
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const float *m = nullptr, *sx = nullptr, *sy = nullptr, *sz = nullptr, *tx = nullptr, *ty = nullptr,
                *tz = nullptr, *g = nullptr;
    float *gm = nullptr, *gs = nullptr, *gt = nullptr;
    sg.add(m_, ns, true, false, &m);
    sg.add(sx_, ns, true, false, &sx);
    sg.add(sy_, ns, true, false, &sy);
    sg.add(sz_, ns, true, false, &sz);
    sg.add(tx_, nt, true, false, &tx);
    sg.add(ty_, nt, true, false, &ty);
    sg.add(tz_, nt, true, false, &tz);
    sg.add(g_, nt, true, false, &g);
    sg.add((const float *)grad_m, grad_m ? ns : 0, false, true, &gm);
    sg.add((const float *)grad_src, grad_src ? 3 * ns : 0, false, true, &gs);
    sg.add((const float *)grad_tgt, grad_tgt ? 3 * nt : 0, false, true, &gt);
    Layout L;
    sg.plan(L);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    HALMA_TRY(sg.bind_and_upload(base, st));
    const int self = mask == HALMA_MASK_SELF;
    constexpr int T = 2;
    const int cap = device_sm_count() * 8;
    if (gt) {
        const int64_t tiles = (nt + 32 * T - 1) / (32 * T);
        const int grid = (int)std::min<int64_t>((tiles + kGWarps - 1) / kGWarps, cap);
        HALMA_LAUNCH((adjoint_kernel<T, false>), grid, 256, 0, st, sx, sy, sz, m, ns, tx, ty, tz, nt, (float)eps2,
                     self, self_offset, g, (float *)nullptr, gt);
    }
    if (gm || gs) {
        const int64_t tiles = (ns + 32 * T - 1) / (32 * T);
        const int grid = (int)std::min<int64_t>((tiles + kGWarps - 1) / kGWarps, cap);
        HALMA_LAUNCH((adjoint_kernel<T, true>), grid, 256, 0, st, tx, ty, tz, g, nt, sx, sy, sz, ns, (float)eps2,
                     self, -self_offset, m, gm, gs);
    }
    return sg.download(st);
}
