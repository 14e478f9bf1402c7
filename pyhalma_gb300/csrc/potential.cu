// Brute-force potential kernels and the C ABI that replaces the f2py symbol
// particle.particle.brute_force_binding_energy (particle_subroutines.f90:466-514).
//
// Layout: sources are read as float32 SoA (m, x, y, z) and staged per warp in shared memory
// as float4 chunks of 32; each lane owns T targets, so one shared-memory broadcast feeds T
// pair terms.  Work items are (target tile of 32*T, source slice); warps stride over items.
#include <math.h>

#include "common.cuh"
#include "pair_math.cuh"
#include "unbind.cuh"

namespace halma {

constexpr int kWarpsPerBlock = 8;
constexpr float kPadCoord = 3.0e30f;   // pad sources: m = 0 at a far point -> exact +0 term

__device__ __forceinline__ float4 load_source(const float *__restrict__ m, const float *__restrict__ x,
                                              const float *__restrict__ y, const float *__restrict__ z,
                                              int64_t j, int64_t end) {
    if (j < end) return make_float4(__ldg(x + j), __ldg(y + j), __ldg(z + j), __ldg(m + j));
    return make_float4(kPadCoord, kPadCoord, kPadCoord, 0.0f);
}

// HALMA_POT_REFERENCE: one target per lane, sources in order, bit-identical to the
// Fortran loop body (f90:497-510).
__global__ void __launch_bounds__(256) bf_potential_reference_kernel(
    const float *__restrict__ m, const float *__restrict__ x, const float *__restrict__ y,
    const float *__restrict__ z, int64_t ns, const float *__restrict__ tx,
    const float *__restrict__ ty, const float *__restrict__ tz, int64_t nt, float *__restrict__ out) {
    __shared__ float4 buf[kWarpsPerBlock][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t gwarp = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t nwarps = (int64_t)gridDim.x * kWarpsPerBlock;
    const int64_t ntiles = (nt + 31) / 32;
    for (int64_t tile = gwarp; tile < ntiles; tile += nwarps) {
        const int64_t i = tile * 32 + lane;
        const bool valid = i < nt;
        const float px = valid ? tx[i] : 0.f, py = valid ? ty[i] : 0.f, pz = valid ? tz[i] : 0.f;
        float acc = 0.0f;
        float4 nxt = load_source(m, x, y, z, lane, ns);
        for (int64_t j0 = 0; j0 < ns; j0 += 32) {
            __syncwarp();
            buf[w][lane] = nxt;
            __syncwarp();
            nxt = load_source(m, x, y, z, j0 + 32 + lane, ns);
            const int cnt = (int)min((int64_t)32, ns - j0);
            for (int k = 0; k < cnt; ++k) acc = pair_term_reference(buf[w][k], px, py, pz, acc);
        }
        if (valid) out[i] = acc;
    }
}

// HALMA_POT_FAST: T targets per lane, FP32 rsqrt pair terms with the reference mask, each
// 32-source chunk summed in FP32 and folded into a TwoSum-compensated accumulator.
// MASK: HALMA_MASK_COORD (reference mask), HALMA_MASK_SELF (skip j == i + self_offset) or
// HALMA_MASK_NONE.
template <int T, int MASK>
__global__ void __launch_bounds__(256) bf_potential_fast_kernel(
    const float *__restrict__ m, const float *__restrict__ x, const float *__restrict__ y,
    const float *__restrict__ z, int64_t ns, const float *__restrict__ tx,
    const float *__restrict__ ty, const float *__restrict__ tz, int64_t nt, float eps2,
    int n_split, int64_t split_len, int64_t self_offset, float *__restrict__ out,
    double *__restrict__ partial) {
    __shared__ float4 buf[kWarpsPerBlock][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t gwarp = (int64_t)blockIdx.x * kWarpsPerBlock + w;
    const int64_t nwarps = (int64_t)gridDim.x * kWarpsPerBlock;
    const int64_t ntiles = (nt + 32 * T - 1) / (32 * T);
    const int64_t nitems = ntiles * n_split;
    for (int64_t item = gwarp; item < nitems; item += nwarps) {
        const int64_t tile = item / n_split;
        const int s = (int)(item - tile * n_split);
        const int64_t jb = (int64_t)s * split_len;
        const int64_t je = min(ns, jb + split_len);
        float px[T], py[T], pz[T], sum[T], comp[T];
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int64_t i = tile * 32 * T + t * 32 + lane;
            const bool v = i < nt;
            px[t] = v ? tx[i] : kPadCoord;
            py[t] = v ? ty[i] : kPadCoord;
            pz[t] = v ? tz[i] : kPadCoord;
            sum[t] = 0.f;
            comp[t] = 0.f;
        }
        float4 nxt = load_source(m, x, y, z, jb + lane, je);
        for (int64_t j0 = jb; j0 < je; j0 += 32) {
            __syncwarp();
            buf[w][lane] = nxt;
            __syncwarp();
            nxt = load_source(m, x, y, z, j0 + 32 + lane, je);
            float part[T];
#pragma unroll
            for (int t = 0; t < T; ++t) part[t] = 0.f;
            if (MASK == HALMA_MASK_COORD) {
#pragma unroll 8
                for (int k = 0; k < 32; ++k) {
                    const float4 q = buf[w][k];
#pragma unroll
                    for (int t = 0; t < T; ++t) part[t] = pair_term_fast_masked(q, px[t], py[t], pz[t], eps2, part[t]);
                }
            } else if (MASK == HALMA_MASK_NONE) {
#pragma unroll 8
                for (int k = 0; k < 32; ++k) {
                    const float4 q = buf[w][k];
#pragma unroll
                    for (int t = 0; t < T; ++t) part[t] = pair_term_fast(q, px[t], py[t], pz[t], eps2, part[t]);
                }
            } else {
                // source index of target t's self pair relative to this chunk
                int64_t rel[T];
#pragma unroll
                for (int t = 0; t < T; ++t) rel[t] = tile * 32 * T + t * 32 + lane + self_offset - j0;
#pragma unroll 4
                for (int k = 0; k < 32; ++k) {
                    const float4 q = buf[w][k];
#pragma unroll
                    for (int t = 0; t < T; ++t) {
                        const float v = pair_term_fast(q, px[t], py[t], pz[t], eps2, part[t]);
                        part[t] = (rel[t] == k) ? part[t] : v;
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < T; ++t) two_sum_acc(sum[t], comp[t], part[t]);
        }
#pragma unroll
        for (int t = 0; t < T; ++t) {
            const int64_t i = tile * 32 * T + t * 32 + lane;
            if (i < nt) {
                if (n_split == 1) out[i] = sum[t] + comp[t];
                else partial[(int64_t)s * nt + i] = (double)sum[t] + (double)comp[t];
            }
        }
    }
}

// Deterministic combine of the per-slice partial sums (fixed slice order, FP64).
__global__ void reduce_partials_kernel(const double *__restrict__ partial, int n_split, int64_t nt,
                                       float *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt;
         i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int s = 0; s < n_split; ++s) acc += partial[(int64_t)s * nt + i];
        out[i] = (float)acc;
    }
}

// Plain FP64 path: one target per thread, FP64 pair terms and FP64 sum.
__global__ void __launch_bounds__(256) potential_f64_kernel(
    const double *__restrict__ m, const double *__restrict__ sx, const double *__restrict__ sy,
    const double *__restrict__ sz, int64_t ns, const double *__restrict__ tx,
    const double *__restrict__ ty, const double *__restrict__ tz, int64_t nt, double eps2,
    int mask, int64_t self_offset, double *__restrict__ phi) {
    __shared__ double4 buf[256];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool valid = i < nt;
    const double px = valid ? tx[i] : 0.0, py = valid ? ty[i] : 0.0, pz = valid ? tz[i] : 0.0;
    const int64_t self = valid ? i + self_offset : -1;
    double acc = 0.0;
    for (int64_t j0 = 0; j0 < ns; j0 += 256) {
        const int64_t j = j0 + threadIdx.x;
        __syncthreads();
        buf[threadIdx.x] = (j < ns) ? make_double4(sx[j], sy[j], sz[j], m[j]) : make_double4(0, 0, 0, 0);
        __syncthreads();
        const int cnt = (int)min((int64_t)256, ns - j0);
        for (int k = 0; k < cnt; ++k) {
            const double4 q = buf[k];
            const double dx = q.x - px, dy = q.y - py, dz = q.z - pz;
            bool keep = true;
            if (mask == HALMA_MASK_COORD) keep = (q.x != px) && (q.y != py) && (q.z != pz);
            else if (mask == HALMA_MASK_SELF) keep = (j0 + k) != self;
            const double r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2)));
            if (keep) acc = fma(q.w, rsqrt(r2), acc);
        }
    }
    if (valid) phi[i] = acc;
}

// Number of source slices so that (target tiles x slices) keeps every SM busy.
static void choose_split(int64_t ns, int64_t nt, int T, int *n_split, int64_t *split_len) {
    const int sms = device_sm_count();
    const int64_t ntiles = (nt + 32 * T - 1) / (32 * T);
    const int64_t want_items = (int64_t)sms * 64;   // ~2 waves of resident warps
    int64_t s = 1;
    if (ntiles < want_items) s = (want_items + ntiles - 1) / ntiles;
    const int64_t max_s = std::max<int64_t>(1, ns / 2048);   // keep slices >= 2048 sources
    s = std::min(s, max_s);
    s = std::min<int64_t>(s, 1024);
    int64_t len = (ns + s - 1) / s;
    len = (len + 31) / 32 * 32;
    s = std::max<int64_t>(1, (ns + len - 1) / len);
    *n_split = (int)s;
    *split_len = std::max<int64_t>(len, 32);
}

template <int T>
static int launch_fast(const float *m, const float *x, const float *y, const float *z, int64_t ns,
                       const float *tx, const float *ty, const float *tz, int64_t nt, float eps2,
                       int n_split, int64_t split_len, int mask, int64_t self_offset, float *out,
                       double *partial, cudaStream_t st) {
    const int64_t ntiles = (nt + 32 * T - 1) / (32 * T);
    const int64_t nitems = ntiles * n_split;
    const int sms = device_sm_count();
    const int grid = (int)std::min<int64_t>((nitems + kWarpsPerBlock - 1) / kWarpsPerBlock, (int64_t)sms * 8);
    if (mask == HALMA_MASK_COORD)
        HALMA_LAUNCH((bf_potential_fast_kernel<T, HALMA_MASK_COORD>), grid, 256, 0, st, m, x, y, z, ns, tx, ty, tz,
                     nt, eps2, n_split, split_len, self_offset, out, partial);
    else if (mask == HALMA_MASK_SELF)
        HALMA_LAUNCH((bf_potential_fast_kernel<T, HALMA_MASK_SELF>), grid, 256, 0, st, m, x, y, z, ns, tx, ty, tz,
                     nt, eps2, n_split, split_len, self_offset, out, partial);
    else
        HALMA_LAUNCH((bf_potential_fast_kernel<T, HALMA_MASK_NONE>), grid, 256, 0, st, m, x, y, z, ns, tx, ty, tz,
                     nt, eps2, n_split, split_len, self_offset, out, partial);
    return HALMA_OK;
}

// Stages the caller's arrays and runs the FP32-compensated kernel with the given mask.
static int potential_fast_api(int64_t ns, const float *mm, const float *sx_, const float *sy_, const float *sz_,
                              int64_t nt, const float *tx_, const float *ty_, const float *tz_, double eps2,
                              int mask, int64_t self_offset, float *out_, cudaStream_t st) {
    constexpr int T = 4;
    int n_split = 1;
    int64_t split_len = ns;
    if (ns > 0) choose_split(ns, nt, T, &n_split, &split_len);
    Stager sg;
    const float *m = nullptr, *x = nullptr, *y = nullptr, *z = nullptr, *tx = nullptr, *ty = nullptr, *tz = nullptr;
    float *out = nullptr;
    sg.add(mm, ns, true, false, &m);
    sg.add(sx_, ns, true, false, &x);
    sg.add(sy_, ns, true, false, &y);
    sg.add(sz_, ns, true, false, &z);
    sg.add(tx_, nt, true, false, &tx);
    sg.add(ty_, nt, true, false, &ty);
    sg.add(tz_, nt, true, false, &tz);
    sg.add((const float *)out_, nt, false, true, &out);
    Layout L;
    sg.plan(L);
    const size_t off_part = (n_split > 1) ? L.add(sizeof(double) * (size_t)n_split * nt) : 0;
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    HALMA_TRY(sg.bind_and_upload(base, st));
    if (ns == 0) {
        HALMA_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * nt, st));
    } else {
        double *partial = n_split > 1 ? at<double>(base, off_part) : nullptr;
        HALMA_TRY(launch_fast<T>(m, x, y, z, ns, tx, ty, tz, nt, (float)eps2, n_split, split_len, mask, self_offset,
                                 out, partial, st));
        if (n_split > 1)
            HALMA_LAUNCH(reduce_partials_kernel, grid_for(nt, 256, 4096), 256, 0, st, partial, n_split, nt, out);
    }
    return sg.download(st);
}

// ---------------------------------------------------------------------------------------
// Targets that are the first nt sources (self-potential of a set, plus other sources): the
// pairs inside the set go through the symmetric block kernel of the unbinding, each pair
// evaluated once for both particles; the remaining sources through the tile kernel.
constexpr int64_t kSymMinTargets = 8192;

__global__ void pack_sources_kernel(int64_t n, const float *__restrict__ m, const float *__restrict__ x,
                                    const float *__restrict__ y, const float *__restrict__ z, float4 *__restrict__ pk) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        pk[i] = make_float4(x[i], y[i], z[i], m[i]);
}

// phi_i = the set's slices in block order + the other sources (float32 or per-slice FP64
// partials) + the self term m_i eps^-1 when the self pair is counted (mask NONE); FP64 sum.
__global__ void sym_finish_kernel(int64_t nt, int nblk, int64_t npad, const float2 *__restrict__ part,
                                  const float *__restrict__ tail, const double *__restrict__ tail_part, int n_tail,
                                  const float *__restrict__ m, double self_scale, float *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nt; i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int b = 0; b < nblk; ++b) {
            const float2 v = part[(int64_t)b * npad + i];
            acc += (double)v.x + (double)v.y;
        }
        if (tail) acc += (double)tail[i];
        for (int s = 0; s < n_tail; ++s) acc += tail_part[(int64_t)s * nt + i];
        acc += self_scale * (double)m[i];
        out[i] = (float)acc;
    }
}

static int potential_sym_api(int64_t ns, const float *m, const float *x, const float *y, const float *z, int64_t nt,
                             double eps2, int mask, float *out, cudaStream_t st) {
    constexpr int T = 4;
    const int nblk = sym_block_count((int)nt);
    const int64_t npad = (nt + 31) / 32 * 32;
    const int64_t nrest = ns - nt;
    int n_split = 1;
    int64_t split_len = nrest;
    if (nrest > 0) choose_split(nrest, nt, T, &n_split, &split_len);
    Layout L;
    const size_t o_pk = L.add(sizeof(float4) * npad), o_part = L.add(sizeof(float2) * (size_t)nblk * npad);
    const size_t o_desc = L.add(512);
    const size_t o_tail = L.add(sizeof(float) * (nrest > 0 && n_split == 1 ? nt : 1));
    const size_t o_tp = L.add(sizeof(double) * (nrest > 0 && n_split > 1 ? (size_t)n_split * nt : 1));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 9));
    float4 *pk = at<float4>(base, o_pk);
    float2 *part = at<float2>(base, o_part);
    const int g = std::min(device_sm_count() * 8, grid_for(nt, 256));
    HALMA_LAUNCH(pack_sources_kernel, g, 256, 0, st, nt, m, x, y, z, pk);
    HALMA_TRY(sym_self_potential_device(pk, (int)nt, (float)eps2, part, at<void>(base, o_desc), st));
    float *tail = nullptr;
    double *tail_part = nullptr;
    if (nrest > 0) {
        if (n_split > 1) tail_part = at<double>(base, o_tp);
        else tail = at<float>(base, o_tail);
        HALMA_TRY(launch_fast<T>(m + nt, x + nt, y + nt, z + nt, nrest, x, y, z, nt, (float)eps2, n_split, split_len,
                                 HALMA_MASK_NONE, 0, tail, tail_part, st));
    }
    const double self_scale = (mask == HALMA_MASK_NONE && eps2 > 0.0) ? 1.0 / sqrt(eps2) : 0.0;
    HALMA_LAUNCH(sym_finish_kernel, g, 256, 0, st, nt, nblk, npad, part, tail, tail_part, tail_part ? n_split : 0, m,
                 self_scale, out);
    return HALMA_OK;
}

}  // namespace halma

using namespace halma;

extern "C" int halma_bf_potential_f32(int64_t ntotal, const float *total_mass, const float *total_x,
                                      const float *total_y, const float *total_z, int64_t ntest,
                                      const float *test_x, const float *test_y, const float *test_z,
                                      float *binding_energy, int32_t mode, double eps2,
                                      halma_stream_t stream) {
    if (ntotal < 0 || ntest < 0) return fail(HALMA_ERR_INVALID, "negative size (ntotal=%lld ntest=%lld)", (long long)ntotal, (long long)ntest);
    if (ntest == 0) return HALMA_OK;
    if (!binding_energy || !test_x || !test_y || !test_z) return fail(HALMA_ERR_INVALID, "null target/output pointer");
    if (ntotal > 0 && (!total_mass || !total_x || !total_y || !total_z)) return fail(HALMA_ERR_INVALID, "null source pointer");
    if (mode != HALMA_POT_REFERENCE && mode != HALMA_POT_FAST) return fail(HALMA_ERR_INVALID, "unknown mode %d", mode);
    if (!(eps2 >= 0.0) || !isfinite(eps2)) return fail(HALMA_ERR_INVALID, "eps2 must be finite and >= 0");
    if (mode == HALMA_POT_REFERENCE && eps2 != 0.0) return fail(HALMA_ERR_INVALID, "reference mode has no softening (eps2 must be 0)");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    if (mode == HALMA_POT_FAST)
        return potential_fast_api(ntotal, total_mass, total_x, total_y, total_z, ntest, test_x, test_y, test_z, eps2,
                                  HALMA_MASK_COORD, 0, binding_energy, st);
    Stager sg;
    const float *m = nullptr, *x = nullptr, *y = nullptr, *z = nullptr, *tx = nullptr, *ty = nullptr, *tz = nullptr;
    float *out = nullptr;
    sg.add(total_mass, ntotal, true, false, &m);
    sg.add(total_x, ntotal, true, false, &x);
    sg.add(total_y, ntotal, true, false, &y);
    sg.add(total_z, ntotal, true, false, &z);
    sg.add(test_x, ntest, true, false, &tx);
    sg.add(test_y, ntest, true, false, &ty);
    sg.add(test_z, ntest, true, false, &tz);
    sg.add((const float *)binding_energy, ntest, false, true, &out);
    Layout L;
    sg.plan(L);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    HALMA_TRY(sg.bind_and_upload(base, st));
    if (ntotal == 0) {
        HALMA_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * ntest, st));
    } else {
        const int64_t ntiles = (ntest + 31) / 32;
        const int grid = (int)std::min<int64_t>((ntiles + kWarpsPerBlock - 1) / kWarpsPerBlock, (int64_t)device_sm_count() * 16);
        HALMA_LAUNCH(bf_potential_reference_kernel, grid, 256, 0, st, m, x, y, z, ntotal, tx, ty, tz, ntest, out);
    }
    return sg.download(st);
}

extern "C" int halma_potential_f32(int64_t ns, const float *m, const float *sx, const float *sy, const float *sz,
                                   int64_t nt, const float *tx, const float *ty, const float *tz, double eps2,
                                   int32_t mask, int64_t self_offset, float *phi, halma_stream_t stream) {
    if (ns < 0 || nt < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (nt == 0) return HALMA_OK;
    if (!phi || !tx || !ty || !tz) return fail(HALMA_ERR_INVALID, "null target/output pointer");
    if (ns > 0 && (!m || !sx || !sy || !sz)) return fail(HALMA_ERR_INVALID, "null source pointer");
    if (mask < HALMA_MASK_COORD || mask > HALMA_MASK_NONE) return fail(HALMA_ERR_INVALID, "unknown mask %d", mask);
    if (!(eps2 >= 0.0) || !isfinite(eps2)) return fail(HALMA_ERR_INVALID, "eps2 must be finite and >= 0");
    std::lock_guard<std::mutex> guard(api_mutex());
    // targets that are the first sources (device arrays): the set's pairs once for both
    // particles; eps2 > 0 with mask NONE (the self pair is then a finite term), or mask SELF
    // skipping exactly the self pair
    const bool self_set = tx == sx && ty == sy && tz == sz && nt >= kSymMinTargets && nt <= ns &&
                          nt <= 65535ll * 1024 && ((mask == HALMA_MASK_NONE && eps2 > 0.0) ||
                                                   (mask == HALMA_MASK_SELF && self_offset == 0));
    if (self_set && is_device_pointer(m) && is_device_pointer(sx) && is_device_pointer(sy) && is_device_pointer(sz) &&
        is_device_pointer(phi))
        return potential_sym_api(ns, m, sx, sy, sz, nt, eps2, mask, phi, (cudaStream_t)stream);
    return potential_fast_api(ns, m, sx, sy, sz, nt, tx, ty, tz, eps2, mask, self_offset, phi, (cudaStream_t)stream);
}

extern "C" int halma_potential_f64(int64_t ns, const double *mm, const double *sx_, const double *sy_,
                                   const double *sz_, int64_t nt, const double *tx_, const double *ty_,
                                   const double *tz_, double eps2, int32_t mask, int64_t self_offset,
                                   double *phi, halma_stream_t stream) {
    if (ns < 0 || nt < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (nt == 0) return HALMA_OK;
    if (!phi || !tx_ || !ty_ || !tz_) return fail(HALMA_ERR_INVALID, "null target/output pointer");
    if (ns > 0 && (!mm || !sx_ || !sy_ || !sz_)) return fail(HALMA_ERR_INVALID, "null source pointer");
    if (mask < HALMA_MASK_COORD || mask > HALMA_MASK_NONE) return fail(HALMA_ERR_INVALID, "unknown mask %d", mask);
    if (!(eps2 >= 0.0) || !isfinite(eps2)) return fail(HALMA_ERR_INVALID, "eps2 must be finite and >= 0");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *m = nullptr, *sx = nullptr, *sy = nullptr, *sz = nullptr, *tx = nullptr, *ty = nullptr, *tz = nullptr;
    double *out = nullptr;
    sg.add(mm, ns, true, false, &m);
    sg.add(sx_, ns, true, false, &sx);
    sg.add(sy_, ns, true, false, &sy);
    sg.add(sz_, ns, true, false, &sz);
    sg.add(tx_, nt, true, false, &tx);
    sg.add(ty_, nt, true, false, &ty);
    sg.add(tz_, nt, true, false, &tz);
    sg.add((const double *)phi, nt, false, true, &out);
    Layout L;
    sg.plan(L);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    HALMA_TRY(sg.bind_and_upload(base, st));
    HALMA_LAUNCH(potential_f64_kernel, grid_for(nt, 256), 256, 0, st, m, sx, sy, sz, ns, tx, ty, tz, nt,
                 eps2, (int)mask, self_offset, out);
    return sg.download(st);
}

// ---------------------------------------------------------------------------------------
// Allocation-free variant of the fast (compensated FP32) potential.
//
// Some callers cannot let a library allocate device memory.  Simulation codes that embed the
// halo finder (an AMR code calling it between time steps, say) usually reserve almost all of
// the GPU's memory up front for their own pool and hand out pieces themselves, so a
// cudaMalloc from the library either fails or breaks the host's accounting; and a cudaFree
// synchronises the whole device, which stalls every other stream of a caller that keeps
// several streams busy.  This entry point serves such callers: it takes device arrays only
// and keeps its scratch -- the per-slice partial sums of the source-split kernel -- in the
// fixed array below instead of the library's cached workspace.  It calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// Limit: the scratch holds kNoAllocScratchDoubles = 2,097,152 partial sums (16 MiB).  The call
// splits the sources exactly as halma_bf_potential_f32 does in HALMA_POT_FAST mode and runs
// the same kernels, so the two return identical values; when that split needs more than
// 2,097,152 partial sums (source slices x targets) the call is rejected with
// HALMA_ERR_CAPACITY.
//
// Every GPU that loads this library holds the 16 MiB array until the process exits.  All calls
// share it and it keeps the previous call's contents; each partial sum a call reads is written
// by the same call first, so nothing needs clearing.  Calls that overlap on the GPU (two
// streams, or two host threads without ordering) race on the array and give wrong results.
// The first call on each device looks up the array's device address (cudaGetSymbolAddress with
// that device current); make that first call before any stream capture begins.
constexpr int64_t kNoAllocScratchDoubles = 1ll << 21;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {};

// Memory the current device's kernels can use in place: device memory of this device, or
// managed memory.  Another GPU's device memory is refused rather than read over the peer link.
bool is_local_device_pointer(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == current_device();
}

// Device address of g_noalloc_scratch on the current device (looked up once per device).
int noalloc_scratch(double **out) {
    const int dev = current_device();
    if (dev < 0 || dev >= kMaxDevices) return fail(HALMA_ERR_CAPACITY, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> g(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        HALMA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return HALMA_OK;
}
}  // namespace

extern "C" int halma_bf_potential_f32_noalloc(int64_t ntotal, const float *total_mass, const float *total_x,
                                              const float *total_y, const float *total_z, int64_t ntest,
                                              const float *test_x, const float *test_y, const float *test_z,
                                              float *binding_energy, double eps2, halma_stream_t stream) {
    if (ntotal < 0 || ntest < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (ntest == 0) return HALMA_OK;
    if (!binding_energy || !test_x || !test_y || !test_z) return fail(HALMA_ERR_INVALID, "null target/output pointer");
    if (ntotal > 0 && (!total_mass || !total_x || !total_y || !total_z)) return fail(HALMA_ERR_INVALID, "null source pointer");
    if (!(eps2 >= 0.0) || !isfinite(eps2)) return fail(HALMA_ERR_INVALID, "eps2 must be finite and >= 0");
    const void *arrays[8] = {test_x, test_y, test_z, binding_energy, total_mass, total_x, total_y, total_z};
    for (int k = 0; k < (ntotal > 0 ? 8 : 4); ++k)
        if (!is_local_device_pointer(arrays[k]))
            return fail(HALMA_ERR_INVALID,
                        "the allocation-free entry point takes arrays in the current device's memory only");
    cudaStream_t st = (cudaStream_t)stream;
    if (ntotal == 0) {
        HALMA_CUDA(cudaMemsetAsync(binding_energy, 0, sizeof(float) * ntest, st));
        return HALMA_OK;
    }
    constexpr int T = 4;
    int n_split = 1;
    int64_t split_len = ntotal;
    choose_split(ntotal, ntest, T, &n_split, &split_len);
    if (n_split > 1 && (int64_t)n_split * ntest > kNoAllocScratchDoubles)
        return fail(HALMA_ERR_CAPACITY,
                    "this call needs %lld partial sums (%d source slices x %lld targets); the allocation-free "
                    "scratch holds %lld — use halma_bf_potential_f32",
                    (long long)n_split * ntest, n_split, (long long)ntest, (long long)kNoAllocScratchDoubles);
    double *scratch = nullptr;
    HALMA_TRY(noalloc_scratch(&scratch));
    double *partial = n_split > 1 ? scratch : nullptr;
    HALMA_TRY(launch_fast<T>(total_mass, total_x, total_y, total_z, ntotal, test_x, test_y, test_z, ntest,
                             (float)eps2, n_split, split_len, HALMA_MASK_COORD, 0, binding_energy, partial, st));
    if (n_split > 1)
        HALMA_LAUNCH(reduce_partials_kernel, grid_for(ntest, 256, 4096), 256, 0, st, partial, n_split, ntest,
                     binding_energy);
    return HALMA_OK;
}
