// Per-halo FP64 reductions over CSR halo segments (python_scripts/halo_properties.py):
//   total_mass (:16-24), center_of_mass (:26-43), CM_velocity (:45-60),
//   furthest_particle (:98-111), half_mass_radius (:365-392), sigma_effective (:607-625).
// One block per halo for the sums; the half-mass radius needs the members in increasing
// distance from the centre, obtained with two stable radix sorts over all particles (by the
// FP64 distance bits, then by halo id), after which each halo walks its own segment.
#include <limits.h>
#include <math.h>

#include "common.cuh"
#include "sort.cuh"

namespace halma {
namespace {

struct Red {
    double M, cx, cy, cz, vx, vy, vz, rmax, r05, sigma, n, mref;
};

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double wmax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

template <int NV>
__device__ void bsum(double (&v)[NV], double (*sh)[32]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        const double s = wsum(v[q]);
        if (lane == 0) sh[q][w] = s;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = lane < nw ? sh[q][lane] : 0.0;
            s = wsum(s);
            if (lane == 0) sh[q][0] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) v[q] = sh[q][0];
    __syncthreads();
}

// Sums, centre, bulk velocity, R_max, and the sort keys (distance bits, halo id).
__global__ void __launch_bounds__(256) red_sums_kernel(const int64_t *__restrict__ off, const double *__restrict__ x,
                                                       const double *__restrict__ y, const double *__restrict__ z,
                                                       const double *__restrict__ vx, const double *__restrict__ vy,
                                                       const double *__restrict__ vz, const double *__restrict__ m,
                                                       const unsigned char *__restrict__ mask,
                                                       const double *__restrict__ about, Red *__restrict__ red,
                                                       uint64_t *__restrict__ dkey, double *__restrict__ dist,
                                                       uint32_t *__restrict__ hid) {
    const int h = blockIdx.x;
    __shared__ double sh[8][32];
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int64_t b = off[h], e = off[h + 1];
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        if (mask && !mask[i]) continue;
        const double mi = m[i];
        v[0] += mi;
        v[1] += mi * x[i];
        v[2] += mi * y[i];
        v[3] += mi * z[i];
        v[4] += mi * vx[i];
        v[5] += mi * vy[i];
        v[6] += mi * vz[i];
        v[7] += 1.0;
    }
    bsum<8>(v, sh);
    const double M = v[0];
    double cx = 0, cy = 0, cz = 0, ux = 0, uy = 0, uz = 0;
    if (M > 0) {
        cx = v[1] / M; cy = v[2] / M; cz = v[3] / M;
        ux = v[4] / M; uy = v[5] / M; uz = v[6] / M;
    }
    double Mref = M, r05_in = NAN;
    if (about) {
        const double *a = about + (int64_t)h * HALMA_ABOUT_NFIELDS;
        if (!isnan(a[HALMA_ABOUT_CX])) cx = a[HALMA_ABOUT_CX];
        if (!isnan(a[HALMA_ABOUT_CY])) cy = a[HALMA_ABOUT_CY];
        if (!isnan(a[HALMA_ABOUT_CZ])) cz = a[HALMA_ABOUT_CZ];
        if (!isnan(a[HALMA_ABOUT_VX])) ux = a[HALMA_ABOUT_VX];
        if (!isnan(a[HALMA_ABOUT_VY])) uy = a[HALMA_ABOUT_VY];
        if (!isnan(a[HALMA_ABOUT_VZ])) uz = a[HALMA_ABOUT_VZ];
        if (!isnan(a[HALMA_ABOUT_MASS])) Mref = a[HALMA_ABOUT_MASS];
        r05_in = a[HALMA_ABOUT_R05];
    }
    double rmax = 0.0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const bool in = !mask || mask[i];
        const double dx = cx - x[i], dy = cy - y[i], dz = cz - z[i];
        // (dx**2 + dy**2 + dz**2)**0.5 as the reference evaluates it (halo_properties.py:104-107),
        // each operation rounded on its own so that d < R05 splits members the same way
        const double d = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
        dist[i] = d;
        if (in) rmax = fmax(rmax, d);
        // excluded particles sort after every member (+inf)
        dkey[i] = in ? (uint64_t)__double_as_longlong(d) : 0x7ff0000000000000ull;
        hid[i] = (uint32_t)h;
    }
    __shared__ double shm[32];
    const double wm = wmax(rmax);
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = wm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r = fmax(r, shm[q]);
        Red o;
        o.M = M; o.cx = cx; o.cy = cy; o.cz = cz; o.vx = ux; o.vy = uy; o.vz = uz;
        o.rmax = r; o.r05 = r05_in; o.sigma = 0; o.n = v[7]; o.mref = Mref;
        red[h] = o;
    }
}

__global__ void gather_hid_kernel(int64_t n, const int *__restrict__ perm, const uint32_t *__restrict__ hid,
                                  uint32_t *__restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = hid[perm[k]];
}

// Half-mass radius: walk the halo's members by increasing distance, running FP64 mass sum;
// R05 is the distance of the last member before the sum first exceeds M/2 (the smallest
// distance if the first member already exceeds it).  Then sigma inside R05.
__global__ void __launch_bounds__(256) red_r05_kernel(const int64_t *__restrict__ off, const int *__restrict__ order,
                                                      const double *__restrict__ dist, const double *__restrict__ vx,
                                                      const double *__restrict__ vy, const double *__restrict__ vz,
                                                      const double *__restrict__ m, const unsigned char *__restrict__ mask,
                                                      Red *__restrict__ red) {
    const int h = blockIdx.x;
    const int64_t b = off[h], e = off[h + 1];
    const Red r = red[h];
    const int64_t nmem = (int64_t)r.n;
    __shared__ long long first;
    const double half = 0.5 * r.mref;
    const bool given = !isnan(r.r05);   // caller supplied R05: skip the search
    if (threadIdx.x == 0) first = LLONG_MAX;
    __syncthreads();
    if (!given) {
        // one running FP64 sum in increasing distance, added in order like the reference's loop
        // (halo_properties.py:385-390): the block stages 1024 masses in shared memory, thread 0
        // adds them one by one and stops at the first sum above M/2
        __shared__ double tile[1024];
        __shared__ double cum;
        if (threadIdx.x == 0) cum = 0.0;
        for (int64_t k0 = 0; k0 < nmem; k0 += 1024) {
            const int cnt = nmem - k0 < 1024 ? (int)(nmem - k0) : 1024;
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) tile[q] = m[order[b + k0 + q]];
            __syncthreads();
            if (threadIdx.x == 0) {
                // eight masses at a time: the loads and the chain of adds do not wait on each
                // other's branches; the first sum above M/2 is found after each batch
                double c = cum;
                long long f = LLONG_MAX;
                int q = 0;
                for (; q + 8 <= cnt && f == LLONG_MAX; q += 8) {
                    double t[8], cs[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) t[u] = tile[q + u];
                    cs[0] = __dadd_rn(c, t[0]);
#pragma unroll
                    for (int u = 1; u < 8; ++u) cs[u] = __dadd_rn(cs[u - 1], t[u]);
#pragma unroll
                    for (int u = 7; u >= 0; --u)
                        if (cs[u] > half) f = k0 + q + u;
                    c = cs[7];
                }
                for (; q < cnt && f == LLONG_MAX; ++q) {
                    c = __dadd_rn(c, tile[q]);
                    if (c > half) f = k0 + q;
                }
                if (f != LLONG_MAX) first = f;
                cum = c;
            }
            __syncthreads();
            if (first != LLONG_MAX) break;
        }
    }
    __syncthreads();
    __shared__ double r05s;
    if (threadIdx.x == 0) {
        double r05 = 0.0;
        if (given) {
            r05 = r.r05;
        } else if (nmem > 0) {
            const long long f = first == LLONG_MAX ? -1 : first;
            if (f > 0) r05 = dist[order[b + f - 1]];
            else if (f == 0) r05 = dist[order[b]];
            else r05 = dist[order[b + nmem - 1]];
        }
        r05s = r05;
    }
    __syncthreads();
    const double r05 = r05s;
    __shared__ double sh[2][32];
    double v[2] = {0, 0};
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        if (mask && !mask[i]) continue;
        if (dist[i] < r05) {
            const double dx = vx[i] - r.vx, dy = vy[i] - r.vy, dz = vz[i] - r.vz;
            v[0] += dx * dx + dy * dy + dz * dz;
            v[1] += 1.0;
        }
    }
    bsum<2>(v, sh);
    if (threadIdx.x == 0) {
        red[h].r05 = r05;
        red[h].sigma = v[1] > 0 ? sqrt(v[0] / 3.0 / v[1]) : 0.0;
    }
}

__global__ void red_out_kernel(int nh, const Red *__restrict__ red, double *__restrict__ out) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
        const Red r = red[h];
        double *o = out + (int64_t)h * HALMA_RED_NFIELDS;
        o[HALMA_RED_MASS] = r.M;
        o[HALMA_RED_CX] = r.cx; o[HALMA_RED_CY] = r.cy; o[HALMA_RED_CZ] = r.cz;
        o[HALMA_RED_VX] = r.vx; o[HALMA_RED_VY] = r.vy; o[HALMA_RED_VZ] = r.vz;
        o[HALMA_RED_RMAX] = r.rmax;
        o[HALMA_RED_R05] = r.r05;
        o[HALMA_RED_SIGMA] = r.sigma;
        o[HALMA_RED_N] = r.n;
    }
}

__global__ void iota_kernel(int64_t n, int *__restrict__ v) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        v[k] = (int)k;
}

}  // namespace

int reductions_device(int64_t n, int nh, const int64_t *off, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, const double *m,
                      const unsigned char *mask, const double *about, double *out, cudaStream_t st) {
    const int N = (int)std::max<int64_t>(n, 1);
    const size_t s64 = sort_pairs_u64_i32_bytes(N, 64), s32 = sort_pairs_u32_i32_bytes(N);
    Layout L;
    const size_t o_red = L.add(sizeof(Red) * nh);
    const size_t o_dk = L.add(8ull * N), o_dk2 = L.add(8ull * N), o_dist = L.add(8ull * N);
    const size_t o_hid = L.add(4ull * N), o_hid2 = L.add(4ull * N), o_hid3 = L.add(4ull * N);
    const size_t o_v0 = L.add(4ull * N), o_v1 = L.add(4ull * N), o_v2 = L.add(4ull * N);
    const size_t o_tmp = L.add(std::max(s64, s32));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    Red *red = at<Red>(base, o_red);
    auto *dk = at<uint64_t>(base, o_dk), *dk2 = at<uint64_t>(base, o_dk2);
    auto *dist = at<double>(base, o_dist);
    auto *hid = at<uint32_t>(base, o_hid), *hid2 = at<uint32_t>(base, o_hid2), *hid3 = at<uint32_t>(base, o_hid3);
    auto *v0 = at<int>(base, o_v0), *v1 = at<int>(base, o_v1), *v2 = at<int>(base, o_v2);
    void *tmp = at<void>(base, o_tmp);
    HALMA_LAUNCH(red_sums_kernel, nh, 256, 0, st, off, x, y, z, vx, vy, vz, m, mask, about, red, dk, dist, hid);
    if (n > 0) {
        const int g = std::min(device_sm_count() * 8, grid_for(n, 256));
        HALMA_LAUNCH(iota_kernel, g, 256, 0, st, n, v0);
        HALMA_TRY(sort_pairs_u64_i32(tmp, s64, dk, dk2, v0, v1, (int)n, 64, st));
        HALMA_LAUNCH(gather_hid_kernel, g, 256, 0, st, n, v1, hid, hid2);
        HALMA_TRY(sort_pairs_u32_i32(tmp, s32, hid2, hid3, v1, v2, (int)n, 32, st));
    }
    HALMA_LAUNCH(red_r05_kernel, nh, 256, 0, st, off, v2, dist, vx, vy, vz, m, mask, red);
    HALMA_LAUNCH(red_out_kernel, grid_for(nh, 256), 256, 0, st, nh, red, out);
    return HALMA_OK;
}

}  // namespace halma

using namespace halma;

extern "C" int halma_halo_reductions(int64_t n, int64_t n_haloes, const int64_t *offsets, const double *x,
                                     const double *y, const double *z, const double *vx, const double *vy,
                                     const double *vz, const double *m, const uint8_t *mask, const double *about_, double *out,
                                     halma_stream_t stream) {
    if (n < 0 || n_haloes < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= (1ll << 31) - 1 || n_haloes >= (1ll << 31) - 1) return fail(HALMA_ERR_CAPACITY, "too many particles or haloes");
    if (n_haloes == 0) return HALMA_OK;
    if (!offsets || !out || (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const int64_t *off = nullptr;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dvx = nullptr, *dvy = nullptr, *dvz = nullptr,
                 *dm = nullptr;
    const uint8_t *dmask = nullptr;
    double *dout = nullptr;
    sg.add(offsets, n_haloes + 1, true, false, &off);
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(vx, n, true, false, &dvx);
    sg.add(vy, n, true, false, &dvy);
    sg.add(vz, n, true, false, &dvz);
    sg.add(m, n, true, false, &dm);
    sg.add(mask, mask ? n : 0, true, false, &dmask);
    const double *dabout = nullptr;
    sg.add(about_, about_ ? n_haloes * HALMA_ABOUT_NFIELDS : 0, true, false, &dabout);
    sg.add((const double *)out, n_haloes * HALMA_RED_NFIELDS, false, true, &dout);
    void *stage = nullptr;
    if (sg.any_host) {
        Layout L;
        sg.plan(L);
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
    }
    int s = sg.bind_and_upload(stage, st);
    if (s == HALMA_OK)
        s = reductions_device(n, (int)n_haloes, off, dx, dy, dz, dvx, dvy, dvz, dm, dmask, dabout, dout, st);
    if (s == HALMA_OK) s = sg.download(st);
    if (stage) {
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
    }
    return s;
}
