// Ball gather: the particles inside spheres around many halo centres, all spheres in one
// launch sequence.  Replaces the per-halo range queries of pyHALMA's gas / potential set-up
// (python_scripts/halo_gas.py:223-277 st_gas_dm_particles_inside):
//   * st_kdtree / dm_kdtree.query_ball_point([cx, cy, cz], R)  (halo_gas.py:254, 268): every
//     particle with ((dx*dx + dy*dy) + dz*dz) <= R*R in IEEE double (scipy's KDTree pair rule,
//     the one its FoF uses);
//   * parallel_inside(x, y, z, R, cx, cy, cz) (halo_gas.py:218-220, 237):
//     sqrt((x-cx)**2 + (y-cy)**2 + (z-cz)**2) < R (strict).
//
// Pipeline (one stream): particles get a row-major cell key at a cell side h chosen from the
// radii and are radix-sorted by it (stable, so a cell keeps its particles in index order);
// their FP64 coordinates are gathered into sorted SoA arrays.  Per sphere one block covers
// the (x, y) columns of cells that the sphere touches: each lane binary-searches the sorted
// keys for one column's z-range of cells, then the warp scans the 32 columns' particle ranges
// with coalesced loads and applies the exact predicate.  A count pass, an exclusive scan and a
// fill pass give CSR output; one radix sort of (sphere, index) keys puts every sphere's
// indices in ascending order.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

struct BallGrid {
    double xmin, ymin, zmin, inv_h;
    long long ncx, ncy, ncz;
};

__device__ __forceinline__ uint64_t cell_key(const BallGrid &g, long long cx, long long cy, long long cz) {
    return ((uint64_t)cx * (uint64_t)g.ncy + (uint64_t)cy) * (uint64_t)g.ncz + (uint64_t)cz;
}

__device__ __forceinline__ long long cell_of(double v, double vmin, double inv_h, long long nc) {
    long long c = (long long)floor((v - vmin) * inv_h);
    return min(max(c, 0ll), nc - 1);
}

__global__ void bg_keys_kernel(int n, const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, BallGrid g, uint64_t *__restrict__ keys,
                               int *__restrict__ vals) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        keys[i] = cell_key(g, cell_of(x[i], g.xmin, g.inv_h, g.ncx), cell_of(y[i], g.ymin, g.inv_h, g.ncy),
                           cell_of(z[i], g.zmin, g.inv_h, g.ncz));
        vals[i] = i;
    }
}

__global__ void bg_sorted_soa_kernel(int n, const int *__restrict__ idx, const double *__restrict__ x,
                                     const double *__restrict__ y, const double *__restrict__ z,
                                     double *__restrict__ sx, double *__restrict__ sy, double *__restrict__ sz) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = idx[k];
        sx[k] = x[i];
        sy[k] = y[i];
        sz[k] = z[i];
    }
}

__device__ __forceinline__ int lower_bound_u64(const uint64_t *__restrict__ keys, int n, uint64_t k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Cell range [c0, c1] along one axis that can hold a point within r of c (a margin of 1e-6
// cells absorbs the rounding of the cell arithmetic); c0 > c1 when the sphere misses the grid.
__device__ __forceinline__ void cell_span(double c, double r, double vmin, double inv_h, long long nc,
                                          long long &c0, long long &c1) {
    const double lo = floor((c - r - vmin) * inv_h - 1e-6), hi = floor((c + r - vmin) * inv_h + 1e-6);
    if (!(hi >= 0.0) || !(lo <= (double)(nc - 1))) {
        c0 = 1;
        c1 = 0;
        return;
    }
    c0 = lo < 0.0 ? 0 : (long long)lo;
    c1 = hi > (double)(nc - 1) ? nc - 1 : (long long)hi;
}

__device__ __forceinline__ bool inside(double px, double py, double pz, double cx, double cy, double cz, double r,
                                       double r2, int strict) {
    const double dx = __dsub_rn(px, cx), dy = __dsub_rn(py, cy), dz = __dsub_rn(pz, cz);
    const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return strict ? __dsqrt_rn(d2) < r : d2 <= r2;
}

// Work items: a sphere's (x, y) cell columns cut into runs of 32, one warp per run, so a big
// sphere spreads over many warps.  span[s] = the sphere's cell ranges (x0, x1, y0, y1, z0, z1).
__global__ void bg_span_kernel(int nb, const double *__restrict__ bx, const double *__restrict__ by,
                               const double *__restrict__ bz, const double *__restrict__ br, BallGrid g,
                               long long *__restrict__ span, int *__restrict__ nitems) {
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nb; s += gridDim.x * blockDim.x) {
        long long c[6];
        const double r = br[s];
        cell_span(bx[s], r, g.xmin, g.inv_h, g.ncx, c[0], c[1]);
        cell_span(by[s], r, g.ymin, g.inv_h, g.ncy, c[2], c[3]);
        cell_span(bz[s], r, g.zmin, g.inv_h, g.ncz, c[4], c[5]);
        const long long ncols = (c[1] >= c[0] && c[3] >= c[2] && c[5] >= c[4]) ? (c[1] - c[0] + 1) * (c[3] - c[2] + 1) : 0;
        for (int q = 0; q < 6; ++q) span[6 * (int64_t)s + q] = c[q];
        nitems[s] = (int)((ncols + 31) / 32);
    }
}

__device__ __forceinline__ int item_owner(const int *__restrict__ istart, int nb, int item) {
    int lo = 0, hi = nb - 1;   // last sphere whose first item is <= item
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (istart[mid] <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// FILL = false: counts[item] = particles inside the item's sphere in its 32 columns.
// FILL = true: writes (sphere << 32 | index) for them from offs[item] on (any order).
template <bool FILL>
__global__ void __launch_bounds__(256) bg_item_kernel(
    int nitem, int nb, const int *__restrict__ istart, const long long *__restrict__ span,
    const double *__restrict__ bx, const double *__restrict__ by, const double *__restrict__ bz,
    const double *__restrict__ br, int strict, BallGrid g, int n, const uint64_t *__restrict__ keys,
    const double *__restrict__ sx, const double *__restrict__ sy, const double *__restrict__ sz,
    const int *__restrict__ sidx, int64_t *__restrict__ counts, const int64_t *__restrict__ offs,
    uint64_t *__restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int item = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; item < nitem; item += warps) {
        const int s = item_owner(istart, nb, item);
        const long long *c = span + 6 * (int64_t)s;
        const long long nyc = c[3] - c[2] + 1;
        const long long ncols = (c[1] - c[0] + 1) * nyc;
        const double cx = bx[s], cy = by[s], cz = bz[s], r = br[s];
        const double r2 = __dmul_rn(r, r);
        const long long col = (long long)(item - istart[s]) * 32 + lane;
        int lo = 0, hi = 0;
        if (col < ncols) {
            const long long ix = c[0] + col / nyc, iy = c[2] + col % nyc;
            // the column's closest point to the centre in x-y; a column entirely outside the
            // sphere is skipped, the others scan only the cells the chord through that point
            // can reach (radius enlarged by 1e-9 and 1e-6 cells of margin: the exact test
            // below decides membership, the pruning only has to keep every candidate)
            const double h = 1.0 / g.inv_h;
            const double xl = g.xmin + (double)ix * h, yl = g.ymin + (double)iy * h;
            const double ex = fmax(0.0, fmax(xl - cx, cx - (xl + h))), ey = fmax(0.0, fmax(yl - cy, cy - (yl + h)));
            const double rr = r * (1.0 + 1e-9) + 1e-6 * h;
            const double rest = rr * rr - (ex * ex + ey * ey);
            if (rest >= 0.0) {
                const double zh = sqrt(rest);
                long long z0 = (long long)floor((cz - zh - g.zmin) * g.inv_h - 1e-6);
                long long z1 = (long long)floor((cz + zh - g.zmin) * g.inv_h + 1e-6);
                z0 = z0 < c[4] ? c[4] : z0;
                z1 = z1 > c[5] ? c[5] : z1;
                if (z1 >= z0) {
                    lo = lower_bound_u64(keys, n, cell_key(g, ix, iy, z0));
                    hi = lower_bound_u64(keys, n, cell_key(g, ix, iy, z1) + 1);
                }
            }
        }
        long long hits = 0;
        unsigned long long base = FILL ? (unsigned long long)offs[item] : 0ull;
        for (int t = 0; t < 32; ++t) {
            const int b = __shfl_sync(0xffffffffu, lo, t), e = __shfl_sync(0xffffffffu, hi, t);
            for (int p0 = b; p0 < e; p0 += 32) {
                const int p = p0 + lane;
                const bool in = p < e && inside(sx[p], sy[p], sz[p], cx, cy, cz, r, r2, strict);
                if (!FILL) {
                    hits += in ? 1 : 0;
                } else {
                    const unsigned bal = __ballot_sync(0xffffffffu, in);
                    if (in) out[base + __popc(bal & ((1u << lane) - 1u))] = ((uint64_t)s << 32) | (uint64_t)(uint32_t)sidx[p];
                    base += __popc(bal);
                }
            }
        }
        if (!FILL) {
            for (int o = 16; o > 0; o >>= 1) hits += __shfl_down_sync(0xffffffffu, hits, o);
            if (lane == 0) counts[item] = hits;
        }
    }
}

// Per-sphere output offsets from the items' offsets (a sphere without items starts where
// the next items start); off[nb] = total.
__global__ void bg_sphere_off_kernel(int nb, int nitem, const int *__restrict__ istart,
                                     const int64_t *__restrict__ item_off, const int64_t *__restrict__ item_cnt,
                                     int64_t *__restrict__ off) {
    const int64_t total = nitem > 0 ? item_off[nitem - 1] + item_cnt[nitem - 1] : 0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s <= nb; s += gridDim.x * blockDim.x)
        off[s] = (s < nb && istart[s] < nitem) ? item_off[istart[s]] : total;
}

__global__ void bg_extract_kernel(int64_t m, const uint64_t *__restrict__ keys, int *__restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (int)(uint32_t)(keys[k] & 0xffffffffull);
}

int bits_of(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_ball_gather(int64_t n, const double *x, const double *y, const double *z, int64_t n_balls,
                                 const double *cx, const double *cy, const double *cz, const double *radius,
                                 int32_t strict, int64_t *offsets, int32_t *indices, int64_t capacity,
                                 int64_t *n_found, halma_stream_t stream) {
    if (!n_found) return fail(HALMA_ERR_INVALID, "n_found must not be NULL");
    if (n < 0 || n_balls < 0 || capacity < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= INT32_MAX || n_balls >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles and spheres");
    if (strict != 0 && strict != 1) return fail(HALMA_ERR_INVALID, "strict must be 0 or 1");
    if ((n > 0 && (!x || !y || !z)) || (n_balls > 0 && (!cx || !cy || !cz || !radius)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    *n_found = 0;
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    // the spheres on the host: validity and the cell side
    std::vector<double> hb(4 * (size_t)n_balls);
    const double *bsrc[4] = {cx, cy, cz, radius};
    for (int q = 0; q < 4; ++q)
        if (n_balls > 0) HALMA_CUDA(cudaMemcpy(hb.data() + q * n_balls, bsrc[q], 8ull * n_balls, cudaMemcpyDefault));
    std::vector<double> rs(hb.begin() + 3 * n_balls, hb.end());
    for (int64_t s = 0; s < n_balls; ++s) {
        if (!(rs[s] >= 0.0) || !isfinite(rs[s])) return fail(HALMA_ERR_INVALID, "radius %lld is not finite and >= 0", (long long)s);
        for (int q = 0; q < 3; ++q)
            if (!isfinite(hb[q * n_balls + s])) return fail(HALMA_ERR_INVALID, "centre %lld is not finite", (long long)s);
    }
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dbx = nullptr, *dby = nullptr, *dbz = nullptr,
                 *dbr = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(cx, n_balls, true, false, &dbx);
    sg.add(cy, n_balls, true, false, &dby);
    sg.add(cz, n_balls, true, false, &dbz);
    sg.add(radius, n_balls, true, false, &dbr);
    // phase-1 data lives in workspace slot 4 (the bounding box uses slot 0), the work items in
    // slot 5, the fill in slot 8
    const int N = (int)std::max<int64_t>(n, 1), NB = (int)std::max<int64_t>(n_balls, 1);
    const size_t s64 = sort_pairs_u64_i32_bytes(N, 64), scan_b = exclusive_sum_i64_bytes(NB);
    Layout L;
    sg.plan(L);
    const size_t o_kin = L.add(8ull * N), o_kout = L.add(8ull * N), o_vin = L.add(4ull * N), o_vout = L.add(4ull * N);
    const size_t o_sx = L.add(8ull * N), o_sy = L.add(8ull * N), o_sz = L.add(8ull * N);
    const size_t o_span = L.add(48ull * NB), o_nit = L.add(4ull * NB), o_ist = L.add(4ull * NB);
    const size_t o_off = L.add(8ull * (NB + 1)), o_tmp = L.add(std::max(s64, std::max(scan_b,
                                                                                    exclusive_sum_i32_bytes(NB))));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 4));
    HALMA_TRY(sg.bind_and_upload(base, st));
    auto *kin = at<uint64_t>(base, o_kin), *kout = at<uint64_t>(base, o_kout);
    auto *vin = at<int>(base, o_vin), *vout = at<int>(base, o_vout);
    auto *sx = at<double>(base, o_sx), *sy = at<double>(base, o_sy), *sz = at<double>(base, o_sz);
    auto *span = at<long long>(base, o_span);
    int *nit = at<int>(base, o_nit), *ist = at<int>(base, o_ist);
    auto *offs = at<int64_t>(base, o_off);
    void *tmp = at<void>(base, o_tmp);
    const int sms = device_sm_count();
    int64_t total = 0;
    if (n > 0 && n_balls > 0) {
        double bb[7];
        HALMA_TRY(bbox_device((int)n, dx, dy, dz, bb, st));
        if (bb[6] != 0.0) return fail(HALMA_ERR_INVALID, "non-finite particle position");
        // cell side: a quarter of the median radius, at least 1/512 of the largest (a big sphere
        // then covers at most ~1025 x 1025 columns) and 2^-20 of the extent (at most ~1e6 cells
        // a side)
        std::vector<double> r2 = rs;
        std::nth_element(r2.begin(), r2.begin() + r2.size() / 2, r2.end());
        const double rmax = *std::max_element(rs.begin(), rs.end());
        const double ext = std::max(bb[3] - bb[0], std::max(bb[4] - bb[1], bb[5] - bb[2]));
        double h = std::max(0.25 * r2[r2.size() / 2], std::max(rmax / 512.0, ext * 0x1p-20));
        if (!(h > 0.0)) h = 1.0;
        BallGrid g;
        g.xmin = bb[0];
        g.ymin = bb[1];
        g.zmin = bb[2];
        g.inv_h = 1.0 / h;
        g.ncx = (long long)floor((bb[3] - bb[0]) * g.inv_h) + 1;
        g.ncy = (long long)floor((bb[4] - bb[1]) * g.inv_h) + 1;
        g.ncz = (long long)floor((bb[5] - bb[2]) * g.inv_h) + 1;
        if ((long double)g.ncx * g.ncy * g.ncz > 4.0e18L) return fail(HALMA_ERR_CAPACITY, "cell grid too large");
        const int end_bit = bits_of((uint64_t)(g.ncx * g.ncy * g.ncz - 1));
        const int g1 = std::min(sms * 8, grid_for(n, 256));
        HALMA_LAUNCH(bg_keys_kernel, g1, 256, 0, st, (int)n, dx, dy, dz, g, kin, vin);
        HALMA_TRY(sort_pairs_u64_i32(tmp, s64, kin, kout, vin, vout, (int)n, end_bit, st));
        HALMA_LAUNCH(bg_sorted_soa_kernel, g1, 256, 0, st, (int)n, vout, dx, dy, dz, sx, sy, sz);
        // work items: 32-column runs of every sphere
        HALMA_LAUNCH(bg_span_kernel, grid_for(n_balls, 256), 256, 0, st, (int)n_balls, dbx, dby, dbz, dbr, g, span, nit);
        HALMA_TRY(exclusive_sum_i32(tmp, exclusive_sum_i32_bytes(NB), nit, ist, (int)n_balls, st));
        int last[2];
        HALMA_CUDA(cudaMemcpyAsync(&last[0], ist + n_balls - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaMemcpyAsync(&last[1], nit + n_balls - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        const int64_t nitem64 = (int64_t)last[0] + last[1];
        if (nitem64 >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "too many cell columns to scan");
        const int nitem = (int)nitem64;
        const int NI = std::max(nitem, 1);
        Layout I;
        const size_t o_icnt = I.add(8ull * NI), o_ioff = I.add(8ull * NI), o_itmp = I.add(exclusive_sum_i64_bytes(NI));
        void *ib = nullptr;
        HALMA_TRY(workspace(I.total, &ib, st, 5));
        auto *icnt = at<int64_t>(ib, o_icnt), *ioff = at<int64_t>(ib, o_ioff);
        const int gi = std::min(sms * 16, grid_for((int64_t)nitem * 32, 256));
        if (nitem > 0) {
            HALMA_LAUNCH(bg_item_kernel<false>, gi, 256, 0, st, nitem, (int)n_balls, ist, span, dbx, dby, dbz, dbr,
                         strict, g, (int)n, kout, sx, sy, sz, vout, icnt, nullptr, nullptr);
            HALMA_TRY(exclusive_sum_i64(at<void>(ib, o_itmp), exclusive_sum_i64_bytes(NI), icnt, ioff, nitem, st));
        }
        HALMA_LAUNCH(bg_sphere_off_kernel, grid_for(n_balls + 1, 256), 256, 0, st, (int)n_balls, nitem, ist, ioff, icnt,
                     offs);
        HALMA_CUDA(cudaMemcpyAsync(&total, offs + n_balls, 8, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        *n_found = total;
        if (offsets) HALMA_CUDA(cudaMemcpyAsync(offsets, offs, 8ull * (n_balls + 1), cudaMemcpyDefault, st));
        if (indices && total > 0) {
            if (total > capacity) {
                HALMA_CUDA(cudaStreamSynchronize(st));
                return fail(HALMA_ERR_CAPACITY, "%lld particles found, capacity %lld", (long long)total,
                            (long long)capacity);
            }
            if (total >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "more than 2^31-2 particles found");
            const int eb = 32 + bits_of((uint64_t)n_balls);
            const size_t sk = sort_keys_u64_bytes((int)total, eb);
            Layout F;
            const size_t o_a = F.add(8ull * total), o_b = F.add(8ull * total), o_i = F.add(4ull * total),
                         o_t = F.add(sk);
            void *fb = nullptr;
            HALMA_TRY(workspace(F.total, &fb, st, 8));
            auto *ka = at<uint64_t>(fb, o_a), *kb = at<uint64_t>(fb, o_b);
            int *di = is_device_pointer(indices) ? indices : at<int>(fb, o_i);
            HALMA_LAUNCH(bg_item_kernel<true>, gi, 256, 0, st, nitem, (int)n_balls, ist, span, dbx, dby, dbz, dbr,
                         strict, g, (int)n, kout, sx, sy, sz, vout, nullptr, ioff, ka);
            HALMA_TRY(sort_keys_u64(at<void>(fb, o_t), sk, ka, kb, (int)total, eb, st));
            HALMA_LAUNCH(bg_extract_kernel, std::min(sms * 8, grid_for(total, 256)), 256, 0, st, total, kb, di);
            if (di != indices) HALMA_CUDA(cudaMemcpyAsync(indices, di, 4ull * total, cudaMemcpyDeviceToHost, st));
        }
    } else if (offsets) {
        std::vector<int64_t> z0(n_balls + 1, 0);
        HALMA_CUDA(cudaMemcpyAsync(offsets, z0.data(), 8ull * (n_balls + 1), cudaMemcpyDefault, st));
    }
    HALMA_CUDA(cudaStreamSynchronize(st));
    return HALMA_OK;
}
