// Friends-of-friends on the GPU: the C ABI that replaces python_scripts/fof.py:18-79.
//
// Pipeline (all on one stream):
//   1. bounding box (FP64) -> host picks the cell geometry (cell side = ll * (1 + 2^-20));
//   2. each particle gets a row-major cell key; keys are radix-sorted with their indices;
//   3. per sorted particle: a float4 record (position inside its cell in units of ll, and
//      the original index), run heads of equal keys -> cell table -> per cell the first
//      positions and counts of its 13 forward neighbour cells, found by lower bounds in the
//      sorted cell keys (the key grid is padded so that a neighbour key is a constant offset);
//   4. work items = 32-particle chunks of a cell; one warp per item tests its particles
//      against the same cell and the 13 neighbour cells that sort after it, staging each
//      neighbour chunk in shared memory (coalesced float4 loads, broadcast reads);
//   5. a pair whose float32 distance is clearly inside (outside) the linking length is
//      accepted (rejected); pairs in a +-1e-5 band are re-tested with the exact FP64
//      predicate ((dx*dx + dy*dy) + dz*dz) <= ll*ll, every operation rounded on its own;
//   6. accepted pairs join a lock-free union-find over sorted positions (atomicCAS hooks
//      the larger root under the smaller one, path halving on every find);
//   7. each component's label = the smallest ORIGINAL index among its members
//      (atomicMin), -1 for particles that never linked.
// The result is the reference's partition exactly: same components, same canonical labels.
#include <math.h>
#include <limits.h>
#include <string.h>

#include "common.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {

namespace {

constexpr int kFofWarps = 8;
constexpr int kUfCapDefault = 1 << 26;   // bound on any union-find loop (never reached in practice)
// The bound the kernels use: halma_set_union_find_cap changes it (a debug knob, so that tests
// can make the loops run out); pushed to each device before its next FoF.
__constant__ int c_uf_cap = kUfCapDefault;

struct FofGeom {
    double xmin, ymin, zmin;
    double cell, inv_cell, inv_scale, r2;
    float cs, lo, hi;
    long long ncx, ncy, ncz;
    // key dimensions: ncy + 1 and ncz + 1.  Every y-row and z-column of the key grid ends in an
    // empty pad cell, so that a neighbour's key is the cell's key plus a constant that never
    // wraps onto an occupied cell (a wrap lands on a pad cell or past the last slab)
    long long ky, kz;
    int sb;   // low key bits holding the 4 x 4 x 4 sub-cell (Morton order) within the cell: 6 or 0
};

// Segmented FoF (links only inside a segment): every segment gets its own origin (the
// minimum corner of its bounding box) and its own run of x columns of one virtual cell grid,
// followed by an empty column, so that a cell's forward neighbours are either cells of the
// same segment or empty.  All pointers are null for a plain FoF.
struct SegGeom {
    const int *seg_of = nullptr;       // segment of each particle
    const double *smin = nullptr;      // [3 * nseg] origin of each segment
    const long long *scol = nullptr;   // [4 * nseg] first virtual x column, columns in x, y, z
};

__device__ __forceinline__ int uf_find(int *parent, int v, int *err) {
    int p = __ldcg(parent + v);
    int guard = 0;
    const int cap = c_uf_cap;
    while (p != v) {
        const int gp = __ldcg(parent + p);
        if (gp != p) __stcg(parent + v, gp);   // path halving: gp is an ancestor of v
        v = p;
        p = gp;
        if (++guard > cap) {
            atomicOr(err, 1);
            break;
        }
    }
    return v;
}

// The cached walk below, continued from p = parent[v] loaded earlier (so that the caller can
// issue that load next to other independent ones).
__device__ __forceinline__ int uf_find_from(int *parent, int v, int p, int *err) {
    int guard = 0;
    const int cap = c_uf_cap;
    while (p != v) {
        const int gp = parent[p];
        if (gp != p) __stcg(parent + v, gp);
        v = p;
        p = gp;
        if (++guard > cap) {
            atomicOr(err, 1);
            break;
        }
    }
    return v;
}

// Same walk with L1-cached loads, for the linking kernel.  A value read from L1 may be older
// than the one in L2 (another SM hooked or compressed since), which is harmless there: an
// older parent is still an ancestor (parents only move toward the root, and every value in a
// chain is smaller than the last), equal roots still prove the same set, and any hook goes
// through an atomicCAS on L2 that sees the current value.  The final labels are read by a
// later kernel.
__device__ __forceinline__ int uf_find_cached(int *parent, int v, int *err) {
    int p = parent[v];
    int guard = 0;
    const int cap = c_uf_cap;
    while (p != v) {
        const int gp = parent[p];
        if (gp != p) __stcg(parent + v, gp);
        v = p;
        p = gp;
        if (++guard > cap) {
            atomicOr(err, 1);
            break;
        }
    }
    return v;
}

// Joins the sets of two ancestors a and b (roots or not): hooks the larger root under the
// smaller, retrying from the current roots when the CAS finds that a is no longer a root.
// Every root of a tree is its smallest sorted position.  Returns the node hooked under (or
// the common root when the two are one set already): an ancestor of every member of both
// sets, which the caller may use in place of a fresh find.
__device__ __forceinline__ int uf_union(int *parent, int a, int b, int *err) {
    int guard = 0;
    const int cap = c_uf_cap;
    while (a != b) {
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(parent + a, a, b);
        if (old == a) return b;
        a = uf_find(parent, old, err);
        b = uf_find(parent, b, err);
        if (++guard > cap) {
            atomicOr(err, 1);
            return b;
        }
    }
    return a;
}

// Doubles as order-preserving signed 64-bit integers (sign-magnitude turned into two's
// complement), so that a bounding box is integer min / max: GB300 issues FP64 instructions at
// a small fraction of its integer rate.  -0.0 orders just below +0.0; NaN and infinities are
// flagged separately.
__device__ __forceinline__ long long ord_of(double v) {
    const long long u = __double_as_longlong(v);
    return u ^ ((u >> 63) & 0x7fffffffffffffffll);
}

__device__ __forceinline__ double val_of(long long k) {
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

__device__ __forceinline__ bool nonfinite(double v) {
    return (__double_as_longlong(v) & 0x7ff0000000000000ll) == 0x7ff0000000000000ll;
}

// part[7 * block + q]: the block's min x, y, z and max x, y, z as order keys, and a non-finite flag.
__global__ void bbox_partial_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                    const double *__restrict__ z, int n, long long *__restrict__ part) {
    long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    bool bad = false;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            bad |= nonfinite(v[d]);
            const long long k = ord_of(v[d]);
            mn[d] = min(mn[d], k);
            mx[d] = max(mx[d], k);
        }
    }
    __shared__ long long sh[7][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long vals[7] = {mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], __any_sync(0xffffffffu, bad) ? 1ll : 0ll};
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        long long v = vals[q];
        for (int o = 16; o > 0; o >>= 1) {
            const long long u = __shfl_down_sync(0xffffffffu, v, o);
            v = (q < 3) ? min(v, u) : max(v, u);
        }
        if (lane == 0) sh[q][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        const int q = threadIdx.x;
        long long v = sh[q][0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) v = (q < 3) ? min(v, sh[q][k]) : max(v, sh[q][k]);
        part[blockIdx.x * 7 + q] = v;
    }
}

// One block of 256 threads: the g partial boxes strided over the threads, then a tree; out =
// min x, y, z, max x, y, z as doubles and 1.0 if any coordinate is not finite.
__global__ void __launch_bounds__(256) bbox_final_kernel(const long long *__restrict__ part, int g,
                                                         double *__restrict__ out) {
    __shared__ long long sh[7][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long v[7];
#pragma unroll
    for (int q = 0; q < 7; ++q) v[q] = q < 3 ? LLONG_MAX : LLONG_MIN;
    for (int k = threadIdx.x; k < g; k += blockDim.x)
#pragma unroll
        for (int q = 0; q < 7; ++q) v[q] = q < 3 ? min(v[q], part[k * 7 + q]) : max(v[q], part[k * 7 + q]);
#pragma unroll
    for (int q = 0; q < 7; ++q) {
        for (int o = 16; o > 0; o >>= 1) {
            const long long u = __shfl_down_sync(0xffffffffu, v[q], o);
            v[q] = q < 3 ? min(v[q], u) : max(v[q], u);
        }
        if (lane == 0) sh[q][w] = v[q];
    }
    __syncthreads();
    if (threadIdx.x < 7) {
        const int q = threadIdx.x;
        long long r = sh[q][0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) r = q < 3 ? min(r, sh[q][k]) : max(r, sh[q][k]);
        out[q] = q < 6 ? val_of(r) : (r ? 1.0 : 0.0);
    }
}

// floor(t) and the value t - 4 * floor(t / 4) of a double t, clamped to [0, qmax], from the
// double's bits with integer operations only: a particle's cell and sub-cell come from one FMA
// per axis, and the rest of the conversion (double to integer, the remainder, the float in-cell
// coordinate) would otherwise be half a dozen more FP64-pipe instructions per axis -- the
// kernel's bound on GB300, whose FP64 rate is a small fraction of its integer rate.  The
// remainder w (quarter cells, in [0, 4) away from the grid's edges) is truncated to 24
// significant bits, an error below 1e-7 of a cell: far inside the +-1e-5 band whose pairs are
// re-tested in FP64.
__device__ __forceinline__ void quarter_split(double t, long long qmax, long long &q, float &w) {
    const long long bits = __double_as_longlong(t);
    if (bits <= 0) {   // +0.0 or negative (the sign bit makes the pattern negative)
        q = 0;
        w = 0.f;
        return;
    }
    const int e = (int)((bits >> 52) & 0x7ff) - 1023;
    const unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffll) | (1ull << 52);
    if (e < 0) {   // t < 1: the float with the double's exponent and top mantissa bits
        q = 0;
        w = e + 127 > 0 ? __int_as_float(((e + 127) << 23) | (int)((m >> 29) & 0x7fffff)) : 0.f;
        return;
    }
    if (e > 52) {   // no fraction bits (cell grids beyond 2^51 quarter cells on an axis)
        const long long qq = e - 52 < 10 ? (long long)(m << (e - 52)) : LLONG_MAX;
        q = min(qq, qmax);
        w = (float)(qq - ((q >> 2) << 2));
        return;
    }
    const int sh = 52 - e;
    const long long qq = (long long)(m >> sh);
    q = min(qq, qmax);
    // remainder as a fixed-point number with sh fraction bits, then its top 24 bits as a float
    const unsigned long long v = ((unsigned long long)(qq - ((q >> 2) << 2)) << sh) | (m & ((1ull << sh) - 1));
    if (v == 0) {
        w = 0.f;
        return;
    }
    const int lz = __clzll((long long)v);
    const int fe = (63 - lz) - sh + 127;   // biased exponent of v * 2^-sh
    w = fe > 0 ? __int_as_float((fe << 23) | (int)(((v << lz) >> 40) & 0x7fffff)) : 0.f;
}

// floor(x * s4 * 2^24) + B exactly, with integer operations only (s4 = S * 2^(es - 52) a
// positive double with 53-bit mantissa S): the product of the two 53-bit mantissas as a 128-bit
// integer, shifted to 24 fraction bits and floored (towards -inf for negative x).  A map that
// is exact to 2^-24 quarter cells and monotone in x, for callers that keep |x * s4| and |B|
// below 2^37 quarter cells.
__device__ __forceinline__ long long fixed_quarter(double x, unsigned long long S, int es, long long B) {
    const long long bits = __double_as_longlong(x);
    int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long X = (unsigned long long)(bits & 0xfffffffffffffll);
    if (ex == 0)
        ex = 1;   // zero or subnormal: no implicit bit
    else
        X |= 1ull << 52;
    const unsigned long long lo = X * S, hi = __umul64hi(X, S);
    const int sh = 80 - (ex - 1023) - es;   // (X * S) * 2^-sh = x * s4 * 2^24
    unsigned long long mag;
    bool rem;
    if (sh <= 0) {   // outside the callers' range: saturate
        mag = 1ull << 62;
        rem = false;
    } else if (sh < 64) {
        mag = (hi << (64 - sh)) | (lo >> sh);
        rem = (lo & ((1ull << sh) - 1)) != 0;
    } else if (sh < 128) {
        mag = hi >> (sh - 64);
        rem = lo != 0 || (hi & ((1ull << (sh - 64)) - 1)) != 0;
    } else {
        mag = 0;
        rem = (hi | lo) != 0;
    }
    const long long p = bits < 0 ? -(long long)mag - (rem ? 1 : 0) : (long long)mag;
    return p + B;
}

// quarter_split for a fixed-point t (24 fraction bits): floor(t) clamped to [0, qmax] and the
// remainder t - 4 * floor(t / 4) as a float truncated to 24 significant bits.
__device__ __forceinline__ void quarter_split_fixed(long long t, long long qmax, long long &q, float &w) {
    if (t < 0) {
        q = 0;
        w = 0.f;
        return;
    }
    q = min(t >> 24, qmax);
    const unsigned long long v = (unsigned long long)(t - ((q >> 2) << 26));
    if (v == 0) {
        w = 0.f;
        return;
    }
    const int lz = __clzll((long long)v);
    const int fe = (63 - lz) - 24 + 127;   // biased exponent of v * 2^-24
    w = __int_as_float((fe << 23) | (int)(((v << lz) >> 40) & 0x7fffff));
}

// Sort key: row-major cell index, then (when there is room) the particle's 4 x 4 x 4 sub-cell in
// Morton order, so that each 32-particle chunk of a crowded cell is spatially compact.  The
// order of particles inside a cell does not change the partition.  The kernel also writes the
// particle's position inside its cell in units of the linking length (pre[i], in input order,
// with the index in .w), so that the sorted records are one 16-byte gather.
//
// Cell coordinates: t = 4 * (x - origin) / cell is evaluated as one FMA, x * (4 / cell) -
// origin * (4 / cell); the cell is floor(t) >> 2 and the sub-cell floor(t) & 3.  Any rounding
// here is harmless as long as it is the same for every particle: the cell side is
// ll * (1 + 2^-20), so two points within ll of each other stay in the same or adjacent cells
// whenever the cell coordinate's error is below 2^-21 cells (it is ~1e-12 cells).
//
// FIXED (plain FoF on coordinates and grids within 2^37 quarter cells): the quarter-cell
// coordinate is the exact integer map fixed_quarter instead of the FP64 FMA, so that the
// kernel issues no FP64 instruction at all (with three FMAs a particle it was FP64-bound:
// ncu showed the FP64 pipe 78 % busy).  Both maps are consistent over all particles, which is
// all the cell assignment needs; B = floor(-origin * (4 / cell) * 2^24) per axis.
template <bool FIXED>
__global__ void keys_kernel(const double *__restrict__ x, const double *__restrict__ y,
                            const double *__restrict__ z, int n, FofGeom g, SegGeom sg, long long Bx, long long By,
                            long long Bz, uint64_t *__restrict__ keys, int *__restrict__ vals,
                            float4 *__restrict__ pre) {
    const double s4 = 4.0 * g.inv_cell;   // exact: a power-of-two scaling
    const float cs4 = 0.25f * g.cs;
    const double bx0 = -g.xmin * s4, by0 = -g.ymin * s4, bz0 = -g.zmin * s4;
    const long long s4bits = __double_as_longlong(s4);
    const unsigned long long S4 = (unsigned long long)(s4bits & 0xfffffffffffffll) | (1ull << 52);
    const int es4 = (int)((s4bits >> 52) & 0x7ff) - 1023;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double bx = bx0, by = by0, bz = bz0;   // -origin * (4 / cell)
        long long x0 = 0, nx = g.ncx, ny = g.ncy, nz = g.ncz;
        if (sg.seg_of) {
            const int s = sg.seg_of[i];
            bx = -sg.smin[3 * s] * s4;
            by = -sg.smin[3 * s + 1] * s4;
            bz = -sg.smin[3 * s + 2] * s4;
            x0 = sg.scol[4 * s];
            nx = sg.scol[4 * s + 1];
            ny = sg.scol[4 * s + 2];
            nz = sg.scol[4 * s + 3];
        }
        // quarter-cell coordinates, clamped to the grid (rounding can put a point on the
        // grid's edge a hair outside it), and the position inside the cell in quarter cells
        long long qx, qy, qz;
        float wx, wy, wz;
        if (FIXED) {
            quarter_split_fixed(fixed_quarter(x[i], S4, es4, Bx), 4 * nx - 1, qx, wx);
            quarter_split_fixed(fixed_quarter(y[i], S4, es4, By), 4 * ny - 1, qy, wy);
            quarter_split_fixed(fixed_quarter(z[i], S4, es4, Bz), 4 * nz - 1, qz, wz);
        } else {
            quarter_split(fma(x[i], s4, bx), 4 * nx - 1, qx, wx);
            quarter_split(fma(y[i], s4, by), 4 * ny - 1, qy, wy);
            quarter_split(fma(z[i], s4, bz), 4 * nz - 1, qz, wz);
        }
        const long long cx = qx >> 2, cy = qy >> 2, cz = qz >> 2;
        uint64_t key = ((uint64_t)(x0 + cx) * (uint64_t)g.ky + (uint64_t)cy) * (uint64_t)g.kz + (uint64_t)cz;
        if (g.sb) {
            const int sx = (int)(qx & 3), sy = (int)(qy & 3), sz = (int)(qz & 3);
            const int mort = ((sx >> 1) << 5) | ((sy >> 1) << 4) | ((sz >> 1) << 3) | ((sx & 1) << 2) |
                             ((sy & 1) << 1) | (sz & 1);
            key = (key << 6) | (uint64_t)mort;
        }
        keys[i] = key;
        vals[i] = i;
        pre[i] = make_float4(wx * cs4, wy * cs4, wz * cs4, __int_as_float(i));
    }
}

// Sorted records, run heads, union-find / label initialisation.
// Sorted records, cell heads and label slots.  With runstart (sub-cells in the key), the
// sub-cell runs' starts for the run-head scan (see subrun below) instead of the union-find
// initialisation, which preunion_kernel then writes.
__global__ void prep_kernel(int n, int sb, const uint64_t *__restrict__ keys, const int *__restrict__ idx,
                            const float4 *__restrict__ pre, float4 *__restrict__ rec, int *__restrict__ head,
                            int *__restrict__ parent, unsigned char *__restrict__ has, int *__restrict__ minidx,
                            int *__restrict__ runstart) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint64_t full = keys[k], prev = k > 0 ? keys[k - 1] : ~full;
        rec[k] = pre[idx[k]];
        head[k] = (k == 0 || (prev >> sb) != (full >> sb)) ? 1 : 0;
        if (runstart) {
            runstart[k] = (k == 0 || prev != full) ? k : 0;
        } else {
            parent[k] = k;
            has[k] = 0;
        }
        minidx[k] = INT_MAX;
    }
}

// Particles with the same full key (cell and 4 x 4 x 4 sub-cell) lie at most sqrt(3)/4 of a
// cell (0.44 LL) apart, so they are friends whatever the rounding: each such run is joined
// up front, every member under the run's first sorted position (which keeps "a root is the
// smallest position of its tree").  runstart[k] = k at a run's first position, else 0
// (prep_kernel); an inclusive max-scan turns it into the run head of every position.

__global__ void preunion_kernel(int n, const uint64_t *__restrict__ keys, const int *__restrict__ runhead,
                                int *__restrict__ parent, unsigned char *__restrict__ has) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        parent[k] = runhead[k];
        const bool friend_before = k > 0 && keys[k - 1] == keys[k];
        const bool friend_after = k + 1 < n && keys[k + 1] == keys[k];
        has[k] = (friend_before || friend_after) ? 1 : 0;
    }
}

// Dense cells (>= kDenseMin particles): the occupied 4 x 4 x 4 sub-cells of a cell (side
// cell/4) are joined without pair tests when every pair of their points is closer than the
// linking length: for a sub-cell offset d, the largest distance is sqrt(sum_i (|d_i|+1)^2)/4
// cells, and offsets with sum_i (|d_i|+1)^2 <= 15 stay below 0.97 LL (the rounding of the
// sub-cell assignment moves a point by ~1e-8 cells at most).  One warp per dense cell finds
// the components of its occupied sub-cells under those offsets (bitmask flood fill, see
// subcell_dilate), hooks every run head under the smallest run head of its component (a
// smaller sorted position, so a root stays the smallest position of its tree), marks the
// particles of multi-particle components as having friends, and records whether the whole
// cell is one component (conn[c]).  Smaller cells are connected when all their particles
// share one run.
constexpr int kDenseMin = 32;

__device__ __forceinline__ int lower_bound_key(const uint64_t *__restrict__ keys, int lo, int hi, uint64_t k) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Cells of fewer than kDenseMin particles, one thread each: one component when the first and
// last particles share a sub-cell run; the dense cells are listed for dense_cell_kernel (the
// list order does not matter: each dense cell only joins runs of its own).
__global__ void small_cell_kernel(const int *__restrict__ ncell_p, const int *__restrict__ cell_start,
                                  const uint64_t *__restrict__ keys, unsigned char *__restrict__ conn,
                                  int *__restrict__ dense, int *__restrict__ ndense) {
    const int nc = *ncell_p;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int cs = cell_start[c], ce = cell_start[c + 1];
        if (ce - cs < kDenseMin) conn[c] = keys[cs] == keys[ce - 1] ? 1 : 0;
        else dense[atomicAdd(ndense, 1)] = c;
    }
}

// Sub-cell sets as 64-bit masks, bit 16 x + 4 y + z for sub-cell (x, y, z).  subcell_dilate
// adds every sub-cell within the guaranteed-link offsets of the set: the 3 x 3 x 3 cube, and
// +-2 along one axis with at most one of the other two offsets +-1 ((3,2,2) gives 17 > 15).
__device__ __forceinline__ unsigned long long subcell_dilate(unsigned long long m) {
    constexpr unsigned long long Z0 = 0x1111111111111111ull, Z1 = Z0 << 1, Z2 = Z0 << 2, Z3 = Z0 << 3;
    constexpr unsigned long long Y0 = 0x000F000F000F000Full, Y1 = Y0 << 4, Y2 = Y0 << 8, Y3 = Y0 << 12;
    const unsigned long long zl = ((m << 1) & ~Z0) | ((m >> 1) & ~Z3);   // z +- 1
    const unsigned long long yl = ((m << 4) & ~Y0) | ((m >> 4) & ~Y3);   // y +- 1
    const unsigned long long xl = (m << 16) | (m >> 16);                 // x +- 1
    const unsigned long long a = m | zl;
    const unsigned long long b = a | ((a << 4) & ~Y0) | ((a >> 4) & ~Y3);
    const unsigned long long cube = b | (b << 16) | (b >> 16);
    const unsigned long long cyz = a | yl, cxz = a | xl, cxy = m | xl | yl;   // plus shapes
    return cube | (cyz << 32) | (cyz >> 32) | ((cxz << 8) & ~(Y0 | Y1)) | ((cxz >> 8) & ~(Y2 | Y3)) |
           ((cxy << 2) & ~(Z0 | Z1)) | ((cxy >> 2) & ~(Z2 | Z3));
}

// Bit of Morton sub-cell code m (x1 y1 z1 x0 y0 z0) in the mask layout.
__device__ __forceinline__ int subcell_bit(int m) {
    const int x = (((m >> 5) & 1) << 1) | ((m >> 2) & 1), y = (((m >> 4) & 1) << 1) | ((m >> 1) & 1),
              z = (((m >> 3) & 1) << 1) | (m & 1);
    return (x << 4) | (y << 2) | z;
}

__global__ void __launch_bounds__(256) dense_cell_kernel(const int *__restrict__ ndense_p, const int *__restrict__ dense,
                                                         const int *__restrict__ cell_start,
                                                         const uint64_t *__restrict__ keys, int *__restrict__ parent,
                                                         unsigned char *__restrict__ has, unsigned char *__restrict__ conn) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nd = *ndense_p;
    const int warps = gridDim.x * (blockDim.x >> 5);
    const int bit0 = subcell_bit(lane), bit1 = subcell_bit(lane + 32);
    for (int di = blockIdx.x * (blockDim.x >> 5) + w; di < nd; di += warps) {
        const int c = dense[di];
        const int cs = cell_start[c], ce = cell_start[c + 1];
        const uint64_t ck = keys[cs] & ~63ull;   // the cell's key with the sub-cell bits cleared
        int lo[2], hi[2];
        bool occ[2];
        for (int r = 0; r < 2; ++r) {
            const int m = lane + 32 * r;
            lo[r] = lower_bound_key(keys, cs, ce, ck | (uint64_t)m);
            hi[r] = lower_bound_key(keys, lo[r], ce, (ck | (uint64_t)m) + 1);
            occ[r] = hi[r] > lo[r];
        }
        const unsigned long long mine = (occ[0] ? 1ull << bit0 : 0ull) | (occ[1] ? 1ull << bit1 : 0ull);
        const unsigned long long occm =
            (unsigned long long)__reduce_or_sync(0xffffffffu, (unsigned)mine) |
            ((unsigned long long)__reduce_or_sync(0xffffffffu, (unsigned)(mine >> 32)) << 32);
        unsigned long long rem = occm;
        bool first = true, one = false;
        while (rem) {   // one component per round, from its lowest remaining sub-cell (warp-uniform)
            unsigned long long comp = rem & (~rem + 1ull);
            for (;;) {
                const unsigned long long grown = subcell_dilate(comp) & occm;
                if (grown == comp) break;
                comp = grown;
            }
            if (first) one = comp == occm;
            first = false;
            rem &= ~comp;
            const bool in0 = occ[0] && ((comp >> bit0) & 1ull), in1 = occ[1] && ((comp >> bit1) & 1ull);
            // the component's smallest run head (sorted positions grow with the Morton code)
            const int L = __reduce_min_sync(0xffffffffu, in0 ? lo[0] : (in1 ? lo[1] : INT_MAX));
            const bool multi = (comp & (comp - 1ull)) != 0;
            for (int r = 0; r < 2; ++r) {
                if (!(r == 0 ? in0 : in1)) continue;
                if (L != lo[r]) parent[lo[r]] = L;   // run head under the component's smallest run head
                if (multi || hi[r] - lo[r] > 1)
                    for (int q = lo[r]; q < hi[r]; ++q) has[q] = 1;
            }
        }
        if (lane == 0) conn[c] = one ? 1 : 0;
    }
}

// Start and key of every occupied cell (cells in sorted order), from the exclusive scan of
// the run heads.
__global__ void cell_table_kernel(int n, int sb, const uint64_t *__restrict__ keys, const int *__restrict__ head,
                                  const int *__restrict__ cellpos, int *__restrict__ cell_start,
                                  uint64_t *__restrict__ cell_key, int *__restrict__ ncell) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (head[k]) {
            const int c = cellpos[k];
            cell_start[c] = k;
            cell_key[c] = keys[k] >> sb;
        }
        if (k == n - 1) {
            const int m = cellpos[k] + head[k];
            *ncell = m;
            cell_start[m] = n;
        }
    }
}

// Marks the first particle of every 32-particle chunk of every cell that has linking work
// (bit 13 of its neighbour mask, see nbmask_kernel).
__global__ void itemflag_kernel(int n, const int *__restrict__ head, const int *__restrict__ cellpos,
                                const int *__restrict__ cell_start, const int *__restrict__ cmask,
                                int *__restrict__ flag) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int c = cellpos[k] + head[k] - 1;
        flag[k] = ((cmask[c] >> 13) & 1) && ((k - cell_start[c]) & 31) == 0 ? 1 : 0;
    }
}

// A work item as the linking kernel reads it, in one 16-byte load: the chunk's first sorted
// position, the cell's end with the cell's one-component flag in bit 31, and the cell's index
// (its row of the neighbour table).
struct __align__(16) ItemRec {
    int k0, ce_conn, cell, pad;
};

__global__ void items_kernel(int n, const int *__restrict__ head, const int *__restrict__ cellpos,
                             const int *__restrict__ flag, const int *__restrict__ itempos,
                             const int *__restrict__ cell_start, const unsigned char *__restrict__ conn,
                             ItemRec *__restrict__ items, int *__restrict__ nitems) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (flag[k]) {
            const int c = cellpos[k] + head[k] - 1;
            ItemRec r;
            r.k0 = k;
            r.ce_conn = cell_start[c + 1] | (conn[c] ? (int)0x80000000u : 0);
            r.cell = c;
            r.pad = 0;
            items[itempos[k]] = r;
        }
        if (k == n - 1) *nitems = itempos[k] + flag[k];
    }
}

__device__ __forceinline__ bool exact_link(const double *__restrict__ x, const double *__restrict__ y,
                                           const double *__restrict__ z, int i, int j, double r2) {
    // scipy's p = 2 distance: ((dx*dx + dy*dy) + dz*dz) <= r*r, each operation rounded
    const double dx = __dsub_rn(x[i], x[j]);
    const double dy = __dsub_rn(y[i], y[j]);
    const double dz = __dsub_rn(z[i], z[j]);
    double s = __dmul_rn(dx, dx);
    s = __dadd_rn(s, __dmul_rn(dy, dy));
    s = __dadd_rn(s, __dmul_rn(dz, dz));
    return s <= r2;
}

__constant__ int c_stencil[13][3] = {{0, 0, 1},  {0, 1, -1}, {0, 1, 0},  {0, 1, 1},  {1, -1, -1},
                                     {1, -1, 0}, {1, -1, 1}, {1, 0, -1}, {1, 0, 0},  {1, 0, 1},
                                     {1, 1, -1}, {1, 1, 0},  {1, 1, 1}};

// Lower bound of q in the sorted keys[lo, n), searched forward from lo: doubling steps, then
// bisection of the last step.
__device__ __forceinline__ int gallop_lower_bound(const uint64_t *__restrict__ keys, int lo, int n, uint64_t q) {
    if (lo >= n || keys[lo] >= q) return lo;
    int prev = lo;   // keys[prev] < q
    long long cur = (long long)lo + 1, step = 1;
    while (cur < n && keys[cur] < q) {
        prev = (int)cur;
        step <<= 1;
        cur = prev + step;
    }
    int a = prev + 1, b = (int)(cur < n ? cur : n);
    while (a < b) {
        const int mid = (a + b) >> 1;
        if (keys[mid] < q) a = mid + 1;
        else b = mid;
    }
    return a;
}

// The 13 forward neighbours of every cell, found in the sorted cell keys, one thread per cell.
// On the padded key grid a neighbour's key is the cell's key plus a constant, so (0, 0, +1) is
// the next cell or none, and for each of the stencil's four columns (0, 1), (1, -1), (1, 0),
// (1, 1), whose bases increase, one lower bound of the column's z - 1 key -- galloping forward
// from the cell itself, then from the previous column's bound -- gives its three z neighbours
// in order.  nbinfo[13 c + j] = (first sorted position, count | one-component flag << 31) of
// stencil cell j, (0, 0) when it holds no particle; cmask[c] = the 13-bit mask of occupied
// neighbours, and bit 13 when the cell has linking work: an occupied neighbour, or more than
// one particle in a cell that is not one component already.  Cells without work (isolated
// particles, isolated one-component cells) get no work item.
__global__ void nbtab_kernel(const int *__restrict__ ncell_p, const int *__restrict__ cell_start,
                             const uint64_t *__restrict__ cell_key, const unsigned char *__restrict__ conn,
                             long long ky, long long kz, int2 *__restrict__ nbinfo, int *__restrict__ cmask) {
    const int nc = *ncell_p;
    const uint64_t zrow = (uint64_t)kz, slab = (uint64_t)ky * (uint64_t)kz;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const uint64_t key = cell_key[c];
        int2 *row = nbinfo + (int64_t)c * 13;
        int m = 0;
        auto put = [&](int j, int d) {
            int2 v = make_int2(0, 0);
            if (d >= 0) {
                const int s0 = cell_start[d];
                v = make_int2(s0, (cell_start[d + 1] - s0) | (conn[d] ? (int)0x80000000u : 0));
                m |= 1 << j;
            }
            row[j] = v;
        };
        put(0, (c + 1 < nc && cell_key[c + 1] == key + 1) ? c + 1 : -1);
        const uint64_t base[4] = {key + zrow, key + slab - zrow, key + slab, key + slab + zrow};
        int lb = c + 1;
#pragma unroll
        for (int col = 0; col < 4; ++col) {
            lb = gallop_lower_bound(cell_key, lb, nc, base[col] - 1);
            int at_ = lb;
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz) {
                int d = -1;
                if (at_ < nc && cell_key[at_] == base[col] + (uint64_t)(long long)dz) d = at_++;
                put(1 + 3 * col + (dz + 1), d);
            }
        }
        const int count = cell_start[c + 1] - cell_start[c];
        const bool work = m != 0 || (count > 1 && !conn[c]);
        cmask[c] = m | (work ? 1 << 13 : 0);
    }
}

// One warp per item (a chunk of up to 32 particles of one cell).  The candidates of the item
// are the later particles of its own cell (j > k) and every particle of the 13 forward
// neighbour cells; they are concatenated into one list ("segments" 0..12 = stencil cells, 13 =
// the home cell from the chunk start) and walked 32 at a time, so a sparse region costs one
// or two rounds of loads per item instead of one per neighbour cell.  Each candidate is moved
// into the home cell's frame when it is loaded.
//
// Segment of a candidate: the non-empty segments are ranked in lane order (a per-warp table
// maps rank -> segment); in a round, the segments that start inside it set one bit each of a
// start mask (one OR-reduction), and a candidate's rank is the rank of the round's first
// segment plus the starts at or before it.
//
// Pair tests: the candidates that need a test (within reach of the home chunk's bounding box,
// not already in the home chunk's set) are tested one at a time against all home particles,
// or -- when the chunk holds fewer particles than that (sparse cells) -- the home particles
// one at a time against all those candidates.
constexpr int kHomeSeg = 13;

__global__ void __launch_bounds__(256, 6) link_kernel(
    const float4 *__restrict__ rec, const ItemRec *__restrict__ items, const int *__restrict__ nitems_p, int *item_counter, const int2 *__restrict__ nbinfo, FofGeom g,
    const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
    int *parent, unsigned char *has, int *err) {
    __shared__ float4 buf[kFofWarps][32];    // candidates of the round (candidate-major tests)
    __shared__ float4 hbuf[kFofWarps][32];   // home particles of the item (home-major tests)
    __shared__ int rbuf[kFofWarps][32];
    __shared__ int jbuf[kFofWarps][32];
    __shared__ int segtab[kFofWarps][16];    // rank of a non-empty segment -> segment (lane)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int nitems = *nitems_p;
    // items come from a counter: their cost varies by orders of magnitude (dense cores).  The
    // next item's number, its record and its row of the neighbour table (lanes 0..12) are
    // fetched while the current item is processed.
    int nxt = 0;
    if (lane == 0) nxt = atomicAdd(item_counter, 1);
    int item = __shfl_sync(0xffffffffu, nxt, 0);
    int4 ia_next = make_int4(0, 0, 0, 0);
    int2 nb_next = make_int2(0, 0);
    if (item < nitems) {
        ia_next = __ldg(reinterpret_cast<const int4 *>(items + item));
        if (lane < 13) nb_next = __ldg(nbinfo + (int64_t)ia_next.z * 13 + lane);
    }
    if (lane == 0) nxt = atomicAdd(item_counter, 1);
    for (;;) {
        if (item >= nitems) break;
        const int4 ia = ia_next;
        const int2 nbr = nb_next;   // this lane's neighbour cell (lanes 0..12): first position, count | flag
        item = __shfl_sync(0xffffffffu, nxt, 0);
        if (item < nitems) {
            ia_next = __ldg(reinterpret_cast<const int4 *>(items + item));
            if (lane == 0) nxt = atomicAdd(item_counter, 1);
        }
        const int k0 = ia.x;
        const int ce = ia.y & 0x7fffffff;
        const bool home_conn = ia.y < 0;
        const int k = k0 + lane;
        const bool hv = k < ce;
        const float4 hp = hv ? rec[k] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int pk0 = hv ? parent[k] : -1;   // issued with the record; walked further below
        const int hidx = __float_as_int(hp.w);
        const unsigned homes = __ballot_sync(0xffffffffu, hv);
        const int nhome = __popc(homes);
        // lane s < 13 owns stencil cell s, lane 13 the rest of the home cell
        int sjs = 0, sn = 0, soff = 0x15;   // soff: stencil offset + 1 per axis, 2 bits each
        bool sconn = false;                 // the segment's cell is one component
        if (lane < 13) {   // an empty neighbour has count 0
            soff = (c_stencil[lane][0] + 1) | (c_stencil[lane][1] + 1) << 2 | (c_stencil[lane][2] + 1) << 4;
            sjs = nbr.x;
            sn = nbr.y & 0x7fffffff;
            sconn = nbr.y < 0;
        } else if (lane == kHomeSeg && !home_conn) {   // a cell that is one component has no new pair inside
            sjs = k0 + 1;
            sn = ce - sjs;
        }
        // exclusive prefix of the segment lengths over lanes 0..13
        int incl = sn;
        for (int o = 1; o < 16; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        const int spre = incl - sn;
        const int total = __shfl_sync(0xffffffffu, incl, kHomeSeg);
        const bool nonempty = lane <= kHomeSeg && sn > 0;
        const unsigned ne_mask = __ballot_sync(0xffffffffu, nonempty);
        __syncwarp();
        if (nonempty) segtab[w][__popc(ne_mask & lt_mask)] = lane;
        hbuf[w][lane] = hp;
        __syncwarp();
        // bounding box of the home chunk: a candidate farther than the linking length from it
        // cannot link to any home particle
        float bl[3] = {hv ? hp.x : INFINITY, hv ? hp.y : INFINITY, hv ? hp.z : INFINITY};
        float bh[3] = {hv ? hp.x : -INFINITY, hv ? hp.y : -INFINITY, hv ? hp.z : -INFINITY};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                bl[d] = fminf(bl[d], __shfl_xor_sync(0xffffffffu, bl[d], o));
                bh[d] = fmaxf(bh[d], __shfl_xor_sync(0xffffffffu, bh[d], o));
            }
        }
        // the next item's neighbour row, now that its record has arrived
        if (item < nitems && lane < 13) nb_next = __ldg(nbinfo + (int64_t)ia_next.z * 13 + lane);
        int myroot = hv ? uf_find_from(parent, k, pk0, err) : -1;
        int next = 0;
        for (int v0 = 0; v0 < total; v0 = next) {
            next = v0 + 32;
            // rank of the segment holding candidate v0, and the segments starting in this round
            const int rfirst = __popc(__ballot_sync(0xffffffffu, nonempty && spre <= v0)) - 1;
            const int so = spre - v0;
            const unsigned starts =
                __reduce_or_sync(0xffffffffu, (nonempty && so > 0 && so < 32) ? (1u << so) : 0u);
            // a round starting in a neighbour cell that is one component, already in the set of a
            // home chunk that is itself in one set, skips the rest of that cell
            {
                const int seg0 = segtab[w][rfirst];
                const int n0 = __shfl_sync(0xffffffffu, sn, seg0);
                const int js = __shfl_sync(0xffffffffu, sjs, seg0);
                const int end0 = __shfl_sync(0xffffffffu, spre, seg0) + n0;
                if (seg0 < kHomeSeg && n0 >= 16 && __shfl_sync(0xffffffffu, (int)sconn, seg0)) {
                    if (v0 > 0 && hv) myroot = uf_find_cached(parent, k, err);
                    const int r0 = __shfl_sync(0xffffffffu, myroot, 0);
                    if (__all_sync(0xffffffffu, !hv || myroot == r0)) {
                        int rr = -1;
                        if (lane == 0) rr = uf_find_cached(parent, js, err);
                        rr = __shfl_sync(0xffffffffu, rr, 0);
                        if (rr == r0) {
                            next = end0;   // > v0: the loop always moves forward
                            continue;
                        }
                    }
                }
            }
            const int v = v0 + lane;
            bool cv = v < total;
            // candidate v's segment: the round's first segment plus the starts at or before v
            const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);
            const int seg = segtab[w][rfirst + __popc(starts & upto)];
            const int jl = __shfl_sync(0xffffffffu, sjs, seg) + v - __shfl_sync(0xffffffffu, spre, seg);
            const int off = __shfl_sync(0xffffffffu, soff, seg);
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            int rql = -1;
            // the candidates' parents and the home particles' own are loaded next to the
            // candidate records, so that the root walks below start without another round trip
            const int pj = cv ? parent[jl] : -1;
            const int pk = (v0 > 0 && hv) ? parent[k] : -1;
            if (cv) {
                q = rec[jl];
                q.x += (float)((off & 3) - 1) * g.cs;
                q.y += (float)(((off >> 2) & 3) - 1) * g.cs;
                q.z += (float)(((off >> 4) & 3) - 1) * g.cs;
                const float ex = fmaxf(0.f, fmaxf(bl[0] - q.x, q.x - bh[0]));
                const float ey = fmaxf(0.f, fmaxf(bl[1] - q.y, q.y - bh[1]));
                const float ez = fmaxf(0.f, fmaxf(bl[2] - q.z, q.z - bh[2]));
                cv = fmaf(ex, ex, fmaf(ey, ey, ez * ez)) <= g.hi;
            }
            if (!__any_sync(0xffffffffu, cv)) continue;
            // roots of the candidates, found once per round instead of once per hit; a root
            // read here may be outdated by later unions, which is safe: equal roots prove the
            // same set, unequal ones are re-checked by uf_union
            if (cv) rql = uf_find_from(parent, jl, pj, err);
            // pick up unions made by other warps since the last look
            if (v0 > 0 && hv) myroot = uf_find_from(parent, k, pk, err);
            // when every home particle is in one set, candidates already in it need no test
            const int r0 = __shfl_sync(0xffffffffu, myroot, 0);   // lane 0 is always a home particle
            const bool uniform = __all_sync(0xffffffffu, !hv || myroot == r0);
            const bool mine = cv && !(uniform && rql == r0);
            unsigned todo = __ballot_sync(0xffffffffu, mine);
            if (!todo) continue;
            const int jb = seg == kHomeSeg ? jl : ~jl;   // home-cell candidates keep the j > k test
            if (__popc(todo) > nhome) {
                // home-major: each home particle against all candidates of the round
                unsigned hm = homes;
                while (hm) {
                    const int p = __ffs(hm) - 1;
                    hm &= hm - 1;
                    const float4 pp = hbuf[w][p];
                    const int kp = k0 + p;
                    bool hit = false;
                    if (mine) {
                        const float dx = q.x - pp.x, dy = q.y - pp.y, dz = q.z - pp.z;
                        const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        hit = d2 <= g.hi && (jb < 0 || jb > kp);
                        if (hit && d2 >= g.lo) hit = exact_link(x, y, z, __float_as_int(pp.w), __float_as_int(q.w), g.r2);
                    }
                    if (!__any_sync(0xffffffffu, hit)) continue;
                    // the candidates' roots as this round knows them against home particle p's
                    const int rp = __shfl_sync(0xffffffffu, myroot, p);
                    const bool need = hit && rql != rp;
                    const unsigned nm = __ballot_sync(0xffffffffu, need);
                    if (!nm) continue;
                    // one union per distinct candidate root among the lanes that hit
                    const unsigned peers = __match_any_sync(0xffffffffu, need ? rql : ~lane);
                    const bool leader = need && lane == __ffs(peers) - 1;
                    int nr = 0;
                    if (leader) nr = uf_union(parent, rp, rql, err);
                    if (need) has[jb < 0 ? ~jb : jb] = 1;
                    if (lane == p) has[k] = 1;
                    // the joined sets' members now carry the node each union returned
                    unsigned lm = __ballot_sync(0xffffffffu, leader);
                    while (lm) {
                        const int l = __ffs(lm) - 1;
                        lm &= lm - 1;
                        const int old = __shfl_sync(0xffffffffu, rql, l);
                        const int nw = __shfl_sync(0xffffffffu, nr, l);
                        if (myroot == old || myroot == rp) myroot = nw;
                        if (rql == old || rql == rp) rql = nw;
                    }
                }
                continue;
            }
            __syncwarp();
            buf[w][lane] = q;
            rbuf[w][lane] = rql;
            jbuf[w][lane] = jb;
            __syncwarp();
            while (todo) {
                const int t = __ffs(todo) - 1;
                todo &= todo - 1;
                const float4 qq = buf[w][t];
                const int jt = jbuf[w][t];
                const float dx = qq.x - hp.x, dy = qq.y - hp.y, dz = qq.z - hp.z;
                const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                bool hit = hv && d2 <= g.hi && (jt < 0 || jt > k);
                if (hit && d2 >= g.lo) hit = exact_link(x, y, z, hidx, __float_as_int(qq.w), g.r2);
                if (!__any_sync(0xffffffffu, hit)) continue;
                // the candidate's root as this round knows it: refreshed after every union of
                // the round below, without a memory round trip; a root another warp has hooked
                // since is still an ancestor, which uf_union handles
                const int rq = rbuf[w][t];
                const bool need = hit && myroot != rq;
                const unsigned nm = __ballot_sync(0xffffffffu, need);
                if (!nm) continue;
                // one union per distinct root among the home particles that hit: in a crowded
                // cell most of the 32 share one, and their unions would all contend for it
                const unsigned peers = __match_any_sync(0xffffffffu, need ? myroot : ~lane);
                const bool leader = need && lane == __ffs(peers) - 1;
                int nr = 0;
                if (leader) nr = uf_union(parent, myroot, rq, err);
                if (need) has[k] = 1;
                if (lane == __ffs(nm) - 1) has[jt < 0 ? ~jt : jt] = 1;
                // the joined sets' members (home particles, the round's candidates) now carry
                // the node each union returned
                unsigned lm = __ballot_sync(0xffffffffu, leader);
                while (lm) {
                    const int l = __ffs(lm) - 1;
                    lm &= lm - 1;
                    const int old = __shfl_sync(0xffffffffu, myroot, l);
                    const int nw = __shfl_sync(0xffffffffu, nr, l);
                    if (myroot == old || myroot == rq) myroot = nw;
                    if (rql == old || rql == rq) rql = nw;
                }
                rbuf[w][lane] = rql;
                __syncwarp();
            }
        }
    }
}

// Root of every sorted position, and per root the smallest original index of its members.
// Consecutive sorted positions mostly share a root (a cell, a group), so the lanes of a warp
// first take the minimum per distinct root and issue one atomicMin each.  The loop runs the
// same number of rounds on every lane of a warp (blockDim.x is a multiple of 32).
__global__ void root_kernel(int n, const int *__restrict__ idx, int *parent,
                            const unsigned char *__restrict__ has, int *__restrict__ root,
                            int *__restrict__ minidx, int *err) {
    const int lane = threadIdx.x & 31;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k - lane < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int r = -1, v = INT_MAX;
        if (k < n) {
            r = uf_find(parent, (int)k, err);
            root[k] = r;
            if (has[k]) v = idx[k];
        }
        unsigned todo = __ballot_sync(0xffffffffu, v != INT_MAX);
        while (todo) {
            const int rl = __shfl_sync(0xffffffffu, r, __ffs(todo) - 1);
            const bool mine = r == rl && v != INT_MAX;
            const int m = __reduce_min_sync(0xffffffffu, mine ? v : INT_MAX);
            const unsigned grp = __ballot_sync(0xffffffffu, mine);
            if (lane == __ffs(grp) - 1) atomicMin(minidx + rl, m);
            todo &= ~grp;
        }
    }
}

__global__ void label_kernel(int n, const int *__restrict__ idx, const unsigned char *__restrict__ has,
                             const int *__restrict__ root, const int *__restrict__ minidx,
                             int *__restrict__ labels, int *__restrict__ ngroups) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = idx[k];
        const int r = root[k];
        labels[i] = has[k] ? minidx[r] : -1;
        if (has[k] && r == k) atomicAdd(ngroups, 1);
    }
}

int bits_for(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

// --- segmented FoF: per-segment origin and columns -------------------------------------
__global__ void seg_fill_kernel(int nseg, const int64_t *__restrict__ off, int *__restrict__ seg_of) {
    for (int s = blockIdx.x; s < nseg; s += gridDim.x)
        for (int64_t i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) seg_of[i] = s;
}

// One block per segment: its bounding box (sbox[6s..6s+5] = min xyz, max xyz), the largest
// extent over all segments (as the bits of a non-negative double) and a non-finite flag.
__global__ void __launch_bounds__(256) seg_bbox_kernel(int nseg, const int64_t *__restrict__ off,
                                                       const double *__restrict__ x, const double *__restrict__ y,
                                                       const double *__restrict__ z, double *__restrict__ sbox,
                                                       unsigned long long *__restrict__ ext_bits, int *__restrict__ bad) {
    __shared__ long long sh[6][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
        long long mn[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, mx[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
        bool nf = false;
        for (int64_t i = off[s] + threadIdx.x; i < off[s + 1]; i += blockDim.x) {
            const double v[3] = {x[i], y[i], z[i]};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                nf |= nonfinite(v[d]);
                const long long k = ord_of(v[d]);
                mn[d] = min(mn[d], k);
                mx[d] = max(mx[d], k);
            }
        }
        if (__any_sync(0xffffffffu, nf) && lane == 0) atomicOr(bad, 1);
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            for (int o = 16; o > 0; o >>= 1) {
                mn[d] = min(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
                mx[d] = max(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
            }
            if (lane == 0) {
                sh[d][w] = mn[d];
                sh[3 + d][w] = mx[d];
            }
        }
        __syncthreads();
        if (threadIdx.x < 6) {
            const int q = threadIdx.x;
            long long v = sh[q][0];
            for (int k = 1; k < (int)(blockDim.x >> 5); ++k) v = q < 3 ? min(v, sh[q][k]) : max(v, sh[q][k]);
            sh[q][0] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const bool empty = off[s + 1] <= off[s];
            double b[6];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                b[q] = empty ? (q < 3 ? INFINITY : -INFINITY) : val_of(sh[q][0]);
                sbox[6 * (int64_t)s + q] = b[q];
            }
            const double e = empty ? 0.0 : fmax(b[3] - b[0], fmax(b[4] - b[1], b[5] - b[2]));
            if (isfinite(e) && e > 0.0) atomicMax(ext_bits, (unsigned long long)__double_as_longlong(e));
        }
        __syncthreads();
    }
}

// One block: columns of every segment at cell side 1/inv_cell, the first virtual x column of
// each (exclusive prefix of columns + 1 gap), and out = {total columns, max y columns, max z
// columns}.  An empty segment takes one column.
__global__ void __launch_bounds__(1024) seg_cols_kernel(int nseg, const double *__restrict__ sbox, double inv_cell,
                                                        double *__restrict__ smin, long long *__restrict__ scol,
                                                        long long *__restrict__ out) {
    __shared__ long long part[1024];
    __shared__ long long my[1024], mz[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int per = (nseg + nt - 1) / nt;
    const int s0 = min(nseg, t * per), s1 = min(nseg, s0 + per);
    long long sum = 0, ay = 1, az = 1;
    for (int s = s0; s < s1; ++s) {
        const double *b = sbox + 6 * (int64_t)s;
        long long cx = 1, cy = 1, cz = 1;
        if (b[3] >= b[0]) {   // non-empty
            cx = (long long)floor((b[3] - b[0]) * inv_cell) + 1;
            cy = (long long)floor((b[4] - b[1]) * inv_cell) + 1;
            cz = (long long)floor((b[5] - b[2]) * inv_cell) + 1;
            smin[3 * (int64_t)s] = b[0];
            smin[3 * (int64_t)s + 1] = b[1];
            smin[3 * (int64_t)s + 2] = b[2];
        } else {
            smin[3 * (int64_t)s] = smin[3 * (int64_t)s + 1] = smin[3 * (int64_t)s + 2] = 0.0;
        }
        scol[4 * (int64_t)s + 1] = cx;
        scol[4 * (int64_t)s + 2] = cy;
        scol[4 * (int64_t)s + 3] = cz;
        sum += cx + 1;
        ay = max(ay, cy);
        az = max(az, cz);
    }
    part[t] = sum;
    my[t] = ay;
    mz[t] = az;
    __syncthreads();
    if (t == 0) {   // 1024 partial sums: a serial pass is cheap next to the per-segment work
        long long run = 0, by = 1, bz = 1;
        for (int k = 0; k < nt; ++k) {
            const long long v = part[k];
            part[k] = run;
            run += v;
            by = max(by, my[k]);
            bz = max(bz, mz[k]);
        }
        out[0] = run;
        out[1] = by;
        out[2] = bz;
    }
    __syncthreads();
    long long run = part[t];
    for (int s = s0; s < s1; ++s) {
        scol[4 * (int64_t)s] = run;
        run += scol[4 * (int64_t)s + 1] + 1;
    }
}

// Cell side, band and scale for linking length ll; ext = the largest extent (ll == 0 only).
void set_scale(FofGeom &g, double ll, double ext) {
    if (ll > 0.0) {
        g.cell = ll * (1.0 + 0x1p-20);
        g.inv_scale = 1.0 / ll;
        g.lo = 1.0f - 1e-5f;
        g.hi = 1.0f + 1e-5f;
    } else {
        // ll == 0 links coincident points only: every float candidate is re-tested exactly
        g.cell = ext > 0.0 ? ext * 0x1p-16 : 1.0;
        g.inv_scale = 1.0 / g.cell;
        g.lo = -1.0f;
        g.hi = 1e-6f;
    }
    g.inv_cell = 1.0 / g.cell;
    g.cs = (float)(g.cell * g.inv_scale);
    g.r2 = ll * ll;
}

int g_uf_cap_host = kUfCapDefault;   // guarded by api_mutex()
int g_uf_cap_pushed[64];             // value last copied to each device (0 = never)
bool g_uf_cap_init = false;

// Copies the host's union-find cap to the current device when it differs from the last copy.
int push_uf_cap(cudaStream_t st) {
    if (!g_uf_cap_init) {
        for (int &v : g_uf_cap_pushed) v = kUfCapDefault;   // the __constant__ initialiser
        g_uf_cap_init = true;
    }
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return fail(HALMA_ERR_CAPACITY, "device ordinal %d out of range", dev);
    if (g_uf_cap_pushed[dev] != g_uf_cap_host) {
        HALMA_CUDA(cudaMemcpyToSymbolAsync(c_uf_cap, &g_uf_cap_host, sizeof(int), 0, cudaMemcpyHostToDevice, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        g_uf_cap_pushed[dev] = g_uf_cap_host;
    }
    return HALMA_OK;
}

// Keys, sort, cells, links and labels for a geometry whose cell grid is known.
int fof_core(int n, const double *x, const double *y, const double *z, FofGeom g, SegGeom sg, int *labels,
             int64_t *n_groups, cudaStream_t st) {
    g.ky = g.ncy + 1;
    g.kz = g.ncz + 1;
    const long double cells = (long double)g.ncx * g.ky * g.kz;
    if (cells > 4.0e18L)
        return fail(HALMA_ERR_CAPACITY, "cell grid too large (%lld x %lld x %lld cells)", g.ncx, g.ncy, g.ncz);
    const int cell_bits = bits_for((uint64_t)(g.ncx * g.ky * g.kz - 1));
    g.sb = cell_bits <= 58 ? 6 : 0;
    const int end_bit = cell_bits + g.sb;
    const int sms = device_sm_count();

    const size_t sort_b = sort_pairs_u64_i32_bytes(n, end_bit);
    const size_t scan_b = std::max(exclusive_sum_i32_bytes(n), inclusive_max_i32_bytes(n));
    Layout M;
    const size_t o_kin = M.add(8ull * n), o_kout = M.add(8ull * n);
    const size_t o_vin = M.add(4ull * n), o_vout = M.add(4ull * n);
    const size_t o_rec = M.add(16ull * n), o_pre = M.add(16ull * n);
    const size_t o_head = M.add(4ull * n), o_cpos = M.add(4ull * n);
    const size_t o_par = M.add(4ull * n), o_has = M.add(1ull * n), o_root = M.add(4ull * n);
    const size_t o_min = M.add(4ull * n);
    const size_t o_cst = M.add(4ull * (n + 1)), o_ckey = M.add(8ull * n);
    const size_t o_cm = M.add(4ull * n);   // occupied-neighbour mask and work flag per cell
    const size_t o_flag = M.add(4ull * n), o_ipos = M.add(4ull * n);
    const size_t o_items = M.add(sizeof(ItemRec) * (size_t)n);
    const size_t o_cnt = M.add(64), o_conn = M.add(1ull * n);
    const size_t o_dlist = M.add(4ull * ((uint64_t)n / kDenseMin + 1));   // cells of >= kDenseMin particles
    const size_t o_tmp = M.add(std::max(sort_b, scan_b));
    void *base = nullptr;
    HALMA_TRY(push_uf_cap(st));
    HALMA_TRY(workspace(M.total, &base, st));
    auto *kin = at<uint64_t>(base, o_kin), *kout = at<uint64_t>(base, o_kout);
    auto *vin = at<int>(base, o_vin), *vout = at<int>(base, o_vout);
    auto *rec = at<float4>(base, o_rec), *pre = at<float4>(base, o_pre);
    auto *head = at<int>(base, o_head), *cpos = at<int>(base, o_cpos);
    auto *parent = at<int>(base, o_par), *root = at<int>(base, o_root), *minidx = at<int>(base, o_min);
    auto *has = at<unsigned char>(base, o_has);
    auto *cst = at<int>(base, o_cst);
    auto *ckey = at<uint64_t>(base, o_ckey);
    auto *cmask = at<int>(base, o_cm);
    auto *flag = at<int>(base, o_flag), *ipos = at<int>(base, o_ipos);
    auto *items = at<ItemRec>(base, o_items);
    int *cnt = at<int>(base, o_cnt);   // [0] ncell [1] nitems [2] ngroups [3] err [5] link item counter [8] dense cells
    void *tmp = at<void>(base, o_tmp);
    const int g1 = std::min(sms * 8, grid_for(n, 256));

    Profile &prof = profile();
    const bool stages = !sg.seg_of;   // stage times of the plain FoF only
    auto mark = [&](int k) { return stages ? prof.fof_mark(k, st) : HALMA_OK; };
    HALMA_CUDA(cudaMemsetAsync(cnt, 0, 64, st));
    // the integer map when the coordinates and the grid stay within 2^37 quarter cells (plain
    // FoF; the segmented one has per-segment origins and keeps the FP64 map)
    const double s4 = 4.0 * g.inv_cell, lim = 0x1p37;
    const double bxd = -g.xmin * s4, byd = -g.ymin * s4, bzd = -g.zmin * s4;
    double reach = fmax(fabs(g.xmin), fabs(g.xmin + g.cell * (double)g.ncx));
    reach = fmax(reach, fmax(fabs(g.ymin), fabs(g.ymin + g.cell * (double)g.ncy)));
    reach = fmax(reach, fmax(fabs(g.zmin), fabs(g.zmin + g.cell * (double)g.ncz))) * s4;
    const bool fixed = !sg.seg_of && s4 >= 0x1p-1000 && reach < lim && fabs(bxd) < lim && fabs(byd) < lim &&
                       fabs(bzd) < lim;
    if (fixed)
        HALMA_LAUNCH(keys_kernel<true>, g1, 256, 0, st, x, y, z, n, g, sg, (long long)floor(bxd * 0x1p24),
                     (long long)floor(byd * 0x1p24), (long long)floor(bzd * 0x1p24), kin, vin, pre);
    else
        HALMA_LAUNCH(keys_kernel<false>, g1, 256, 0, st, x, y, z, n, g, sg, 0ll, 0ll, 0ll, kin, vin, pre);
    HALMA_TRY(mark(1));
    HALMA_TRY(sort_pairs_u64_i32(tmp, sort_b, kin, kout, vin, vout, n, end_bit, st));
    HALMA_TRY(mark(2));
    const bool runs = g.sb != 0 && g.lo > 0.f;   // sub-cells in the key and a positive linking length
    HALMA_LAUNCH(prep_kernel, g1, 256, 0, st, n, g.sb, kout, vout, pre, rec, head, parent, has, minidx,
                 runs ? flag : nullptr);
    if (runs) {
        HALMA_TRY(inclusive_max_i32(tmp, scan_b, flag, root, n, st));
        HALMA_LAUNCH(preunion_kernel, g1, 256, 0, st, n, kout, root, parent, has);
    }
    HALMA_TRY(mark(3));
    HALMA_TRY(exclusive_sum_i32(tmp, scan_b, head, cpos, n, st));
    HALMA_LAUNCH(cell_table_kernel, g1, 256, 0, st, n, g.sb, kout, head, cpos, cst, ckey, cnt + 0);
    // one-component cells (sub-cells in the key and a positive linking length only)
    unsigned char *conn = at<unsigned char>(base, o_conn);
    int *dlist = at<int>(base, o_dlist);
    if (g.sb != 0 && g.lo > 0.f) {
        HALMA_LAUNCH(small_cell_kernel, g1, 256, 0, st, cnt + 0, cst, kout, conn, dlist, cnt + 8);
        HALMA_LAUNCH(dense_cell_kernel, sms * 8, 256, 0, st, cnt + 8, dlist, cst, kout, parent, has, conn);
    } else {
        HALMA_CUDA(cudaMemsetAsync(conn, 0, n, st));
    }
    // the neighbour table (13 x 8 bytes per occupied cell) in its own cached buffer, sized from
    // the cell count
    int ncell = 0;
    HALMA_CUDA(cudaMemcpyAsync(&ncell, cnt + 0, sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    void *nbbase = nullptr;
    HALMA_TRY(workspace(sizeof(int2) * 13 * (size_t)std::max(ncell, 1), &nbbase, st, 10));
    int2 *nbinfo = static_cast<int2 *>(nbbase);
    HALMA_LAUNCH(nbtab_kernel, std::min(sms * 8, grid_for(ncell, 256)), 256, 0, st, cnt + 0, cst, ckey, conn, g.ky,
                 g.kz, nbinfo, cmask);
    HALMA_TRY(mark(4));
    HALMA_LAUNCH(itemflag_kernel, g1, 256, 0, st, n, head, cpos, cst, cmask, flag);
    HALMA_TRY(exclusive_sum_i32(tmp, scan_b, flag, ipos, n, st));
    HALMA_LAUNCH(items_kernel, g1, 256, 0, st, n, head, cpos, flag, ipos, cst, conn, items, cnt + 1);
    HALMA_TRY(mark(5));
    HALMA_LAUNCH(link_kernel, sms * 8, 32 * kFofWarps, 0, st, rec, items, cnt + 1, cnt + 5, nbinfo, g, x, y, z,
                 parent, has, cnt + 3);
    HALMA_TRY(mark(6));
    // the sorted original indices (4 bytes a position) rather than the records' 16
    HALMA_LAUNCH(root_kernel, g1, 256, 0, st, n, vout, parent, has, root, minidx, cnt + 3);
    HALMA_LAUNCH(label_kernel, g1, 256, 0, st, n, vout, has, root, minidx, labels, cnt + 2);
    HALMA_TRY(mark(7));
    int hc[4];
    HALMA_CUDA(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    if (hc[3]) return fail(HALMA_ERR_NOT_CONVERGED, "union-find iteration cap reached");
    if (n_groups) *n_groups = hc[2];
    return HALMA_OK;
}

}  // namespace

// Bounding box of n > 0 device points, returned on the host: min x, y, z, max x, y, z, and a
// non-zero seventh value if any coordinate is not finite.  Uses workspace slot 0.
int bbox_device(int n, const double *x, const double *y, const double *z, double bb[7], cudaStream_t st) {
    const int gb = std::min(device_sm_count() * 4, grid_for(n, 256));
    Layout L;
    const size_t o_part = L.add(sizeof(double) * 7 * gb);
    const size_t o_out = L.add(sizeof(double) * 8);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    HALMA_LAUNCH(bbox_partial_kernel, gb, 256, 0, st, x, y, z, n, at<long long>(base, o_part));
    HALMA_LAUNCH(bbox_final_kernel, 1, 256, 0, st, at<long long>(base, o_part), gb, at<double>(base, o_out));
    HALMA_CUDA(cudaMemcpyAsync(bb, at<double>(base, o_out), 7 * sizeof(double), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    return HALMA_OK;
}

// Full FoF on device arrays (no staging, no locking); used by halma_fof and the pipeline.
int fof_device(int n, const double *x, const double *y, const double *z, double ll, int *labels,
               int64_t *n_groups, cudaStream_t st) {
    if (n == 0) {
        if (n_groups) *n_groups = 0;
        return HALMA_OK;
    }
    FofGeom g{};
    HALMA_TRY(profile().fof_mark(0, st));
    {
        double bb[7];
        HALMA_TRY(bbox_device(n, x, y, z, bb, st));
        if (bb[6] != 0.0) return fail(HALMA_ERR_INVALID, "non-finite particle position");
        g.xmin = bb[0];
        g.ymin = bb[1];
        g.zmin = bb[2];
        const double ext = std::max(bb[3] - bb[0], std::max(bb[4] - bb[1], bb[5] - bb[2]));
        set_scale(g, ll, ext);
        g.ncx = (long long)floor((bb[3] - bb[0]) * g.inv_cell) + 1;
        g.ncy = (long long)floor((bb[4] - bb[1]) * g.inv_cell) + 1;
        g.ncz = (long long)floor((bb[5] - bb[2]) * g.inv_cell) + 1;
    }
    return fof_core(n, x, y, z, g, SegGeom{}, labels, n_groups, st);
}

// FoF inside segments (particles of segment s are rows off[s] .. off[s+1], off on the
// device): one launch sequence for all segments.  Labels are the smallest row index of each
// component, -1 for rows without a friend in their own segment.  The per-segment geometry
// lives in workspace slot 2, the linking scratch in slot 0.
int fof_segmented_device(int n, int nseg, const int64_t *off, const double *x, const double *y, const double *z,
                         double ll, int *labels, int64_t *n_groups, cudaStream_t st) {
    if (n == 0 || nseg == 0) {
        if (n_groups) *n_groups = 0;
        return HALMA_OK;
    }
    Layout L;
    const size_t o_seg = L.add(4ull * n), o_box = L.add(48ull * nseg), o_min = L.add(24ull * nseg);
    const size_t o_col = L.add(32ull * nseg), o_cnt = L.add(64);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 2));
    int *seg_of = at<int>(base, o_seg);
    double *sbox = at<double>(base, o_box), *smin = at<double>(base, o_min);
    long long *scol = at<long long>(base, o_col);
    unsigned long long *ext_bits = at<unsigned long long>(base, o_cnt);
    int *bad = at<int>(base, o_cnt + 8);
    long long *cols = at<long long>(base, o_cnt + 16);
    const int gs = std::min(nseg, device_sm_count() * 16);
    HALMA_CUDA(cudaMemsetAsync(at<void>(base, o_cnt), 0, 64, st));
    HALMA_LAUNCH(seg_fill_kernel, gs, 256, 0, st, nseg, off, seg_of);
    HALMA_LAUNCH(seg_bbox_kernel, gs, 256, 0, st, nseg, off, x, y, z, sbox, ext_bits, bad);
    long long hc[2];
    HALMA_CUDA(cudaMemcpyAsync(hc, at<void>(base, o_cnt), 16, cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    if ((int)hc[1] != 0) return fail(HALMA_ERR_INVALID, "non-finite particle position");
    double ext;
    memcpy(&ext, &hc[0], 8);
    FofGeom g{};
    set_scale(g, ll, ext);
    HALMA_LAUNCH(seg_cols_kernel, 1, 1024, 0, st, nseg, sbox, g.inv_cell, smin, scol, cols);
    long long cc[3];
    HALMA_CUDA(cudaMemcpyAsync(cc, cols, sizeof(cc), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    g.ncx = cc[0];
    g.ncy = cc[1];
    g.ncz = cc[2];
    SegGeom sg;
    sg.seg_of = seg_of;
    sg.smin = smin;
    sg.scol = scol;
    return fof_core(n, x, y, z, g, sg, labels, n_groups, st);
}

}  // namespace halma

using namespace halma;

extern "C" int halma_set_union_find_cap(int32_t cap) {
    std::lock_guard<std::mutex> guard(api_mutex());
    g_uf_cap_host = cap < 0 ? kUfCapDefault : cap;
    return HALMA_OK;
}

extern "C" int halma_fof(int64_t n, const double *x, const double *y, const double *z, double linking_length,
                         int32_t *labels, int64_t *n_groups, halma_stream_t stream) {
    if (n < 0) return fail(HALMA_ERR_INVALID, "negative particle count");
    if (n >= INT_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles per call");
    if (!(linking_length >= 0.0) || !isfinite(linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and >= 0");
    if (n > 0 && (!x || !y || !z || !labels)) return fail(HALMA_ERR_INVALID, "null pointer");
    if (n == 0) {
        if (n_groups) *n_groups = 0;
        return HALMA_OK;
    }
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr;
    int32_t *dl = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add((const int32_t *)labels, n, false, true, &dl);
    if (sg.any_host) {
        // host arrays live in their own allocation so the FoF scratch can reuse the workspace
        std::vector<void *> owned;
        Layout L;
        sg.plan(L);
        void *stage = nullptr;
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
        int s = sg.bind_and_upload(stage, st);
        if (s == HALMA_OK) s = fof_device((int)n, dx, dy, dz, linking_length, dl, n_groups, st);
        if (s == HALMA_OK) s = sg.download(st);
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
        return s;
    }
    HALMA_TRY(sg.bind_and_upload(nullptr, st));
    return fof_device((int)n, dx, dy, dz, linking_length, dl, n_groups, st);
}

namespace halma {
namespace {

// Members per label (a label is the smallest index of its group), one atomic per distinct
// label among the lanes of a warp: group members are often neighbours in index order.
__global__ void group_count_kernel(int n, const int *__restrict__ labels, int *__restrict__ gsize,
                                   int *__restrict__ bad) {
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        int l = i < n ? labels[i] : -1;
        if (l < -1 || l >= n) {   // not a particle index: reported, counted nowhere
            atomicOr(bad, 1);
            l = -1;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, l);
        if (l >= 0 && lane == __ffs(peers) - 1) atomicAdd(gsize + l, __popc(peers));
    }
}

// Per particle: kept (its group has >= minp members) in the low 32 bits and group head (kept,
// and the smallest index of its group) in the high 32 bits, for one exclusive scan giving every
// kept particle its position among the kept particles and every group its index: the heads
// appear in index order, which is the order of the groups' smallest members.
__global__ void group_flag_kernel(int n, const int *__restrict__ labels, const int *__restrict__ gsize, int minp,
                                  long long *__restrict__ flags) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int l = labels[i];
        const bool keep = l >= 0 && l < n && gsize[l] >= minp;
        flags[i] = keep ? (1ll | (l == i ? 1ll << 32 : 0ll)) : 0ll;
    }
}

// Kept particles in index order, keyed by their group's index; the counts go to cnt[2..3]
// and the member count to offsets[groups].
__global__ void group_scatter_kernel(int n, const int *__restrict__ labels, const long long *__restrict__ flags,
                                     const long long *__restrict__ pre, uint32_t *__restrict__ keys,
                                     int *__restrict__ vals, int *__restrict__ cnt, int64_t *__restrict__ offsets) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long f = flags[i];
        if (f) {
            const int pos = (int)(pre[i] & 0xffffffffll);
            keys[pos] = (uint32_t)(pre[labels[i]] >> 32);   // heads before the group's head
            vals[pos] = i;
        }
        if (i == n - 1) {
            const long long t = pre[i] + f;
            cnt[2] = (int)(t >> 32);
            cnt[3] = (int)(t & 0xffffffffll);
            offsets[t >> 32] = t & 0xffffffffll;
        }
    }
}

// Group offsets from the sorted keys: a group starts where its index first appears.
__global__ void group_offsets_kernel(int nm, const uint32_t *__restrict__ keys, int64_t *__restrict__ offsets) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nm; k += gridDim.x * blockDim.x)
        if (k == 0 || keys[k] != keys[k - 1]) offsets[keys[k]] = k;
}

}  // namespace

// Groups of >= minp members in the reference order, on device arrays: members per label,
// flags and one scan over the particles (position among the kept, group index), the kept
// particles keyed by group index in index order, one stable radix sort over the bits of the
// group count, offsets from the sorted keys.  The counts are returned on the host (one
// synchronisation, before the sort).
int fof_groups_device(int n, const int *labels, int minp, int64_t *offsets, int *members,
                      int64_t *n_groups, int64_t *n_members, cudaStream_t st) {
    const size_t sort_b = sort_pairs_u32_i32_bytes(n);
    const size_t scan_b = exclusive_sum_i64_bytes(n);
    Layout L;
    const size_t o_gsize = L.add(4ull * n), o_flag = L.add(8ull * n), o_pre = L.add(8ull * n);
    const size_t o_kin = L.add(4ull * n), o_kout = L.add(4ull * n), o_vin = L.add(4ull * n);
    const size_t o_cnt = L.add(64), o_tmp = L.add(std::max(sort_b, scan_b));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    auto *gsize = at<int>(base, o_gsize);
    auto *flags = at<long long>(base, o_flag), *pre = at<long long>(base, o_pre);
    auto *kin = at<uint32_t>(base, o_kin), *kout = at<uint32_t>(base, o_kout);
    auto *vin = at<int>(base, o_vin);
    int *cnt = at<int>(base, o_cnt);
    void *tmp = at<void>(base, o_tmp);
    const int g1 = std::min(device_sm_count() * 8, grid_for(n, 256));
    HALMA_CUDA(cudaMemsetAsync(cnt, 0, 64, st));
    HALMA_CUDA(cudaMemsetAsync(gsize, 0, 4ull * n, st));
    HALMA_LAUNCH(group_count_kernel, g1, 256, 0, st, n, labels, gsize, cnt);
    HALMA_LAUNCH(group_flag_kernel, g1, 256, 0, st, n, labels, gsize, std::max(minp, 1), flags);
    HALMA_TRY(exclusive_sum_i64(tmp, scan_b, reinterpret_cast<const int64_t *>(flags),
                                reinterpret_cast<int64_t *>(pre), n, st));
    HALMA_LAUNCH(group_scatter_kernel, g1, 256, 0, st, n, labels, flags, pre, kin, vin, cnt, offsets);
    int hc[4];
    HALMA_CUDA(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    if (hc[0]) return fail(HALMA_ERR_INVALID, "labels must be particle indices in [0, n) or -1");
    const int ng = hc[2], nm = hc[3];
    if (nm > 0) {
        if (ng > 1)
            HALMA_TRY(sort_pairs_u32_i32(tmp, sort_b, kin, kout, vin, members, nm, bits_for((uint64_t)(ng - 1)), st));
        else   // one group: already in order
            HALMA_CUDA(cudaMemcpyAsync(members, vin, 4ull * nm, cudaMemcpyDeviceToDevice, st));
        HALMA_LAUNCH(group_offsets_kernel, std::min(device_sm_count() * 8, grid_for(nm, 256)), 256, 0, st, nm,
                     ng > 1 ? kout : kin, offsets);
    }
    *n_groups = ng;
    if (n_members) *n_members = nm;
    return HALMA_OK;
}

}  // namespace halma

extern "C" int halma_fof_groups(int64_t n, const int32_t *labels, int32_t min_members, int64_t *offsets,
                                int32_t *members, int64_t *n_groups, halma_stream_t stream) {
    if (n < 0) return fail(HALMA_ERR_INVALID, "negative particle count");
    if (n >= INT_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles per call");
    if (!offsets || !n_groups || (n > 0 && (!labels || !members))) return fail(HALMA_ERR_INVALID, "null pointer");
    if (n == 0) {
        *n_groups = 0;
        int64_t zero = 0;
        if (is_device_pointer(offsets)) HALMA_CUDA(cudaMemcpy(offsets, &zero, 8, cudaMemcpyHostToDevice));
        else offsets[0] = 0;
        return HALMA_OK;
    }
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    const bool h_lab = !is_device_pointer(labels), h_off = !is_device_pointer(offsets),
               h_mem = !is_device_pointer(members);
    void *stage = nullptr;
    const int *dl = labels;
    int64_t *doff = offsets;
    int *dmem = members;
    if (h_lab || h_off || h_mem) {
        Layout L;
        const size_t a = L.add(4ull * n), b = L.add(8ull * (n + 1)), c = L.add(4ull * n);
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
        if (h_lab) {
            dl = at<int>(stage, a);
            HALMA_CUDA(cudaMemcpyAsync((void *)dl, labels, 4ull * n, cudaMemcpyHostToDevice, st));
        }
        if (h_off) doff = at<int64_t>(stage, b);
        if (h_mem) dmem = at<int>(stage, c);
    }
    int64_t ng = 0, nm = 0;
    int s = fof_groups_device((int)n, dl, min_members, doff, dmem, &ng, &nm, st);
    if (s == HALMA_OK) {
        if (h_off) s = cudaMemcpyAsync(offsets, doff, 8ull * (ng + 1), cudaMemcpyDeviceToHost, st) == cudaSuccess ? s : fail(HALMA_ERR_CUDA, "copy of group offsets failed");
        if (h_mem && nm > 0) s = cudaMemcpyAsync(members, dmem, 4ull * nm, cudaMemcpyDeviceToHost, st) == cudaSuccess ? s : fail(HALMA_ERR_CUDA, "copy of group members failed");
        *n_groups = ng;
    }
    if (stage) cudaFreeAsync(stage, st);
    cudaStreamSynchronize(st);
    return s;
}
