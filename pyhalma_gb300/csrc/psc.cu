// Phase-space cleaning of all FoF groups at once: pyHALMA's calc_cell / clean_cell
// (python_scripts/halo_properties.py:113-278) inside pyHALMA.py's loop over groups
// (pyHALMA.py:774-843).
//
// Reference, per group (part_list P of N0 particles):
//   grid   = np.arange(-(R+LL), R+LL, 2LL) around the centre of mass, R = furthest particle;
//   cell   = per axis np.argmin(|grid - (x - c)|) (first index on ties);
//   per cell (particles in list order): count q, mass, mass-weighted mean velocity v_c and
//            sigma = sqrt(sum |v_c - v|^2 / 3 / q);
//   sweep  = drop a particle when q <= q_fil, or when |v_c - v| / sigma >= fac_sig * sig_fil
//            (the first sweep divides by sigma only when q > 2 and uses 0 otherwise, later
//            sweeps divide when q >= 2);  a drop writes control[ip] = 0 with ip the particle's
//            position in the list being swept, counts it as cleaned and decrements remaining;
//   loop   = fac_sig = 2, then x0.75 after the first sweep; while cleaned/remaining > 0.1 the
//            sweep repeats on a new grid around P[control != 0] (a pass that leaves remaining
//            == 0 ends the group with zero outputs), fac_sig = max(1, 0.75 fac_sig);
//   final  = grid and cells of P[control != 0] (their cells are the which_cell output);
//   main script = control reset to ones when cleaning is off or N0 < min_part; centre, mass and
//            furthest particle of P[control]; the group is kept when it has >= MINP particles.
//
// Here every step runs for all groups in a fixed set of launches: a group's state (centre,
// grid, fac_sig, cleaned / remaining, mode) lives on the device, the current lists are CSR
// over the groups' member positions, cells are found per particle from the grid formula and
// checked against the neighbouring grid points, and the per-cell sums run one thread per cell
// in list order after a stable radix sort by (group, cell).  The host loop only reads how many
// groups still sweep.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "seqsum.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

enum { kModeNone = 0, kModeSweep = 1, kModeFinal = 2 };

struct PscState {
    double cx, cy, cz, M, rr;
    double start, next, delta, step, inv_step, inv_delta, margin;
    double fac_sig;
    long long n, n0;              // grid points per axis: current, and of the first grid
    long long cleaned, remaining;
    int mode, first, zero, passes;
};

__device__ __forceinline__ double grid_at(const PscState &s, long long i) {
    // numpy.arange: a[0] = start, a[1] = start + step, a[i] = start + i * (a[1] - a[0])
    return i == 0 ? s.start : (i == 1 ? s.next : __dadd_rn(s.start, __dmul_rn((double)i, s.delta)));
}

// The grid points are a[i] = start + i * delta rounded, so t = (v - start) / delta locates v
// among them to within ~3n x 1.1e-16 points.  Unless t lies within `margin` (1e-12 (n + 8),
// thousands of times that error) of a midpoint, the nearest point is t rounded (clamped to the
// grid); otherwise it is decided on the grid's own values: the guess from the reciprocal of the
// step (GB300's FP64 divide is a long sequence) is within one point, and both neighbours are
// checked, ties going to the first index as numpy's argmin.
__device__ __forceinline__ long long nearest(const PscState &s, double v) {
    {
        const double t = (v - s.start) * s.inv_delta, fl = floor(t), f = t - fl;
        if (fabs(f - 0.5) > s.margin) {
            const long long k = (long long)fl + (f > 0.5 ? 1 : 0);
            return k < 0 ? 0 : (k > s.n - 1 ? s.n - 1 : k);
        }
    }
    long long k = (long long)floor((v - s.start) * s.inv_step + 0.5);
    k = k < 0 ? 0 : (k > s.n - 1 ? s.n - 1 : k);
    long long best = k;
    double bd = fabs(__dsub_rn(grid_at(s, k), v));
    for (long long c = k - 1; c <= k + 1; c += 2) {
        if (c < 0 || c >= s.n) continue;
        const double d = fabs(__dsub_rn(grid_at(s, c), v));
        if (d < bd || (d == bd && c < best)) {
            bd = d;
            best = c;
        }
    }
    return best;
}

// List entry -> group (CSR fill).
__global__ void psc_fill_kernel(int G, const int64_t *__restrict__ off, int *__restrict__ owner) {
    for (int h = blockIdx.x; h < G; h += gridDim.x)
        for (int64_t e = off[h] + threadIdx.x; e < off[h + 1]; e += blockDim.x) owner[e] = h;
}

// One block per group whose mode matches: FP64 centre of mass of the list (zeros when the
// mass is not positive), furthest particle from it, and the grid around it.  For the main
// script's own step the results go to the output row instead of the state.
// Centre of mass and furthest particle of every group that sweeps or takes its final step
// (with all, of every group: the main script's final values).  A group's list is split over up to
// S blocks of at least kPscMin entries; each block writes its partial sums, and the last block
// of the group to finish (a counter per group, no waiting) adds them in block order.  The
// furthest particle is the square root of the largest squared distance (the square root is
// correctly rounded and monotone, so this is the largest of the square roots).
constexpr int kPscMin = 2048;

__device__ __forceinline__ bool psc_part_of(int bid, int S, int G, const int64_t *__restrict__ off, int &h, int &sh,
                                            int64_t &b, int64_t &e) {
    h = bid / S;
    const int s = bid % S;
    if (h >= G) return false;
    const int64_t b0 = off[h], len = off[h + 1] - b0;
    sh = (int)std::min<int64_t>(S, std::max<int64_t>(1, (len + kPscMin - 1) / kPscMin));
    if (s >= sh) return false;
    b = b0 + len * s / sh;
    e = b0 + len * (s + 1) / sh;
    return true;
}

__global__ void __launch_bounds__(256) psc_sum_kernel(int G, const int64_t *__restrict__ off,
                                                      const int *__restrict__ list, const int *__restrict__ mem,
                                                      const double *__restrict__ x, const double *__restrict__ y,
                                                      const double *__restrict__ z, const double *__restrict__ m,
                                                      int S, int all, const PscState *__restrict__ st,
                                                      double *__restrict__ part, int *__restrict__ ctr,
                                                      double *__restrict__ cen,
                                                      unsigned long long *__restrict__ rr2) {
    int h, sh;
    int64_t b, e;
    if (!psc_part_of(blockIdx.x, S, G, off, h, sh, b, e)) return;
    if (!all && st[h].mode == kModeNone) return;
    __shared__ double sm[4][8];
    __shared__ int last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double v[4] = {0, 0, 0, 0};
    for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
        const int i = mem[list[k]];
        const double mi = m[i];
        v[0] += mi * x[i];
        v[1] += mi * y[i];
        v[2] += mi * z[i];
        v[3] += mi;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
        if (lane == 0) sm[q][w] = v[q];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int s = blockIdx.x % S;
        for (int q = 0; q < 4; ++q) {
            double t = 0.0;
            for (int k = 0; k < nw; ++k) t += sm[q][k];
            part[((int64_t)h * S + s) * 4 + q] = t;
        }
        __threadfence();
        last = atomicAdd(ctr + h, 1) == sh - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double t[4] = {0, 0, 0, 0};
        for (int s = 0; s < sh; ++s)
            for (int q = 0; q < 4; ++q) t[q] += __ldcg(part + ((int64_t)h * S + s) * 4 + q);
        const double M = t[3];
        cen[4 * h + 0] = M > 0 ? t[0] / M : 0.0;
        cen[4 * h + 1] = M > 0 ? t[1] / M : 0.0;
        cen[4 * h + 2] = M > 0 ? t[2] / M : 0.0;
        cen[4 * h + 3] = M > 0 ? M : 0.0;
        rr2[h] = 0ull;
        ctr[h] = 0;
    }
}

__global__ void __launch_bounds__(256) psc_rmax_kernel(int G, const int64_t *__restrict__ off,
                                                       const int *__restrict__ list, const int *__restrict__ mem,
                                                       const double *__restrict__ x, const double *__restrict__ y,
                                                       const double *__restrict__ z, double ll, int S, int all,
                                                       PscState *st, double *out, int64_t *__restrict__ nwhich,
                                                       int *__restrict__ ctr, const double *__restrict__ cen,
                                                       unsigned long long *__restrict__ rr2) {
    int h, sh;
    int64_t b, e;
    if (!psc_part_of(blockIdx.x, S, G, off, h, sh, b, e)) return;
    if (!all && st[h].mode == kModeNone) return;
    __shared__ double sm[8];
    __shared__ int last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const double cx = cen[4 * h], cy = cen[4 * h + 1], cz = cen[4 * h + 2];
    double r2 = 0.0;
    for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
        const int i = mem[list[k]];
        const double dx = __dsub_rn(cx, x[i]), dy = __dsub_rn(cy, y[i]), dz = __dsub_rn(cz, z[i]);
        r2 = fmax(r2, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    }
    for (int o = 16; o > 0; o >>= 1) r2 = fmax(r2, __shfl_down_sync(0xffffffffu, r2, o));
    if (lane == 0) sm[w] = r2;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < nw; ++k) t = fmax(t, sm[k]);
        // non-negative doubles order like their bit patterns
        atomicMax(rr2 + h, (unsigned long long)__double_as_longlong(t));
        __threadfence();
        last = atomicAdd(ctr + h, 1) == sh - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const double r = __dsqrt_rn(__longlong_as_double((long long)atomicAdd(rr2 + h, 0ull)));
        const double M = cen[4 * h + 3];
        ctr[h] = 0;
        if (out) {
            double *o = out + (int64_t)h * HALMA_PSC_NFIELDS;
            o[HALMA_PSC_CX] = cx;
            o[HALMA_PSC_CY] = cy;
            o[HALMA_PSC_CZ] = cz;
            o[HALMA_PSC_MASS] = M;
            o[HALMA_PSC_RMAX] = r;
            o[HALMA_PSC_NPART] = (double)(off[h + 1] - off[h]);
        } else {
            PscState &s = st[h];
            nwhich[h] = off[h + 1] - off[h];   // the which_cell arrays of this grid
            s.cx = cx;
            s.cy = cy;
            s.cz = cz;
            s.M = M;
            s.rr = r;
            // np.arange(-(r + ll), r + ll, 2 ll): length ceil((stop - start) / step)
            const double stop = __dadd_rn(r, ll), start = -stop, step = __dmul_rn(2.0, ll);
            s.start = start;
            s.step = step;
            s.inv_step = 1.0 / step;
            s.next = __dadd_rn(start, step);
            s.delta = __dsub_rn(s.next, start);
            s.inv_delta = 1.0 / s.delta;
            s.n = (long long)ceil(__ddiv_rn(__dsub_rn(stop, start), step));
            if (s.n < 1) s.n = 1;
            s.margin = 1e-12 * (double)(s.n + 8);
            if (s.first) s.n0 = s.n;
        }
    }
}

// Per list entry of a group in SWEEP or FINAL mode: nearest grid point per axis, the which_cell
// output (at the entry's position in its group), and the sort key (group, cell) for the
// per-cell sums (entries of other groups sort last).
__global__ void psc_cell_kernel(int64_t nl, const int *__restrict__ list, const int *__restrict__ owner,
                                const int64_t *__restrict__ off, const int64_t *__restrict__ goff,
                                const int *__restrict__ mem, const double *__restrict__ x,
                                const double *__restrict__ y, const double *__restrict__ z,
                                const PscState *__restrict__ st, int cbits, uint64_t *__restrict__ keys,
                                int *__restrict__ vals, int *__restrict__ wx, int *__restrict__ wy,
                                int *__restrict__ wz) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nl; e += (int64_t)gridDim.x * blockDim.x) {
        const int h = owner[e];
        const PscState &s = st[h];
        uint64_t key = ~0ull;
        if (s.mode != kModeNone) {
            const int i = mem[list[e]];
            const long long ix = nearest(s, __dsub_rn(x[i], s.cx));
            const long long iy = nearest(s, __dsub_rn(y[i], s.cy));
            const long long iz = nearest(s, __dsub_rn(z[i], s.cz));
            const int64_t p = goff[h] + (e - off[h]);
            wx[p] = (int)ix;
            wy[p] = (int)iy;
            wz[p] = (int)iz;
            if (s.mode == kModeSweep) key = ((uint64_t)h << cbits) | (uint64_t)((ix * s.n + iy) * s.n + iz);
        }
        keys[e] = key;
        vals[e] = (int)e;
    }
}

__global__ void psc_head_kernel(int64_t nl, const uint64_t *__restrict__ keys, int *__restrict__ head) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nl; k += (int64_t)gridDim.x * blockDim.x)
        head[k] = (keys[k] != ~0ull && (k == 0 || keys[k] != keys[k - 1])) ? 1 : 0;
}

// Run starts: runstart[r] = first sorted position of cell r; runstart[nrun] = the end of the
// last cell (entries of groups that do not sweep sort last, with key ~0); *nrun_out = nrun.
__global__ void psc_runstart_kernel(int64_t nl, const uint64_t *__restrict__ keys, const int *__restrict__ head,
                                    const int *__restrict__ rpos, int *__restrict__ runstart, int *__restrict__ nrun_out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nl; k += (int64_t)gridDim.x * blockDim.x) {
        if (head[k]) runstart[rpos[k]] = (int)k;
        if (keys[k] != ~0ull && (k + 1 == nl || keys[k + 1] == ~0ull)) {
            runstart[rpos[k] + head[k]] = (int)(k + 1);
            *nrun_out = rpos[k] + head[k];
        }
    }
}

// Velocity and mass of every sorted list entry, gathered into cell order so that the per-cell
// sums read contiguous memory (and can fetch the next 32 members while adding the current).
struct __align__(16) VelMass {
    double vx, vy, vz, m;
};

__global__ void psc_gather_kernel(int64_t nl, const int *__restrict__ vals, const int *__restrict__ list,
                                  const int *__restrict__ mem, const double *__restrict__ vx,
                                  const double *__restrict__ vy, const double *__restrict__ vz,
                                  const double *__restrict__ m, VelMass *__restrict__ gv) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nl; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = mem[list[vals[k]]];
        VelMass p;
        p.vx = vx[i];
        p.vy = vy[i];
        p.vz = vz[i];
        p.m = m[i];
        gv[k] = p;
    }
}

__device__ __forceinline__ VelMass vm_load(const VelMass *__restrict__ gv, int k, int e) {
    if (k < e) return gv[k];
    VelMass z;
    z.vx = z.vy = z.vz = z.m = 0.0;
    return z;
}

// Per cell (members in list order): count, mass, mass-weighted mean velocity, then the
// dispersion; every member's entry gets the cell's index.  Most cells hold a few members, so
// cells of up to kPscSmall members take one thread each (plain sequential FP64 adds, and the
// divisions of 32 cells share one warp instruction); larger cells take one warp each.
constexpr int kPscSmall = 128;

__global__ void psc_small_kernel(const int *__restrict__ nrun_p, const int *__restrict__ runstart,
                                 const int *__restrict__ vals, const VelMass *__restrict__ gv,
                                 double4 *__restrict__ cell_v, double *__restrict__ cell_sig, int *__restrict__ rid) {
    const int nrun = *nrun_p;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrun; r += (int64_t)gridDim.x * blockDim.x) {
        const int b = runstart[r], e = runstart[r + 1];
        if (e - b > kPscSmall) continue;
        double mass = 0.0, sx = 0.0, sy = 0.0, sz = 0.0;
        for (int k = b; k < e; ++k) {
            const VelMass p = gv[k];
            sx = __dadd_rn(sx, __dmul_rn(p.vx, p.m));
            sy = __dadd_rn(sy, __dmul_rn(p.vy, p.m));
            sz = __dadd_rn(sz, __dmul_rn(p.vz, p.m));
            mass = __dadd_rn(mass, p.m);
            rid[vals[k]] = (int)r;
        }
        const double q = (double)(e - b);
        const double ux = __ddiv_rn(sx, mass), uy = __ddiv_rn(sy, mass), uz = __ddiv_rn(sz, mass);
        double s2 = 0.0;
        for (int k = b; k < e; ++k) {
            const VelMass p = gv[k];
            const double dx = __dsub_rn(ux, p.vx), dy = __dsub_rn(uy, p.vy), dz = __dsub_rn(uz, p.vz);
            s2 = __dadd_rn(s2, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
        }
        cell_v[r] = make_double4(ux, uy, uz, q);
        cell_sig[r] = __dsqrt_rn(__ddiv_rn(__ddiv_rn(s2, 3.0), q));
    }
}

// Cells of more than kPscSmall members, one warp each: the lanes take 32 members at a time and
// form their products; the sums are the sequential FP64 ones, added 32 values at a time in
// integer ulps (seqsum.cuh), so the warp does not wait on a chain of FP64 adds.
__global__ void psc_run_kernel(const int *__restrict__ nrun_p, const int *__restrict__ runstart,
                               const int *__restrict__ vals, const VelMass *__restrict__ gv,
                               double4 *__restrict__ cell_v, double *__restrict__ cell_sig, int *__restrict__ rid) {
    const int lane = threadIdx.x & 31;
    const int nrun = *nrun_p;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < nrun; r += warps) {
        const int b = runstart[r], e = runstart[r + 1];
        if (e - b <= kPscSmall) continue;
        SeqSum mass, sx, sy, sz;
        seq_init(mass);
        seq_init(sx);
        seq_init(sy);
        seq_init(sz);
        VelMass nxt = vm_load(gv, b + lane, e);
        for (int k0 = b; k0 < e; k0 += 32) {
            const int k = k0 + lane;
            const VelMass p = nxt;
            nxt = vm_load(gv, k + 32, e);
            double a = 0.0, c = 0.0, d = 0.0;
            if (k < e) {
                a = __dmul_rn(p.vx, p.m);
                c = __dmul_rn(p.vy, p.m);
                d = __dmul_rn(p.vz, p.m);
                rid[vals[k]] = (int)r;
            }
            const int cnt = e - k0 < 32 ? e - k0 : 32;
            seq_add_warp(sx, a, cnt, lane);
            seq_add_warp(sy, c, cnt, lane);
            seq_add_warp(sz, d, cnt, lane);
            seq_add_warp(mass, p.m, cnt, lane);
        }
        const double q = (double)(e - b), M = seq_value(mass);
        const double ux = __ddiv_rn(seq_value(sx), M), uy = __ddiv_rn(seq_value(sy), M), uz = __ddiv_rn(seq_value(sz), M);
        SeqSum s2;
        seq_init(s2);
        nxt = vm_load(gv, b + lane, e);
        for (int k0 = b; k0 < e; k0 += 32) {
            const int k = k0 + lane;
            const VelMass p = nxt;
            nxt = vm_load(gv, k + 32, e);
            double t2 = 0.0;
            if (k < e) {
                const double dx = __dsub_rn(ux, p.vx), dy = __dsub_rn(uy, p.vy), dz = __dsub_rn(uz, p.vz);
                t2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            }
            seq_add_warp(s2, t2, e - k0 < 32 ? e - k0 : 32, lane);
        }
        if (lane == 0) {
            cell_v[r] = make_double4(ux, uy, uz, q);
            cell_sig[r] = __dsqrt_rn(__ddiv_rn(__ddiv_rn(seq_value(s2), 3.0), q));
        }
    }
}

// The sweep, per list entry of a group in SWEEP mode.
__global__ void psc_sweep_kernel(int64_t nl, const int *__restrict__ list, const int *__restrict__ owner,
                                 const int64_t *__restrict__ off, const int64_t *__restrict__ goff,
                                 const int *__restrict__ mem, const double *__restrict__ vx,
                                 const double *__restrict__ vy, const double *__restrict__ vz,
                                 const double4 *__restrict__ cell_v, const double *__restrict__ cell_sig,
                                 const int *__restrict__ rid, double q_fil, double sig_fil, PscState *st,
                                 unsigned char *__restrict__ control) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nl; e += (int64_t)gridDim.x * blockDim.x) {
        const int h = owner[e];
        if (st[h].mode != kModeSweep) continue;
        const int i = mem[list[e]];
        const double4 c = cell_v[rid[e]];
        const double q = c.w;
        bool drop = true;
        if (q > q_fil) {
            const double thr = __dmul_rn(st[h].fac_sig, sig_fil);
            const bool norm = st[h].first ? q > 2.0 : q >= 2.0;
            if (!norm) {
                drop = 0.0 >= thr;   // the reference's bas = 0 when the cell is not normalised
            } else {
                const double dx = __dsub_rn(c.x, vx[i]), dy = __dsub_rn(c.y, vy[i]), dz = __dsub_rn(c.z, vz[i]);
                const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                const double sig = cell_sig[rid[e]];
                // sqrt(d2) / sig >= thr, rounded as the reference rounds it: far from the threshold
                // (relative 4e-12, against rounding errors of ~5e-16) the squares decide it without
                // the FP64 square root and divide; near it, or for a zero or non-finite sigma, the
                // reference's operations do
                const double ts = thr * sig, t2 = ts * ts;
                const bool ok = sig > 0.0 && thr > 0.0 && t2 >= 2.2250738585072014e-308 && t2 < 1e300;
                if (ok && d2 > t2 * (1.0 + 4e-12)) {
                    drop = true;
                } else if (ok && d2 < t2 * (1.0 - 4e-12)) {
                    drop = false;
                } else {
                    drop = __ddiv_rn(__dsqrt_rn(d2), sig) >= thr;
                }
            }
        }
        if (drop) {
            control[goff[h] + (e - off[h])] = 0;   // position in the list being swept
            atomicAdd(reinterpret_cast<unsigned long long *>(&st[h].cleaned), 1ull);
        }
    }
}

// After a sweep: counts, fac_sig and the group's next mode.  After a final step: done.
__global__ void psc_post_kernel(int G, PscState *st, int *counts) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < G; h += gridDim.x * blockDim.x) {
        PscState &s = st[h];
        if (s.mode == kModeFinal) {
            s.mode = kModeNone;
            continue;
        }
        if (s.mode != kModeSweep) continue;
        s.passes += 1;
        s.remaining -= s.cleaned;
        int next;
        if (s.first) {
            s.fac_sig = __dmul_rn(s.fac_sig, 0.75);
            next = (s.remaining > 0 && __ddiv_rn((double)s.cleaned, (double)s.remaining) > 0.1) ? kModeSweep : kModeFinal;
            s.first = 0;
        } else if (s.remaining == 0) {
            s.zero = 1;
            next = kModeNone;
        } else {
            const double frac = __ddiv_rn((double)s.cleaned, (double)s.remaining);
            s.fac_sig = fmax(1.0, __dmul_rn(s.fac_sig, 0.75));
            next = frac > 0.1 ? kModeSweep : kModeFinal;
        }
        s.cleaned = 0;
        s.mode = next;
        if (next == kModeSweep) atomicAdd(counts, 1);
        if (next == kModeFinal) atomicAdd(counts + 1, 1);
    }
}

__global__ void psc_init_kernel(int G, const int64_t *__restrict__ goff, int64_t n0, PscState *st,
                                unsigned char *__restrict__ control) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n0; k += (int64_t)gridDim.x * blockDim.x)
        control[k] = 1;
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < G; h += gridDim.x * blockDim.x) {
        PscState s;
        memset(&s, 0, sizeof(s));
        s.fac_sig = 2.0;
        s.first = 1;
        s.remaining = goff[h + 1] - goff[h];
        s.mode = kModeSweep;
        st[h] = s;
    }
}

__global__ void psc_flag_kernel(int64_t n0, const unsigned char *__restrict__ control, int *__restrict__ flag) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n0; k += (int64_t)gridDim.x * blockDim.x)
        flag[k] = control[k] ? 1 : 0;
}

// The next lists: list[pos[k]] = k for every member position k with control[k]; off[h] = pos
// at the group's first member.
__global__ void psc_compact_kernel(int64_t n0, int G, const int *__restrict__ flag, const int *__restrict__ pos,
                                   const int64_t *__restrict__ goff, int *__restrict__ list,
                                   int64_t *__restrict__ off) {
    const int64_t total = n0 > 0 ? (int64_t)pos[n0 - 1] + flag[n0 - 1] : 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n0; k += (int64_t)gridDim.x * blockDim.x)
        if (flag[k]) list[pos[k]] = (int)k;
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h <= G; h += (int64_t)gridDim.x * blockDim.x)
        off[h] = goff[h] < n0 ? (int64_t)pos[goff[h]] : total;
}

// Main-script step: control reset to ones when cleaning is off or the group is small.
__global__ void psc_reset_kernel(int G, const int64_t *__restrict__ goff, int enabled, int min_part,
                                 unsigned char *__restrict__ control) {
    for (int h = blockIdx.x; h < G; h += gridDim.x) {
        const int64_t b = goff[h], e = goff[h + 1];
        if (enabled && e - b >= min_part) continue;
        for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) control[k] = 1;
    }
}

__global__ void psc_out_kernel(int G, const PscState *__restrict__ st, int minp, double *__restrict__ out) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < G; h += gridDim.x * blockDim.x) {
        double *o = out + (int64_t)h * HALMA_PSC_NFIELDS;
        o[HALMA_PSC_NCELL] = (double)st[h].n0;
        o[HALMA_PSC_KEPT] = o[HALMA_PSC_NPART] >= (double)minp ? 1.0 : 0.0;
        o[HALMA_PSC_PASSES] = (double)st[h].passes;
    }
}

// Input check before any other kernel: bad |= 1 for a member outside [0, n), |= 2 for a
// member with a non-finite position, velocity or mass.
__global__ void psc_check_kernel(int64_t n0, const int *__restrict__ mem, int64_t n, const double *__restrict__ x,
                                 const double *__restrict__ y, const double *__restrict__ z,
                                 const double *__restrict__ vx, const double *__restrict__ vy,
                                 const double *__restrict__ vz, const double *__restrict__ m, int *__restrict__ bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n0; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = mem[k];
        if (i < 0 || (int64_t)i >= n) {
            atomicOr(bad, 1);
            continue;
        }
        if (!isfinite(x[i]) || !isfinite(y[i]) || !isfinite(z[i]) || !isfinite(vx[i]) || !isfinite(vy[i]) ||
            !isfinite(vz[i]) || !isfinite(m[i]))
            atomicOr(bad, 2);
    }
}

int bits_needed(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_phase_space_clean(int64_t n, const double *x, const double *y, const double *z,
                                       const double *vx, const double *vy, const double *vz, const double *m,
                                       int64_t n_groups, const int64_t *group_offsets,
                                       const int32_t *group_members, const halma_psc_params *params,
                                       uint8_t *control, int32_t *which_cell, int64_t *n_which, double *halo_out,
                                       halma_stream_t stream) {
    if (!params) return fail(HALMA_ERR_INVALID, "params must not be NULL");
    if (n < 0 || n_groups < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= INT32_MAX || n_groups >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles and groups");
    const halma_psc_params p = *params;
    if (!(p.linking_length > 0.0) || !isfinite(p.linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and > 0");
    if (!isfinite(p.q_fil) || !isfinite(p.sig_fil)) return fail(HALMA_ERR_INVALID, "q_fil and sig_fil must be finite");
    if (p.max_passes < 1) return fail(HALMA_ERR_INVALID, "max_passes must be >= 1");
    if (!group_offsets || !halo_out || (n_groups > 0 && (!group_members || !control)) ||
        (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    if (n_groups == 0) return HALMA_OK;
    std::vector<int64_t> h_goff(n_groups + 1);
    HALMA_CUDA(cudaMemcpy(h_goff.data(), group_offsets, 8ull * (n_groups + 1), cudaMemcpyDefault));
    if (h_goff[0] != 0) return fail(HALMA_ERR_INVALID, "group offsets must start at 0");
    for (int64_t g = 0; g < n_groups; ++g)
        if (h_goff[g + 1] < h_goff[g]) return fail(HALMA_ERR_INVALID, "group offsets must not decrease");
    const int64_t N0 = h_goff[n_groups];
    if (N0 >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 members");
    const int G = (int)n_groups;
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dvx = nullptr, *dvy = nullptr, *dvz = nullptr,
                 *dm = nullptr;
    const int64_t *dgoff = nullptr;
    const int32_t *dmem = nullptr;
    uint8_t *dctl = nullptr;
    int32_t *dwhich = nullptr;
    int64_t *dnw = nullptr;
    double *dout = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(vx, n, true, false, &dvx);
    sg.add(vy, n, true, false, &dvy);
    sg.add(vz, n, true, false, &dvz);
    sg.add(m, n, true, false, &dm);
    sg.add(group_offsets, n_groups + 1, true, false, &dgoff);
    sg.add(group_members, N0, true, false, &dmem);
    sg.add((const uint8_t *)control, N0, false, true, &dctl);
    sg.add((const int32_t *)which_cell, which_cell ? 3 * N0 : 0, false, true, &dwhich);
    sg.add((const int64_t *)n_which, n_which ? n_groups : 0, false, true, &dnw);
    sg.add((const double *)halo_out, n_groups * HALMA_PSC_NFIELDS, false, true, &dout);
    const int64_t NL = std::max<int64_t>(N0, 1);
    Layout L;
    sg.plan(L);
    const size_t o_st = L.add(sizeof(PscState) * G), o_off = L.add(8ull * (G + 1)), o_list = L.add(4ull * NL);
    const size_t o_own = L.add(4ull * NL), o_kin = L.add(8ull * NL), o_kout = L.add(8ull * NL);
    const size_t o_vin = L.add(4ull * NL), o_vout = L.add(4ull * NL), o_head = L.add(4ull * NL);
    const size_t o_rpos = L.add(4ull * NL), o_rid = L.add(4ull * NL), o_cv = L.add(32ull * NL);
    const size_t o_gv = L.add(sizeof(VelMass) * NL);
    const size_t o_sig = L.add(8ull * NL), o_flag = L.add(4ull * (NL + 1)), o_pos = L.add(4ull * NL);
    const size_t o_w = L.add(12ull * NL), o_nw = L.add(8ull * G), o_cnt = L.add(64);
    const int S = G >= 8192 ? 1 : 16;   // blocks per group for the centre and furthest particle
    const size_t o_part = L.add(32ull * S * G), o_ctr = L.add(4ull * G), o_cen = L.add(32ull * G),
                 o_rr2 = L.add(8ull * G);
    const size_t sort_b = sort_pairs_u64_i32_bytes((int)NL, 64), scan_b = exclusive_sum_i32_bytes((int)NL);
    const size_t o_tmp = L.add(std::max(sort_b, scan_b));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 6));
    HALMA_TRY(sg.bind_and_upload(base, st));
    auto *state = at<PscState>(base, o_st);
    auto *off = at<int64_t>(base, o_off);
    int *list = at<int>(base, o_list), *own = at<int>(base, o_own);
    auto *kin = at<uint64_t>(base, o_kin), *kout = at<uint64_t>(base, o_kout);
    int *vin = at<int>(base, o_vin), *vout = at<int>(base, o_vout), *head = at<int>(base, o_head);
    int *rpos = at<int>(base, o_rpos), *rid = at<int>(base, o_rid);
    auto *cv = at<double4>(base, o_cv);
    auto *gv = at<VelMass>(base, o_gv);
    double *csig = at<double>(base, o_sig);
    int *flag = at<int>(base, o_flag), *pos = at<int>(base, o_pos);
    int *wbuf = dwhich ? dwhich : at<int>(base, o_w);
    int64_t *nw = dnw ? dnw : at<int64_t>(base, o_nw);
    int *cnt = at<int>(base, o_cnt);
    double *part = at<double>(base, o_part), *cen = at<double>(base, o_cen);
    int *ctr = at<int>(base, o_ctr);
    auto *rr2 = at<unsigned long long>(base, o_rr2);
    void *tmp = at<void>(base, o_tmp);
    int *wx = wbuf, *wy = wbuf + N0, *wz = wbuf + 2 * N0;
    const int gS = G * S;
    // centre of mass and furthest particle of the groups that sweep or end (all: every group)
    auto centres = [&](int all, double *o) -> int {
        HALMA_LAUNCH(psc_sum_kernel, gS, 256, 0, st, G, off, list, dmem, dx, dy, dz, dm, S, all, state, part, ctr,
                     cen, rr2);
        HALMA_LAUNCH(psc_rmax_kernel, gS, 256, 0, st, G, off, list, dmem, dx, dy, dz, p.linking_length, S, all, state,
                     o, nw, ctr, cen, rr2);
        return HALMA_OK;
    };
    const int sms = device_sm_count();
    const int gN = std::min(sms * 8, grid_for(NL, 256)), gG = std::min(G, sms * 16), gH = grid_for(G, 256);

    if (N0 > 0) {
        HALMA_CUDA(cudaMemsetAsync(cnt, 0, 4, st));
        HALMA_LAUNCH(psc_check_kernel, gN, 256, 0, st, N0, dmem, n, dx, dy, dz, dvx, dvy, dvz, dm, cnt);
        int bad = 0;
        HALMA_CUDA(cudaMemcpyAsync(&bad, cnt, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        if (bad & 1) return fail(HALMA_ERR_INVALID, "group member outside [0, n)");
        if (bad & 2) return fail(HALMA_ERR_INVALID, "non-finite position, velocity or mass in a group");
    }
    // cell numbers need bits for the largest grid; the group id goes above them
    const int gbits = bits_needed((uint64_t)G);
    HALMA_LAUNCH(psc_init_kernel, std::max(gN, gH), 256, 0, st, G, dgoff, N0, state, dctl);
    HALMA_CUDA(cudaMemsetAsync(nw, 0, 8ull * G, st));
    HALMA_CUDA(cudaMemsetAsync(ctr, 0, 4ull * G, st));
    // the first lists are the groups themselves
    HALMA_LAUNCH(psc_flag_kernel, gN, 256, 0, st, N0, dctl, flag);
    HALMA_TRY(exclusive_sum_i32(tmp, scan_b, flag, pos, (int)NL, st));
    HALMA_LAUNCH(psc_compact_kernel, gN, 256, 0, st, N0, G, flag, pos, dgoff, list, off);
    int sweeping = G, finals = 0;
    for (int pass = 0; (sweeping > 0 || finals > 0) && N0 > 0; ++pass) {
        if (pass >= p.max_passes + 1) return fail(HALMA_ERR_NOT_CONVERGED, "phase-space cleaning did not stop in %d passes", p.max_passes);
        HALMA_LAUNCH(psc_fill_kernel, gG, 256, 0, st, G, off, own);
        HALMA_TRY(centres(0, nullptr));
        // the largest grid decides the cell bits
        std::vector<PscState> hs(G);
        HALMA_CUDA(cudaMemcpyAsync(hs.data(), state, sizeof(PscState) * G, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        long long nmax = 1;
        for (const auto &s : hs)
            if (s.mode != kModeNone) nmax = std::max(nmax, s.n);
        const long double cells = (long double)nmax * nmax * nmax;
        const int cbits = bits_needed((uint64_t)std::min<long double>(cells, 1.8e19L));
        if (cells > 1.0e18L || cbits + gbits > 63)
            return fail(HALMA_ERR_CAPACITY, "cleaning grid of %lld points a side is too large", nmax);
        int64_t nl = 0;
        HALMA_CUDA(cudaMemcpyAsync(&nl, off + G, 8, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        if (nl > 0) {
            const int gl = std::min(sms * 8, grid_for(nl, 256));
            HALMA_LAUNCH(psc_cell_kernel, gl, 256, 0, st, nl, list, own, off, dgoff, dmem, dx, dy, dz, state, cbits,
                         kin, vin, wx, wy, wz);
            if (sweeping > 0) {
                HALMA_TRY(sort_pairs_u64_i32(tmp, sort_b, kin, kout, vin, vout, (int)nl, 64, st));
                HALMA_LAUNCH(psc_head_kernel, gl, 256, 0, st, nl, kout, head);
                HALMA_TRY(exclusive_sum_i32(tmp, scan_b, head, rpos, (int)nl, st));
                HALMA_CUDA(cudaMemsetAsync(cnt + 2, 0, 4, st));
                HALMA_LAUNCH(psc_runstart_kernel, gl, 256, 0, st, nl, kout, head, rpos, flag, cnt + 2);
                HALMA_LAUNCH(psc_gather_kernel, gl, 256, 0, st, nl, vout, list, dmem, dvx, dvy, dvz, dm, gv);
                HALMA_LAUNCH(psc_small_kernel, sms * 8, 256, 0, st, cnt + 2, flag, vout, gv, cv, csig, rid);
                HALMA_LAUNCH(psc_run_kernel, sms * 16, 256, 0, st, cnt + 2, flag, vout, gv, cv, csig, rid);
                HALMA_LAUNCH(psc_sweep_kernel, gl, 256, 0, st, nl, list, own, off, dgoff, dmem, dvx, dvy, dvz, cv, csig,
                             rid, p.q_fil, p.sig_fil, state, dctl);
            }
        }
        HALMA_CUDA(cudaMemsetAsync(cnt, 0, 8, st));
        HALMA_LAUNCH(psc_post_kernel, gH, 256, 0, st, G, state, cnt);
        HALMA_LAUNCH(psc_flag_kernel, gN, 256, 0, st, N0, dctl, flag);
        HALMA_TRY(exclusive_sum_i32(tmp, scan_b, flag, pos, (int)NL, st));
        HALMA_LAUNCH(psc_compact_kernel, gN, 256, 0, st, N0, G, flag, pos, dgoff, list, off);
        int hc[2];
        HALMA_CUDA(cudaMemcpyAsync(hc, cnt, 8, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        sweeping = hc[0];
        finals = hc[1];
    }
    // main-script step: reset, centre / mass / furthest particle of the kept particles
    HALMA_LAUNCH(psc_reset_kernel, gG, 256, 0, st, G, dgoff, p.enabled, p.min_part, dctl);
    HALMA_LAUNCH(psc_flag_kernel, gN, 256, 0, st, N0, dctl, flag);
    HALMA_TRY(exclusive_sum_i32(tmp, scan_b, flag, pos, (int)NL, st));
    HALMA_LAUNCH(psc_compact_kernel, gN, 256, 0, st, N0, G, flag, pos, dgoff, list, off);
    HALMA_TRY(centres(1, dout));
    HALMA_LAUNCH(psc_out_kernel, gH, 256, 0, st, G, state, p.minp, dout);
    HALMA_TRY(sg.download(st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    return HALMA_OK;
}
