// Per-halo FP64 reductions over CSR halo segments (python_scripts/halo_properties.py):
//   total_mass (:16-24), center_of_mass (:26-43), CM_velocity (:45-60),
//   furthest_particle (:98-111), half_mass_radius (:365-392), sigma_effective (:607-625).
// One block per halo for the sums; the half-mass radius needs the members in increasing
// distance from the centre, obtained with two stable radix sorts over all particles (by the
// FP64 distance bits, then by halo id), after which each halo walks its own segment.
#include <limits.h>
#include <math.h>
#include <string.h>

#include "common.cuh"
#include "sort.cuh"

namespace halma {
namespace {

struct Red {
    double M, cx, cy, cz, vx, vy, vz, rmax, r05, sigma, n, mref, plain;
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

// The member range of every halo is cut into chunks of at most kRedChunk members, so that a
// big halo's FP64 sums are spread over many blocks (GB300 issues FP64 instructions at a small
// fraction of its FP32 rate, so one block per halo would leave the biggest halo's SM as the
// critical path).  Chunk c belongs to halo chunk_h[c] and covers its members
// off[h] + (c - cstart[h]) * kRedChunk onward.  The partial sums of a halo's chunks are added
// in chunk order, so results do not depend on scheduling.
constexpr int kRedChunk = 4096;
constexpr int kRedParts = 9;   // M, Mx, My, Mz, Mvx, Mvy, Mvz, count, masses the integer walk cannot take

__global__ void red_chunks_kernel(int nh, const int64_t *__restrict__ off, int *__restrict__ cnum) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h <= nh; h += gridDim.x * blockDim.x) {
        const int64_t n = h < nh ? off[h + 1] - off[h] : 0;
        cnum[h] = h < nh ? (int)(n > 0 ? (n + kRedChunk - 1) / kRedChunk : 1) : 0;
    }
}

__global__ void red_owner_kernel(int nh, const int *__restrict__ cstart, int *__restrict__ chunk_h) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x)
        for (int c = cstart[h]; c < cstart[h + 1]; ++c) chunk_h[c] = h;
}

struct Chunk {
    int h;
    int64_t b, e;
};

__device__ __forceinline__ bool chunk_of(int c, int nh, const int64_t *__restrict__ off, const int *__restrict__ cstart,
                                         const int *__restrict__ chunk_h, Chunk &k) {
    if (c >= cstart[nh]) return false;
    k.h = chunk_h[c];
    k.b = off[k.h] + (int64_t)(c - cstart[k.h]) * kRedChunk;
    k.e = min(off[k.h + 1], k.b + (int64_t)kRedChunk);
    return true;
}

// Per chunk: FP64 sums of m, m x, m v, the member count, and the number of masses that are
// negative, -0.0 or not finite (those haloes walk with plain FP64 adds).
__global__ void __launch_bounds__(256) red_part_kernel(int nh, const int64_t *__restrict__ off,
                                                       const int *__restrict__ cstart, const int *__restrict__ chunk_h,
                                                       const double *__restrict__ x, const double *__restrict__ y,
                                                       const double *__restrict__ z, const double *__restrict__ vx,
                                                       const double *__restrict__ vy, const double *__restrict__ vz,
                                                       const double *__restrict__ m, const unsigned char *__restrict__ mask,
                                                       double *__restrict__ part) {
    Chunk k;
    if (!chunk_of(blockIdx.x, nh, off, cstart, chunk_h, k)) return;
    __shared__ double sh[kRedParts][32];
    double v[kRedParts] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t i = k.b + threadIdx.x; i < k.e; i += blockDim.x) {
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
        const unsigned long long bits = (unsigned long long)__double_as_longlong(mi);
        if ((bits >> 63) || ((bits >> 52) & 0x7ff) == 0x7ff) v[8] += 1.0;
    }
    bsum<kRedParts>(v, sh);
    if (threadIdx.x < kRedParts) part[(int64_t)blockIdx.x * kRedParts + threadIdx.x] = v[threadIdx.x];
}

// One thread per halo: the chunks' sums in order, centre, bulk velocity (or the caller's),
// reference mass and R05; rmax starts at 0 for the distance kernel's atomic maximum.
__global__ void red_center_kernel(int nh, const int *__restrict__ cstart, const double *__restrict__ part,
                                  const double *__restrict__ about, Red *__restrict__ red) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
        double v[kRedParts] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int c = cstart[h]; c < cstart[h + 1]; ++c)
#pragma unroll
            for (int q = 0; q < kRedParts; ++q) v[q] += part[(int64_t)c * kRedParts + q];
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
        Red o;
        o.M = M; o.cx = cx; o.cy = cy; o.cz = cz; o.vx = ux; o.vy = uy; o.vz = uz;
        o.rmax = 0.0; o.r05 = r05_in; o.sigma = 0; o.n = v[7]; o.mref = Mref; o.plain = v[8];
        red[h] = o;
    }
}

// Per chunk: distances, sort keys (distance bits, halo id) and the halo's R_max.
__global__ void __launch_bounds__(256) red_dist_kernel(int nh, const int64_t *__restrict__ off,
                                                       const int *__restrict__ cstart, const int *__restrict__ chunk_h,
                                                       const double *__restrict__ x, const double *__restrict__ y,
                                                       const double *__restrict__ z, const unsigned char *__restrict__ mask,
                                                       Red *__restrict__ red, uint64_t *__restrict__ dkey,
                                                       double *__restrict__ dist, uint32_t *__restrict__ hid) {
    Chunk k;
    if (!chunk_of(blockIdx.x, nh, off, cstart, chunk_h, k)) return;
    const double cx = red[k.h].cx, cy = red[k.h].cy, cz = red[k.h].cz;
    double rmax = 0.0;
    for (int64_t i = k.b + threadIdx.x; i < k.e; i += blockDim.x) {
        const bool in = !mask || mask[i];
        const double dx = cx - x[i], dy = cy - y[i], dz = cz - z[i];
        // (dx**2 + dy**2 + dz**2)**0.5 as the reference evaluates it (halo_properties.py:104-107),
        // each operation rounded on its own so that d < R05 splits members the same way
        const double d = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
        dist[i] = d;
        if (in) rmax = fmax(rmax, d);
        // excluded particles sort after every member (+inf)
        dkey[i] = in ? (uint64_t)__double_as_longlong(d) : 0x7ff0000000000000ull;
        hid[i] = (uint32_t)k.h;
    }
    __shared__ double shm[32];
    const double wm = wmax(rmax);
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = wm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double r = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r = fmax(r, shm[q]);
        // non-negative doubles order like their bit patterns
        atomicMax(reinterpret_cast<unsigned long long *>(&red[k.h].rmax), (unsigned long long)__double_as_longlong(r));
    }
}

__global__ void gather_hid_kernel(int64_t n, const int *__restrict__ perm, const uint32_t *__restrict__ hid,
                                  uint32_t *__restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = hid[perm[k]];
}

// The half-mass walk's running sum (halo_properties.py:385-390: cumulative mass in increasing
// distance, compared with M/2 after every addition) is a chain of dependent FP64 adds, which
// GB300 runs at a small fraction of its integer rate.  For non-negative masses the walk keeps
// the sum as an integer number S of ulps of its binade [2^e, 2^(e+1)), ulp = 2^(e-52): while the
// sum stays in the binade, __dadd_rn(sum, m) equals (S + round(m / ulp)) * ulp, with m / ulp
// rounded to the nearest integer and a tie (a remainder of exactly half an ulp) going to the
// even sum.  So the adds are exact integer adds of per-mass increments that do not depend on
// the sum, except for the parity at a tie.  A step that leaves the binade (or starts from a sum
// that is zero or subnormal) is one __dadd_rn, after which the binade is read from the result.
struct SeqSum {
    double c;       // the sum (current only when !nrm; otherwise S * ulp)
    long long S;    // the sum in ulps of its binade, in [2^52, 2^53), when nrm
    long long hl;   // S > hl  <=>  sum > half
    int e;          // binade exponent
    bool nrm;       // the sum is a normal number
};

constexpr long long kTwo53 = 1ll << 53;

__device__ __forceinline__ void seq_set(SeqSum &q, double c, double half) {
    q.c = c;
    const unsigned long long b = (unsigned long long)__double_as_longlong(c);
    const int ef = (int)((b >> 52) & 0x7ff);
    q.nrm = ef != 0 && ef != 0x7ff && !(b >> 63);
    if (q.nrm) {
        q.e = ef - 1023;
        q.S = (long long)((b & 0xfffffffffffffull) | (1ull << 52));
        const double hs = ldexp(half, 52 - q.e);   // half in ulps of the binade (exact scaling)
        q.hl = !(hs < (double)kTwo53) ? kTwo53 : (hs < 0.0 ? -1ll : (long long)floor(hs));
    }
}

// m / ulp for ulp = 2^(e-52): integer part fl and the rounding of the remainder (0 below half
// an ulp, 1 above, 2 exactly half); big when m / ulp >= 2^53 could not be held.  m is finite,
// non-negative and has a clear sign bit.
__device__ __forceinline__ void mass_ulps(double m, int e, long long &fl, int &code, bool &big) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(m);
    const int ef = (int)(b >> 52);
    const unsigned long long M = (b & 0xfffffffffffffull) | (ef ? (1ull << 52) : 0ull);
    const int d = (e - 52) - (ef ? ef - 1075 : -1074);   // m = M * 2^(e - 52 - d)
    big = d < 0;
    if (d <= 0) {
        fl = (long long)M;
        code = 0;
    } else if (d >= 64) {
        fl = 0;
        code = 0;
    } else {
        fl = (long long)(M >> d);
        const unsigned long long rem = M & ((1ull << d) - 1ull), hb = 1ull << (d - 1);
        code = rem > hb ? 1 : (rem == hb ? 2 : 0);
    }
}

__device__ __forceinline__ long long inc_sum(long long S, long long fl, int code) {
    const long long base = S + fl;
    return base + (code == 1 ? 1 : (code == 2 ? (base & 1) : 0));
}

// One mass; true once the sum exceeds half.
__device__ __forceinline__ bool seq_add(SeqSum &q, double m, double half) {
    if (q.nrm) {
        long long fl;
        int code;
        bool big;
        mass_ulps(m, q.e, fl, code, big);
        const long long T = inc_sum(q.S, fl, code);
        if (!big && T < kTwo53) {
            q.S = T;
            return T > q.hl;
        }
        q.c = ldexp((double)q.S, q.e - 52);   // exact
    }
    seq_set(q, __dadd_rn(q.c, m), half);
    return q.c > half;
}

// Half-mass radius: walk the halo's members by increasing distance with the running sum;
// R05 is the distance of the last member before the sum first exceeds M/2 (the smallest
// distance if the first member already exceeds it, the largest if none does).  The block
// stages 1024 masses at a time in shared memory; warp 0 walks them 32 at a time: every lane
// rounds one mass to ulps, a warp sum gives the batch's end, and only a batch that leaves the
// binade, holds a tie or crosses M/2 is replayed one mass at a time by lane 0.  Haloes with a
// negative, -0.0 or non-finite mass walk with plain __dadd_rn.
__global__ void __launch_bounds__(256) red_walk_kernel(const int64_t *__restrict__ off, const int *__restrict__ order,
                                                       const double *__restrict__ dist, const double *__restrict__ m,
                                                       Red *__restrict__ red) {
    const int h = blockIdx.x;
    const int64_t b = off[h];
    const Red r = red[h];
    if (!isnan(r.r05)) return;   // caller supplied R05
    const int64_t nmem = (int64_t)r.n;
    const double half = 0.5 * r.mref;
    const int lane = threadIdx.x & 31;
    __shared__ double tile[2][1024];   // warp 0 walks one while the other warps fill the next
    __shared__ long long first;
    if (threadIdx.x == 0) first = LLONG_MAX;
    SeqSum q;   // lane 0's state (warp 0)
    q.c = 0.0;
    q.nrm = false;
    q.S = 0;
    q.hl = 0;
    q.e = 0;
    const bool plain = r.plain != 0.0;
    for (int i = threadIdx.x; i < (nmem < 1024 ? (int)nmem : 1024); i += blockDim.x) tile[0][i] = m[order[b + i]];
    __syncthreads();
    int cur = 0;
    for (int64_t k0 = 0; k0 < nmem; k0 += 1024, cur ^= 1) {
        const int cnt = nmem - k0 < 1024 ? (int)(nmem - k0) : 1024;
        if (threadIdx.x >= 32 && k0 + 1024 < nmem) {
            const int64_t k1 = k0 + 1024;
            const int cn = nmem - k1 < 1024 ? (int)(nmem - k1) : 1024;
            for (int i = threadIdx.x - 32; i < cn; i += blockDim.x - 32) tile[cur ^ 1][i] = m[order[b + k1 + i]];
        }
        if (threadIdx.x < 32) {
            long long f = LLONG_MAX;
            for (int q0 = 0; q0 < cnt && f == LLONG_MAX; q0 += 32) {
                const int nb = min(32, cnt - q0);
                bool replay = true;
                if (!plain) {
                    // lane 0's binade, broadcast; a batch from a non-normal sum is replayed
                    const int nrm = __shfl_sync(0xffffffffu, (int)q.nrm, 0);
                    if (nrm) {
                        const int e = __shfl_sync(0xffffffffu, q.e, 0);
                        long long fl = 0;
                        int code = 0;
                        bool big = false;
                        if (lane < nb) mass_ulps(tile[cur][q0 + lane], e, fl, code, big);
                        // increments without ties; a tie or a big mass forces the replay
                        const bool odd = big || code == 2;
                        long long inc = fl + (code == 1 ? 1 : 0);
                        for (int o = 16; o > 0; o >>= 1) inc += __shfl_xor_sync(0xffffffffu, inc, o);
                        if (!__any_sync(0xffffffffu, odd) && lane == 0) {
                            const long long T = q.S + inc;   // no overflow: inc < 32 * 2^53
                            if (T < kTwo53 && T <= q.hl) {
                                q.S = T;
                                replay = false;
                            }
                        }
                        replay = __shfl_sync(0xffffffffu, (int)replay, 0);
                    }
                }
                if (replay && lane == 0) {
                    for (int u = 0; u < nb; ++u) {
                        const bool over = plain ? ((q.c = __dadd_rn(q.c, tile[cur][q0 + u])) > half)
                                                : seq_add(q, tile[cur][q0 + u], half);
                        if (over) {
                            f = k0 + q0 + u;
                            break;
                        }
                    }
                }
                f = __shfl_sync(0xffffffffu, f, 0);
            }
            if (lane == 0 && f != LLONG_MAX) first = f;
        }
        __syncthreads();
        if (first != LLONG_MAX) break;
    }
    if (threadIdx.x == 0) {
        double r05 = 0.0;
        if (nmem > 0) {
            const long long f = first == LLONG_MAX ? -1 : first;
            if (f > 0) r05 = dist[order[b + f - 1]];
            else if (f == 0) r05 = dist[order[b]];
            else r05 = dist[order[b + nmem - 1]];
        }
        red[h].r05 = r05;
    }
}

// Per chunk: sum of |v - v_bulk|^2 and count of the members closer than R05.
__global__ void __launch_bounds__(256) red_sigma_kernel(int nh, const int64_t *__restrict__ off,
                                                        const int *__restrict__ cstart, const int *__restrict__ chunk_h,
                                                        const double *__restrict__ dist, const double *__restrict__ vx,
                                                        const double *__restrict__ vy, const double *__restrict__ vz,
                                                        const unsigned char *__restrict__ mask, const Red *__restrict__ red,
                                                        double *__restrict__ part) {
    Chunk k;
    if (!chunk_of(blockIdx.x, nh, off, cstart, chunk_h, k)) return;
    const Red r = red[k.h];
    __shared__ double sh[2][32];
    double v[2] = {0, 0};
    for (int64_t i = k.b + threadIdx.x; i < k.e; i += blockDim.x) {
        if (mask && !mask[i]) continue;
        if (dist[i] < r.r05) {
            const double dx = vx[i] - r.vx, dy = vy[i] - r.vy, dz = vz[i] - r.vz;
            v[0] += dx * dx + dy * dy + dz * dz;
            v[1] += 1.0;
        }
    }
    bsum<2>(v, sh);
    if (threadIdx.x < 2) part[(int64_t)blockIdx.x * 2 + threadIdx.x] = v[threadIdx.x];
}

__global__ void red_out_kernel(int nh, const int *__restrict__ cstart, const double *__restrict__ part,
                               const Red *__restrict__ red, double *__restrict__ out) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < nh; h += gridDim.x * blockDim.x) {
        const Red r = red[h];
        double s = 0.0, c = 0.0;
        for (int k = cstart[h]; k < cstart[h + 1]; ++k) {
            s += part[(int64_t)k * 2];
            c += part[(int64_t)k * 2 + 1];
        }
        double *o = out + (int64_t)h * HALMA_RED_NFIELDS;
        o[HALMA_RED_MASS] = r.M;
        o[HALMA_RED_CX] = r.cx; o[HALMA_RED_CY] = r.cy; o[HALMA_RED_CZ] = r.cz;
        o[HALMA_RED_VX] = r.vx; o[HALMA_RED_VY] = r.vy; o[HALMA_RED_VZ] = r.vz;
        o[HALMA_RED_RMAX] = r.rmax;
        o[HALMA_RED_R05] = r.r05;
        o[HALMA_RED_SIGMA] = c > 0 ? sqrt(s / 3.0 / c) : 0.0;
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
    if (nh <= 0) return HALMA_OK;
    const int N = (int)std::max<int64_t>(n, 1);
    const int cmax = nh + (int)(n / kRedChunk) + 1;   // chunks: sum over haloes of max(1, ceil(n_h / kRedChunk))
    const size_t s64 = sort_pairs_u64_i32_bytes(N, 64), s32 = sort_pairs_u32_i32_bytes(N);
    const size_t sc = exclusive_sum_i32_bytes(nh + 1);
    Layout L;
    const size_t o_red = L.add(sizeof(Red) * nh);
    const size_t o_dk = L.add(8ull * N), o_dk2 = L.add(8ull * N), o_dist = L.add(8ull * N);
    const size_t o_hid = L.add(4ull * N), o_hid2 = L.add(4ull * N), o_hid3 = L.add(4ull * N);
    const size_t o_v0 = L.add(4ull * N), o_v1 = L.add(4ull * N), o_v2 = L.add(4ull * N);
    const size_t o_cnum = L.add(4ull * (nh + 1)), o_cst = L.add(4ull * (nh + 1)), o_ch = L.add(4ull * cmax);
    const size_t o_part = L.add(8ull * kRedParts * cmax), o_part2 = L.add(16ull * cmax);
    const size_t o_tmp = L.add(std::max(std::max(s64, s32), sc));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st));
    Red *red = at<Red>(base, o_red);
    auto *dk = at<uint64_t>(base, o_dk), *dk2 = at<uint64_t>(base, o_dk2);
    auto *dist = at<double>(base, o_dist);
    auto *hid = at<uint32_t>(base, o_hid), *hid2 = at<uint32_t>(base, o_hid2), *hid3 = at<uint32_t>(base, o_hid3);
    auto *v0 = at<int>(base, o_v0), *v1 = at<int>(base, o_v1), *v2 = at<int>(base, o_v2);
    int *cnum = at<int>(base, o_cnum), *cst = at<int>(base, o_cst), *chunk_h = at<int>(base, o_ch);
    double *part = at<double>(base, o_part), *part2 = at<double>(base, o_part2);
    void *tmp = at<void>(base, o_tmp);
    const int gh = grid_for(nh + 1, 256);
    HALMA_LAUNCH(red_chunks_kernel, gh, 256, 0, st, nh, off, cnum);
    HALMA_TRY(exclusive_sum_i32(tmp, sc, cnum, cst, nh + 1, st));
    HALMA_LAUNCH(red_owner_kernel, gh, 256, 0, st, nh, cst, chunk_h);
    HALMA_LAUNCH(red_part_kernel, cmax, 256, 0, st, nh, off, cst, chunk_h, x, y, z, vx, vy, vz, m, mask, part);
    HALMA_LAUNCH(red_center_kernel, gh, 256, 0, st, nh, cst, part, about, red);
    HALMA_LAUNCH(red_dist_kernel, cmax, 256, 0, st, nh, off, cst, chunk_h, x, y, z, mask, red, dk, dist, hid);
    if (n > 0) {
        const int g = std::min(device_sm_count() * 8, grid_for(n, 256));
        HALMA_LAUNCH(iota_kernel, g, 256, 0, st, n, v0);
        HALMA_TRY(sort_pairs_u64_i32(tmp, s64, dk, dk2, v0, v1, (int)n, 64, st));
        HALMA_LAUNCH(gather_hid_kernel, g, 256, 0, st, n, v1, hid, hid2);
        int hbits = 1;   // halo ids are < nh: sort only their bits
        while (hbits < 32 && ((uint64_t)(nh - 1) >> hbits) != 0) ++hbits;
        HALMA_TRY(sort_pairs_u32_i32(tmp, s32, hid2, hid3, v1, v2, (int)n, hbits, st));
    }
    HALMA_LAUNCH(red_walk_kernel, nh, 256, 0, st, off, v2, dist, m, red);
    HALMA_LAUNCH(red_sigma_kernel, cmax, 256, 0, st, nh, off, cst, chunk_h, dist, vx, vy, vz, mask, red, part2);
    HALMA_LAUNCH(red_out_kernel, gh, 256, 0, st, nh, cst, part2, red, out);
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
    cudaStream_t st = (cudaStream_t)stream;
    // the segments must cover the n rows in order (checked on the host: the kernels size
    // their chunk table from n, index the rows through the offsets and sort all n rows by
    // the halo each belongs to)
    {
        std::vector<int64_t> h_off(n_haloes + 1);
        if (is_device_pointer(offsets)) {
            HALMA_CUDA(cudaMemcpyAsync(h_off.data(), offsets, 8ull * (n_haloes + 1), cudaMemcpyDeviceToHost, st));
            HALMA_CUDA(cudaStreamSynchronize(st));
        } else {
            memcpy(h_off.data(), offsets, 8ull * (n_haloes + 1));
        }
        if (h_off[0] != 0 || h_off[n_haloes] != n) return fail(HALMA_ERR_INVALID, "halo offsets must run from 0 to n");
        for (int64_t h = 0; h < n_haloes; ++h)
            if (h_off[h + 1] < h_off[h]) return fail(HALMA_ERR_INVALID, "halo offsets must not decrease");
    }
    std::lock_guard<std::mutex> guard(api_mutex());
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
