// The O(N) per-halo properties of pyHALMA's property loop (pyHALMA.py:930-1016) for all
// groups at once:
//   half-mass radius, 3-D and projected  (halo_properties.py:365-392, 397-458)
//   bulk velocity                        (CM_velocity, :45-60)
//   specific angular momentum            (angular_momentum, :461-481; its z component is
//                                         sum m (rx*vvy - ry*vvz) / M, as in the reference)
//   Tully-Fisher velocity                (tully_fisher_velocity, :62-96)
//   kappa_co                             (kinematic_morphology, :483-515)
//   shape semi-axes                      (halo_shape_fortran :852-866 -> particle_subroutines
//                                         .f90:160-214: FP32 inertia tensor, Jacobi in FP64)
//   sigma inside R05                     (sigma_effective, :607-625)
//   projected sigma, V/sigma, lambda     (sigma_projections_fortran :781-814 -> f90:217-461)
//
// FP64 sums (the reference's numba loops run with fastmath, order unspecified) are reduced per
// block.  The FP32 Fortran parts are summed in the Fortran's own order with every operation
// rounded on its own, so they equal a one-thread run of the Fortran: the inertia tensor by
// one thread per group over its particles, the projected cells after a stable sort by
// (group, projection, cell) with one thread per cell, and the V/sigma and lambda sums by one
// thread per group and projection over its cells in the Fortran's loop order (empty cells add
// exact zeros there and are skipped here).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

constexpr int kCenFields = 5;   // cx, cy, cz, mass, rmax per group (the cleaning's outputs)

__global__ void pr_gather_kernel(int64_t nm, const int *__restrict__ mem, const double *__restrict__ x,
                                 const double *__restrict__ y, const double *__restrict__ z,
                                 const double *__restrict__ vx, const double *__restrict__ vy,
                                 const double *__restrict__ vz, const double *__restrict__ m,
                                 double *__restrict__ g /* 8 x nm: x y z vx vy vz m 0 */) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = mem[k];
        g[k] = x[i];
        g[nm + k] = y[i];
        g[2 * nm + k] = z[i];
        g[3 * nm + k] = vx[i];
        g[4 * nm + k] = vy[i];
        g[5 * nm + k] = vz[i];
        g[6 * nm + k] = m[i];
        g[7 * nm + k] = 0.0;
    }
}

template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double (*sh)[8]) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
        if (lane == 0) sh[q][w] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double t = 0.0;
        for (int k = 0; k < nw; ++k) t += sh[q][k];
        v[q] = t;
    }
    __syncthreads();
}

// Bulk velocity (sum m v / M with the given mass, zeros when M <= 0) and the "about" rows of
// the four half-mass-radius reductions: 3-D around (cx, cy, cz), and the projections along x,
// y, z as 3-D distances of (y, z, 0), (x, z, 0), (x, y, 0) around (cy, cz, 0), (cx, cz, 0),
// (cx, cy, 0).
__global__ void __launch_bounds__(256) pr_bulk_kernel(int G, const int64_t *__restrict__ off,
                                                      const double *__restrict__ g, int64_t nm,
                                                      const double *__restrict__ cen, double *__restrict__ out,
                                                      double *__restrict__ about /* 4 x G x 8 */) {
    __shared__ double sh[3][8];
    for (int h = blockIdx.x; h < G; h += gridDim.x) {
        double v[3] = {0, 0, 0};
        for (int64_t k = off[h] + threadIdx.x; k < off[h + 1]; k += blockDim.x) {
            const double mi = g[6 * nm + k];
            v[0] += mi * g[3 * nm + k];
            v[1] += mi * g[4 * nm + k];
            v[2] += mi * g[5 * nm + k];
        }
        block_sums<3>(v, sh);
        if (threadIdx.x == 0) {
            const double *c = cen + (int64_t)h * kCenFields;
            const double M = c[3];
            const double ux = M > 0.0 ? v[0] / M : 0.0, uy = M > 0.0 ? v[1] / M : 0.0, uz = M > 0.0 ? v[2] / M : 0.0;
            double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
            o[HALMA_PROP_VX] = ux;
            o[HALMA_PROP_VY] = uy;
            o[HALMA_PROP_VZ] = uz;
            const double cc[4][3] = {{c[0], c[1], c[2]}, {c[1], c[2], 0.0}, {c[0], c[2], 0.0}, {c[0], c[1], 0.0}};
            for (int r = 0; r < 4; ++r) {
                double *a = about + ((int64_t)r * G + h) * HALMA_ABOUT_NFIELDS;
                a[HALMA_ABOUT_CX] = cc[r][0];
                a[HALMA_ABOUT_CY] = cc[r][1];
                a[HALMA_ABOUT_CZ] = cc[r][2];
                a[HALMA_ABOUT_VX] = ux;
                a[HALMA_ABOUT_VY] = uy;
                a[HALMA_ABOUT_VZ] = uz;
                a[HALMA_ABOUT_MASS] = M;
                a[HALMA_ABOUT_R05] = NAN;
            }
        }
        __syncthreads();
    }
}

// Jacobi diagonalisation of particle_subroutines.f90:12-126 (REAL*8 on the REAL*4 tensor),
// every operation rounded on its own; out = eigenvalues as REAL*4.
__device__ void jacobi3(const float in[3][3], float out[3]) {
    double a[3][3], eig[3], b[3], zz[3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = (double)in[i][j];
    for (int i = 0; i < 3; ++i) {
        b[i] = a[i][i];
        eig[i] = b[i];
        zz[i] = 0.0;
    }
    double sum_el = 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) sum_el = __dadd_rn(sum_el, fabs(a[i][j]));
    for (int it = 1; it <= 100; ++it) {
        double suma = 0.0;
        for (int i = 0; i < 2; ++i)
            for (int j = i + 1; j < 3; ++j) suma = __dadd_rn(suma, fabs(a[i][j]));
        if (suma < __dmul_rn((double)1.e-4f, sum_el)) break;
        const double upper = it < 4 ? __dmul_rn(0.2, __dmul_rn(suma, suma)) : 0.0;
        for (int ip = 0; ip < 2; ++ip) {
            for (int iq = ip + 1; iq < 3; ++iq) {
                const double var1 = __dmul_rn(100.0, fabs(a[ip][iq]));
                if (it > 4 && __dadd_rn(fabs(eig[ip]), var1) == fabs(eig[ip]) &&
                    __dadd_rn(fabs(eig[iq]), var1) == fabs(eig[iq])) {
                    a[ip][iq] = 0.0;
                } else if (fabs(a[ip][iq]) > upper) {
                    double var2 = __dsub_rn(eig[iq], eig[ip]);
                    double t;
                    if (__dadd_rn(fabs(var2), var1) == fabs(var2)) {
                        t = __ddiv_rn(a[ip][iq], var2);
                    } else {
                        const double theta = __ddiv_rn(__dmul_rn(0.5, var2), a[ip][iq]);
                        t = __ddiv_rn(1.0, __dadd_rn(fabs(theta), __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(theta, theta)))));
                        if (theta < 0.0) t = -t;
                    }
                    const double c = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(1.0, __dmul_rn(t, t))));
                    const double s = __dmul_rn(t, c);
                    const double tau = __ddiv_rn(s, __dadd_rn(1.0, c));
                    var2 = __dmul_rn(t, a[ip][iq]);
                    zz[ip] = __dsub_rn(zz[ip], var2);
                    zz[iq] = __dadd_rn(zz[iq], var2);
                    eig[ip] = __dsub_rn(eig[ip], var2);
                    eig[iq] = __dadd_rn(eig[iq], var2);
                    a[ip][iq] = 0.0;
                    // g - s (h + g tau), h + s (g - h tau)
#define ROT(G_, H_)                                                                              \
    {                                                                                           \
        const double gg = G_, hh = H_;                                                          \
        G_ = __dsub_rn(gg, __dmul_rn(s, __dadd_rn(hh, __dmul_rn(gg, tau))));                    \
        H_ = __dadd_rn(hh, __dmul_rn(s, __dsub_rn(gg, __dmul_rn(hh, tau))));                    \
    }
                    for (int j = 0; j < ip; ++j) ROT(a[j][ip], a[j][iq]);
                    for (int j = ip + 1; j < iq; ++j) ROT(a[ip][j], a[j][iq]);
                    for (int j = iq + 1; j < 3; ++j) ROT(a[ip][j], a[iq][j]);
#undef ROT
                }
            }
        }
        for (int i = 0; i < 3; ++i) {
            b[i] = __dadd_rn(b[i], zz[i]);
            eig[i] = b[i];
            zz[i] = 0.0;
        }
    }
    for (int i = 0; i < 3; ++i) out[i] = (float)eig[i];
}

constexpr int kTile = 1024;

// Block per group: the FP32 inertia tensor in particle order (f90:183-200), its
// normalisation, Jacobi, the decreasing sort (f90:129-157) and the square roots.  Members
// are staged in shared memory a tile at a time; the nine tensor sums and the mass sum are
// independent chains, so threads 0..9 each add one of them in member order.
__global__ void __launch_bounds__(256) pr_shape_kernel(int G, const int64_t *__restrict__ off,
                                                       const double *__restrict__ g, int64_t nm,
                                                       const double *__restrict__ cen, double *__restrict__ out) {
    __shared__ float sr[4][kTile];   // x, y, z relative to the centre (FP32), mass
    __shared__ float acc[10];
    for (int h = blockIdx.x; h < G; h += gridDim.x) {
        const double *c = cen + (int64_t)h * kCenFields;
        const int t = threadIdx.x;
        float a = 0.f;   // thread t < 9: it[t % 3][t / 3]; thread 9: mass
        for (int64_t b = off[h]; b < off[h + 1]; b += kTile) {
            const int cnt = (off[h + 1] - b < kTile ? (int)(off[h + 1] - b) : kTile);
            for (int q = t; q < cnt; q += blockDim.x) {
                const int64_t k = b + q;
                sr[0][q] = (float)__dsub_rn(g[k], c[0]);
                sr[1][q] = (float)__dsub_rn(g[nm + k], c[1]);
                sr[2][q] = (float)__dsub_rn(g[2 * nm + k], c[2]);
                sr[3][q] = (float)g[6 * nm + k];
            }
            __syncthreads();
            if (t < 9) {
                const int i = t % 3, j = t / 3;
                for (int q = 0; q < cnt; ++q) a = __fadd_rn(a, __fmul_rn(__fmul_rn(sr[3][q], sr[i][q]), sr[j][q]));
            } else if (t == 9) {
                for (int q = 0; q < cnt; ++q) a = __fadd_rn(a, sr[3][q]);
            }
            __syncthreads();
        }
        if (t < 10) acc[t] = a;
        __syncthreads();
        if (t == 0) {
            float it[3][3];
            for (int j = 0; j < 3; ++j)
                for (int i = 0; i < 3; ++i) it[i][j] = __fdiv_rn(acc[i + 3 * j], acc[9]);
            float e[3];
            jacobi3(it, e);
            for (int ii = 0; ii < 2; ++ii) {   // SORT_EIGEN
                int kk = ii;
                float v = e[ii];
                for (int jj = ii + 1; jj < 3; ++jj)
                    if (e[jj] >= v) {
                        kk = jj;
                        v = e[jj];
                    }
                if (kk != ii) {
                    e[kk] = e[ii];
                    e[ii] = v;
                }
            }
            double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
            o[HALMA_PROP_SA] = (double)__fsqrt_rn(e[0]);
            o[HALMA_PROP_SB] = (double)__fsqrt_rn(e[1]);
            o[HALMA_PROP_SC] = (double)__fsqrt_rn(e[2]);
        }
        __syncthreads();
    }
}

// Specific angular momentum (with the reference's z component), then kappa_co and the
// Tully-Fisher velocity about it.
// A group's members are split over up to S blocks of at least kKinMin (the FP64 work per member
// is heavy and GB300's FP64 pipe is narrow, so one block per group would leave the biggest
// group's SM as the critical path); each block writes partial sums and the last block of the
// group to finish (a per-group counter, no waiting) adds them in block order.
constexpr int kKinMin = 2048;

__device__ __forceinline__ bool kin_part_of(int bid, int S, int G, const int64_t *__restrict__ off, int &h, int &sh,
                                            int64_t &b, int64_t &e) {
    h = bid / S;
    const int s = bid % S;
    if (h >= G) return false;
    const int64_t b0 = off[h], len = off[h + 1] - b0;
    sh = (int)std::min<int64_t>(S, std::max<int64_t>(1, (len + kKinMin - 1) / kKinMin));
    if (s >= sh) return false;
    b = b0 + len * s / sh;
    e = b0 + len * (s + 1) / sh;
    return true;
}

// Phase 1: angular momentum (halo_properties.py:461-482); the last block stores j, |j| and the
// unit vector for phase 2.
__global__ void __launch_bounds__(256) pr_kin1_kernel(int G, int S, const int64_t *__restrict__ off,
                                                      const double *__restrict__ g, int64_t nm,
                                                      const double *__restrict__ cen, const double *__restrict__ out,
                                                      double *__restrict__ part, int *__restrict__ ctr,
                                                      double *__restrict__ jvec) {
    int h, sh;
    int64_t b, e;
    if (!kin_part_of(blockIdx.x, S, G, off, h, sh, b, e)) return;
    __shared__ double sm[4][8];
    __shared__ int last;
    const double *c = cen + (int64_t)h * kCenFields;
    const double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
    const double ux = o[HALMA_PROP_VX], uy = o[HALMA_PROP_VY], uz = o[HALMA_PROP_VZ];
    double l[3] = {0, 0, 0};
    for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
        const double rx = g[k] - c[0], ry = g[nm + k] - c[1], rz = g[2 * nm + k] - c[2];
        const double vvx = g[3 * nm + k] - ux, vvy = g[4 * nm + k] - uy, vvz = g[5 * nm + k] - uz;
        const double mk = g[6 * nm + k];
        l[0] += mk * (ry * vvz - rz * vvy);
        l[1] += mk * (rz * vvx - rx * vvz);
        l[2] += mk * (rx * vvy - ry * vvz);   // as angular_momentum (halo_properties.py:478)
    }
    block_sums<3>(l, sm);
    if (threadIdx.x == 0) {
        const int s = blockIdx.x % S;
        for (int q = 0; q < 3; ++q) part[((int64_t)h * S + s) * 4 + q] = l[q];
        __threadfence();
        last = atomicAdd(ctr + h, 1) == sh - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double t[3] = {0, 0, 0};
        for (int s = 0; s < sh; ++s)
            for (int q = 0; q < 3; ++q) t[q] += __ldcg(part + ((int64_t)h * S + s) * 4 + q);
        const double M = c[3];
        const double jx = t[0] / M, jy = t[1] / M, jz = t[2] / M;
        const double jn = sqrt(jx * jx + jy * jy + jz * jz);
        double *jv = jvec + (int64_t)h * 8;
        jv[0] = jx;
        jv[1] = jy;
        jv[2] = jz;
        jv[3] = jn;
        jv[4] = jx / jn;
        jv[5] = jy / jn;
        jv[6] = jz / jn;
        ctr[h] = 0;
    }
}

// Phase 2: kappa_co (kinematic_morphology, halo_properties.py:483-517) and the Tully-Fisher
// shell velocity (tully_fisher_velocity, :63-96); the last block writes the group's outputs.
__global__ void __launch_bounds__(256) pr_kin2_kernel(int G, int S, const int64_t *__restrict__ off,
                                                      const double *__restrict__ g, int64_t nm,
                                                      const double *__restrict__ cen, double *__restrict__ out,
                                                      double *__restrict__ part, int *__restrict__ ctr,
                                                      const double *__restrict__ jvec) {
    int h, sh;
    int64_t b, e;
    if (!kin_part_of(blockIdx.x, S, G, off, h, sh, b, e)) return;
    __shared__ double sm[4][8];
    __shared__ int last;
    const double *c = cen + (int64_t)h * kCenFields;
    double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
    const double ux = o[HALMA_PROP_VX], uy = o[HALMA_PROP_VY], uz = o[HALMA_PROP_VZ];
    const double r05 = o[HALMA_PROP_R05];
    const double *jv = jvec + (int64_t)h * 8;
    const double ex = jv[4], ey = jv[5], ez = jv[6];
    double s[4] = {0, 0, 0, 0};   // kin_corot, kin_total, v_TF, mass in the shell
    for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
        const double rx = g[k] - c[0], ry = g[nm + k] - c[1], rz = g[2 * nm + k] - c[2];
        const double vvx = g[3 * nm + k] - ux, vvy = g[4 * nm + k] - uy, vvz = g[5 * nm + k] - uz;
        const double mk = g[6 * nm + k];
        const double llx = mk * (ry * vvz - rz * vvy), lly = mk * (rz * vvx - rx * vvz),
                     llz = mk * (rx * vvy - ry * vvx);
        const double lz = llx * ex + lly * ey + llz * ez;
        const double zi = rx * ex + ry * ey + rz * ez;
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double R = sqrt(r2 - zi * zi);
        s[1] += 0.5 * mk * (vvx * vvx + vvy * vvy + vvz * vvz);
        if (lz > 0.0) {
            const double q = lz / (mk * R);
            s[0] += 0.5 * mk * q * q;
        }
        const double dist = sqrt(r2);
        if (0.9 * r05 < dist && dist < 1.1 * r05) {
            // R_ip = r - (r.u)u, u_R = R_ip/|R_ip|, v_rot = v - (v.u)u - (v.u_R)u_R
            const double Rx = rx - zi * ex, Ry = ry - zi * ey, Rz = rz - zi * ez;
            const double Rn = sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
            const double qx = Rx / Rn, qy = Ry / Rn, qz = Rz / Rn;
            const double vu = vvx * ex + vvy * ey + vvz * ez, vq = vvx * qx + vvy * qy + vvz * qz;
            const double wx = vvx - vu * ex - vq * qx, wy = vvy - vu * ey - vq * qy, wz = vvz - vu * ez - vq * qz;
            s[2] += sqrt(wx * wx + wy * wy + wz * wz) * mk;
            s[3] += mk;
        }
    }
    block_sums<4>(s, sm);
    if (threadIdx.x == 0) {
        const int sb = blockIdx.x % S;
        for (int q = 0; q < 4; ++q) part[((int64_t)h * S + sb) * 4 + q] = s[q];
        __threadfence();
        last = atomicAdd(ctr + h, 1) == sh - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        double t[4] = {0, 0, 0, 0};
        for (int q0 = 0; q0 < sh; ++q0)
            for (int q = 0; q < 4; ++q) t[q] += __ldcg(part + ((int64_t)h * S + q0) * 4 + q);
        o[HALMA_PROP_JX] = jv[0];
        o[HALMA_PROP_JY] = jv[1];
        o[HALMA_PROP_JZ] = jv[2];
        o[HALMA_PROP_J] = jv[3];
        o[HALMA_PROP_KCO] = t[0] / t[1];
        o[HALMA_PROP_VTF] = t[2] / t[3];   // NaN when no particle lies in 0.9..1.1 R05
        ctr[h] = 0;
    }
}

// --- projected dispersion, V/sigma and lambda (f90:217-461), FP32 -----------------------
struct ProjGrid {
    double start, next, delta, step;
    long long n;
};

__device__ __forceinline__ ProjGrid proj_grid(double rmax, double ll) {
    // np.arange(-(rmax + ll), rmax + ll, 2 ll)
    ProjGrid p;
    const double stop = __dadd_rn(rmax, ll);
    p.start = -stop;
    p.step = __dmul_rn(2.0, ll);
    p.next = __dadd_rn(p.start, p.step);
    p.delta = __dsub_rn(p.next, p.start);
    p.n = (long long)ceil(__ddiv_rn(__dsub_rn(stop, p.start), p.step));
    if (p.n < 1) p.n = 1;
    return p;
}

__device__ __forceinline__ float grid32(const ProjGrid &p, long long i) {
    const double v = i == 0 ? p.start : (i == 1 ? p.next : __dadd_rn(p.start, __dmul_rn((double)i, p.delta)));
    return (float)v;
}

// minloc(abs(grid - v)): first index of the smallest |grid(i) - v| in FP32
__device__ __forceinline__ int minloc32(const ProjGrid &p, float v) {
    long long k = (long long)floor(((double)v - p.start) / p.step + 0.5);
    k = k < 0 ? 0 : (k > p.n - 1 ? p.n - 1 : k);
    long long best = k;
    float bd = fabsf(__fsub_rn(grid32(p, k), v));
    for (long long q = k - 1; q <= k + 1; q += 2) {
        if (q < 0 || q >= p.n) continue;
        const float d = fabsf(__fsub_rn(grid32(p, q), v));
        if (d < bd || (d == bd && q < best)) {
            bd = d;
            best = q;
        }
    }
    return (int)best;
}

// Per member and projection: the cell (inner + outer * n, inner running fastest as in the
// Fortran loops of the V/sigma sums) and the sort key (group, projection, cell).
//   projection 0 (x, plane YZ): cell (iy, iz);  1 (y, XZ): (ix, iz);  2 (z, XY): (ix, iy)
__global__ void pr_pkeys_kernel(int64_t nm, int G, const int64_t *__restrict__ off, const int *__restrict__ owner,
                                const double *__restrict__ g, const double *__restrict__ cen, double ll, int cbits,
                                uint64_t *__restrict__ keys, int *__restrict__ vals) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x) {
        const int h = owner[k];
        const double *c = cen + (int64_t)h * kCenFields;
        const ProjGrid p = proj_grid(c[4], ll);
        const int ix = minloc32(p, __fsub_rn((float)g[k], (float)c[0]));
        const int iy = minloc32(p, __fsub_rn((float)g[nm + k], (float)c[1]));
        const int iz = minloc32(p, __fsub_rn((float)g[2 * nm + k], (float)c[2]));
        const uint64_t cell[3] = {(uint64_t)iy + (uint64_t)iz * p.n, (uint64_t)ix + (uint64_t)iz * p.n,
                                  (uint64_t)ix + (uint64_t)iy * p.n};
        for (int a = 0; a < 3; ++a) {
            keys[a * nm + k] = ((uint64_t)(3 * (int64_t)h + a) << cbits) | cell[a];
            vals[a * nm + k] = (int)(a * nm + k);
        }
    }
}

__global__ void pr_head_kernel(int64_t n, const uint64_t *__restrict__ keys, int *__restrict__ head) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        head[k] = (k == 0 || keys[k] != keys[k - 1]) ? 1 : 0;
}

// Cell starts: runstart[r] = first sorted entry of cell r, runstart[ncell] = n3.
__global__ void pr_runstart_kernel(int64_t n3, const int *__restrict__ head, const int *__restrict__ rpos,
                                   int *__restrict__ runstart) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n3; k += (int64_t)gridDim.x * blockDim.x) {
        if (head[k]) runstart[rpos[k]] = (int)k;
        if (k == n3 - 1) runstart[rpos[k] + head[k]] = (int)n3;
    }
}

// One warp per cell: FP32 mass SD, mass-weighted velocity VCM (then / SD), count, and
// sigma = sqrt(sum (v - VCM)^2 / count), members in order: the lanes load 32 members at a
// time and every lane adds them one by one (shuffles), so the sums are the sequential ones;
// rid[member entry] = cell.
__global__ void pr_cells_kernel(int ncell, int64_t nm, const int *__restrict__ runstart,
                                const uint64_t *__restrict__ keys, const int *__restrict__ vals,
                                const int *__restrict__ owner, const double *__restrict__ g,
                                const double *__restrict__ out, float4 *__restrict__ cellv,
                                uint64_t *__restrict__ cellkey, int *__restrict__ rid) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; r < ncell; r += warps) {
        const int b = runstart[r], e = runstart[r + 1];
        const int a = vals[b] / (int)nm;   // projection of the cell
        float sd = 0.f, vc = 0.f;
        for (int k0 = b; k0 < e; k0 += 32) {
            const int k = k0 + lane;
            float v = 0.f, m = 0.f;
            if (k < e) {
                const int mk = vals[k] - a * (int)nm;
                const double *o = out + (int64_t)owner[mk] * HALMA_PROP_NFIELDS;
                v = (float)__dsub_rn(g[(3 + a) * nm + mk], o[HALMA_PROP_VX + a]);
                m = (float)g[6 * nm + mk];
                rid[vals[k]] = (int)r;
            }
            const int cnt = e - k0 < 32 ? e - k0 : 32;
            for (int t = 0; t < cnt; ++t) {
                const float vt = __shfl_sync(0xffffffffu, v, t), mt = __shfl_sync(0xffffffffu, m, t);
                vc = __fadd_rn(vc, __fmul_rn(vt, mt));
                sd = __fadd_rn(sd, mt);
            }
        }
        if (sd != 0.f) vc = __fdiv_rn(vc, sd);
        float s2 = 0.f;
        for (int k0 = b; k0 < e; k0 += 32) {
            const int k = k0 + lane;
            float d2 = 0.f;
            if (k < e) {
                const int mk = vals[k] - a * (int)nm;
                const double *o = out + (int64_t)owner[mk] * HALMA_PROP_NFIELDS;
                const float d = __fsub_rn((float)__dsub_rn(g[(3 + a) * nm + mk], o[HALMA_PROP_VX + a]), vc);
                d2 = __fmul_rn(d, d);
            }
            const int cnt = e - k0 < 32 ? e - k0 : 32;
            for (int t = 0; t < cnt; ++t) s2 = __fadd_rn(s2, __shfl_sync(0xffffffffu, d2, t));
        }
        if (lane == 0) {
            cellv[r] = make_float4(sd, vc, __fsqrt_rn(__fdiv_rn(s2, (float)(e - b))), 0.f);
            cellkey[r] = keys[b];
        }
    }
}

__device__ __forceinline__ int lower_bound_key(const uint64_t *__restrict__ keys, int n, uint64_t k) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (keys[mid] < k) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Block per group: per projection the mean cell sigma over the members inside the projected
// half-mass radius (members in order), and the V/sigma and lambda sums over the group's cells
// with R_cell < R05 + 2 ll in the Fortran's loop order.  Tiles of members (then of cells) are
// staged in shared memory by the whole block; each sum is then added in order by one thread
// (three for the sigma sums, four per projection for the V/sigma and lambda sums).
__global__ void __launch_bounds__(256) pr_proj_kernel(int G, int64_t nm, const int64_t *__restrict__ off,
                                                      const double *__restrict__ g, const double *__restrict__ cen,
                                                      double ll, int cbits, const int *__restrict__ rid,
                                                      const float4 *__restrict__ cellv,
                                                      const uint64_t *__restrict__ cellkey, int ncell,
                                                      float *__restrict__ res /* G x 3 x 3 */) {
    __shared__ float term[4][kTile];
    __shared__ float red[12];
    const int t = threadIdx.x;
    for (int h = blockIdx.x; h < G; h += gridDim.x) {
        const double *c = cen + (int64_t)h * kCenFields;
        const ProjGrid p = proj_grid(c[4], ll);
        const float cx = (float)c[0], cy = (float)c[1], cz = (float)c[2];
        float r05[3];
        for (int a = 0; a < 3; ++a) r05[a] = res[((int64_t)h * 3 + a) * 3];
        // mean cell sigma inside R05: term[a] = the member's cell sigma (or -1 outside)
        float s05 = 0.f;
        int cnt = 0;
        for (int64_t b = off[h]; b < off[h + 1]; b += kTile) {
            const int nt = (off[h + 1] - b < kTile ? (int)(off[h + 1] - b) : kTile);
            for (int q = t; q < nt; q += blockDim.x) {
                const int64_t k = b + q;
                const float dx = __fsub_rn((float)g[k], cx), dy = __fsub_rn((float)g[nm + k], cy),
                            dz = __fsub_rn((float)g[2 * nm + k], cz);
                const float d2[3] = {__fadd_rn(__fmul_rn(dy, dy), __fmul_rn(dz, dz)),
                                     __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dz, dz)),
                                     __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy))};
                for (int a = 0; a < 3; ++a)
                    term[a][q] = __fsqrt_rn(d2[a]) < r05[a] ? cellv[rid[a * nm + k]].z : -1.f;
            }
            __syncthreads();
            if (t < 3)
                for (int q = 0; q < nt; ++q)
                    if (term[t][q] >= 0.f) {
                        s05 = __fadd_rn(s05, term[t][q]);
                        cnt += 1;
                    }
            __syncthreads();
        }
        if (t < 3) red[t] = cnt > 0 ? __fdiv_rn(s05, (float)cnt) : s05;
        __syncthreads();
        // V/sigma and lambda per projection: term[q] of every cell of the tile (0 outside)
        for (int a = 0; a < 3; ++a) {
            const float lim = __fadd_rn(r05[a], __fmul_rn(2.f, (float)ll));
            const uint64_t k0 = (uint64_t)(3 * (int64_t)h + a) << cbits, k1 = (uint64_t)(3 * (int64_t)h + a + 1) << cbits;
            __shared__ int range[2];
            if (t == 0) {
                int lo = 0, hi = ncell;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cellkey[mid] < k0) lo = mid + 1;
                    else hi = mid;
                }
                int e = lo, hi2 = ncell;
                while (e < hi2) {
                    const int mid = (e + hi2) >> 1;
                    if (cellkey[mid] < k1) e = mid + 1;
                    else hi2 = mid;
                }
                range[0] = lo;
                range[1] = e;
            }
            __syncthreads();
            const int r0 = range[0], r1 = range[1];
            float sum = 0.f;   // thread q < 4: sumV, sumSigma, sumUp, sumDown
            for (int b = r0; b < r1; b += kTile) {
                const int nt = min(kTile, r1 - b);
                for (int q = t; q < nt; q += blockDim.x) {
                    const int r = b + q;
                    const uint64_t cell = cellkey[r] - k0;
                    const float gi = grid32(p, (long long)(cell % (uint64_t)p.n)),
                                go = grid32(p, (long long)(cell / (uint64_t)p.n));
                    const float rbin = __fsqrt_rn(__fadd_rn(__fmul_rn(gi, gi), __fmul_rn(go, go)));
                    const float4 cv = cellv[r];   // (SD, VCM, SIG)
                    const bool in = rbin < lim;
                    term[0][q] = in ? __fmul_rn(__fmul_rn(cv.y, cv.y), cv.x) : -1.f;
                    term[1][q] = __fmul_rn(__fmul_rn(cv.z, cv.z), cv.x);
                    term[2][q] = __fmul_rn(__fmul_rn(cv.x, rbin), fabsf(cv.y));
                    term[3][q] = __fmul_rn(__fmul_rn(cv.x, rbin),
                                           __fsqrt_rn(__fadd_rn(__fmul_rn(cv.y, cv.y), __fmul_rn(cv.z, cv.z))));
                }
                __syncthreads();
                if (t < 4)
                    for (int q = 0; q < nt; ++q)
                        if (term[0][q] >= 0.f) sum = __fadd_rn(sum, term[t][q]);
                __syncthreads();
            }
            if (t < 4) red[3 + t] = sum;
            __syncthreads();
            if (t == 0) {
                float *o = res + ((int64_t)h * 3 + a) * 3;
                o[0] = red[a];
                o[1] = red[4] > 0.f ? __fsqrt_rn(__fdiv_rn(red[3], red[4])) : 0.f;
                o[2] = red[6] > 0.f ? __fdiv_rn(red[5], red[6]) : 0.f;
            }
            __syncthreads();
        }
    }
}

__global__ void pr_fill_kernel(int G, const int64_t *__restrict__ off, int *__restrict__ owner) {
    for (int h = blockIdx.x; h < G; h += gridDim.x)
        for (int64_t e = off[h] + threadIdx.x; e < off[h + 1]; e += blockDim.x) owner[e] = h;
}

// Half-mass radii and sigma_effective from the reductions, and the projected R05 in FP32 for
// the projection sums.
__global__ void pr_r05_kernel(int G, const double *__restrict__ red /* 4 x G x NF */, double *__restrict__ out,
                              float *__restrict__ res) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < G; h += gridDim.x * blockDim.x) {
        double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
        o[HALMA_PROP_R05] = red[(int64_t)h * HALMA_RED_NFIELDS + HALMA_RED_R05];
        o[HALMA_PROP_SIG3D] = red[(int64_t)h * HALMA_RED_NFIELDS + HALMA_RED_SIGMA];
        for (int a = 0; a < 3; ++a) {
            const double r = red[((int64_t)(a + 1) * G + h) * HALMA_RED_NFIELDS + HALMA_RED_R05];
            o[HALMA_PROP_R05X + a] = r;
            res[((int64_t)h * 3 + a) * 3] = (float)r;
        }
    }
}

__global__ void pr_proj_out_kernel(int G, const float *__restrict__ res, double *__restrict__ out) {
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < G; h += gridDim.x * blockDim.x) {
        double *o = out + (int64_t)h * HALMA_PROP_NFIELDS;
        const float *r = res + (int64_t)h * 9;   // [projection][sig05, vsigma, lambda]
        o[HALMA_PROP_SIG1DX] = r[0];
        o[HALMA_PROP_SIG1DY] = r[3];
        o[HALMA_PROP_SIG1DZ] = r[6];
        // (V_sigma_x + V_sigma_y + V_sigma_z) / 3. and the same for lambda (f90:456-457)
        o[HALMA_PROP_VSIGMA] = __fdiv_rn(__fadd_rn(__fadd_rn(r[1], r[4]), r[7]), 3.f);
        o[HALMA_PROP_LAMBDA] = __fdiv_rn(__fadd_rn(__fadd_rn(r[2], r[5]), r[8]), 3.f);
    }
}

int nbits(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) ++b;
    return b < 1 ? 1 : b;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_halo_properties(int64_t n, const double *x, const double *y, const double *z, const double *vx,
                                     const double *vy, const double *vz, const double *m, int64_t n_groups,
                                     const int64_t *group_offsets, const int32_t *group_members,
                                     const double *centre, double linking_length, double *out,
                                     halma_stream_t stream) {
    if (n < 0 || n_groups < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= INT32_MAX || n_groups >= INT32_MAX / 3) return fail(HALMA_ERR_CAPACITY, "too many particles or groups");
    if (!(linking_length > 0.0) || !isfinite(linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and > 0");
    if (!group_offsets || !centre || !out || (n_groups > 0 && !group_members) ||
        (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    if (n_groups == 0) return HALMA_OK;
    const int G = (int)n_groups;
    std::vector<int64_t> h_off(G + 1);
    HALMA_CUDA(cudaMemcpy(h_off.data(), group_offsets, 8ull * (G + 1), cudaMemcpyDefault));
    if (h_off[0] != 0) return fail(HALMA_ERR_INVALID, "group offsets must start at 0");
    for (int h = 0; h < G; ++h)
        if (h_off[h + 1] < h_off[h]) return fail(HALMA_ERR_INVALID, "group offsets must not decrease");
    const int64_t N0 = h_off[G];
    if (3 * N0 >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most (2^31-2)/3 members");
    std::vector<double> hc(5ull * G);
    HALMA_CUDA(cudaMemcpy(hc.data(), centre, 40ull * G, cudaMemcpyDefault));
    double rmax = 0.0;
    for (int h = 0; h < G; ++h) {
        for (int q = 0; q < 5; ++q)
            if (!isfinite(hc[5ull * h + q])) return fail(HALMA_ERR_INVALID, "non-finite centre row %d", h);
        if (!(hc[5ull * h + 4] >= 0.0)) return fail(HALMA_ERR_INVALID, "rmax of group %d is negative", h);
        rmax = std::max(rmax, hc[5ull * h + 4]);
    }
    // cells of the largest projected grid
    const double ncell_max = ceil(2.0 * (rmax + linking_length) / (2.0 * linking_length)) + 2.0;
    if (ncell_max * ncell_max > 1e15) return fail(HALMA_ERR_CAPACITY, "projection grid too large");
    const int cbits = nbits((uint64_t)(ncell_max * ncell_max));
    if (cbits + nbits((uint64_t)3 * G) > 63) return fail(HALMA_ERR_CAPACITY, "projection grid too large");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dvx = nullptr, *dvy = nullptr, *dvz = nullptr,
                 *dm = nullptr, *dcen = nullptr;
    const int64_t *doff = nullptr;
    const int32_t *dmem = nullptr;
    double *dout = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(vx, n, true, false, &dvx);
    sg.add(vy, n, true, false, &dvy);
    sg.add(vz, n, true, false, &dvz);
    sg.add(m, n, true, false, &dm);
    sg.add(group_offsets, n_groups + 1, true, false, &doff);
    sg.add(group_members, N0, true, false, &dmem);
    sg.add(centre, 5 * n_groups, true, false, &dcen);
    sg.add((const double *)out, n_groups * HALMA_PROP_NFIELDS, false, true, &dout);
    const int64_t NM = std::max<int64_t>(N0, 1), N3 = 3 * NM;
    Layout L;
    sg.plan(L);
    const size_t o_g = L.add(64ull * NM), o_ab = L.add(8ull * 4 * G * HALMA_ABOUT_NFIELDS);
    const size_t o_red = L.add(8ull * 4 * G * HALMA_RED_NFIELDS), o_own = L.add(4ull * NM);
    const size_t o_kin = L.add(8ull * N3), o_kout = L.add(8ull * N3), o_vin = L.add(4ull * (N3 + 1)),
                 o_vout = L.add(4ull * N3);
    const size_t o_head = L.add(4ull * N3), o_rpos = L.add(4ull * N3), o_rid = L.add(4ull * N3);
    const size_t o_cv = L.add(16ull * N3), o_ck = L.add(8ull * N3), o_res = L.add(4ull * 9 * G), o_cnt = L.add(64);
    const int S = G >= 8192 ? 1 : 16;   // blocks per group for the angular-momentum kernels
    const size_t o_kp = L.add(32ull * S * G), o_kctr = L.add(4ull * G), o_jv = L.add(64ull * G);
    const size_t sort_b = sort_pairs_u64_i32_bytes((int)N3, 64), scan_b = exclusive_sum_i32_bytes((int)N3);
    const size_t o_tmp = L.add(std::max(sort_b, scan_b));
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 7));
    HALMA_TRY(sg.bind_and_upload(base, st));
    double *gbuf = at<double>(base, o_g), *about = at<double>(base, o_ab), *red = at<double>(base, o_red);
    int *own = at<int>(base, o_own);
    auto *kin = at<uint64_t>(base, o_kin), *kout = at<uint64_t>(base, o_kout);
    int *vin = at<int>(base, o_vin), *vout = at<int>(base, o_vout), *head = at<int>(base, o_head);
    int *rpos = at<int>(base, o_rpos), *rid = at<int>(base, o_rid);
    auto *cellv = at<float4>(base, o_cv);
    auto *cellkey = at<uint64_t>(base, o_ck);
    float *res = at<float>(base, o_res);
    int *cnt = at<int>(base, o_cnt);
    double *kpart = at<double>(base, o_kp), *jvec = at<double>(base, o_jv);
    int *kctr = at<int>(base, o_kctr);
    void *tmp = at<void>(base, o_tmp);
    const int sms = device_sm_count();
    const int gN = std::min(sms * 8, grid_for(NM, 256)), gG = std::min(G, sms * 16), gH = grid_for(G, 128);
    // members in range (validated before any gather)
    {
        std::vector<int32_t> hm;
        const int32_t *mp = group_members;
        if (is_device_pointer(group_members)) {
            hm.resize(N0);
            HALMA_CUDA(cudaMemcpy(hm.data(), group_members, 4ull * N0, cudaMemcpyDeviceToHost));
            mp = hm.data();
        }
        for (int64_t k = 0; k < N0; ++k)
            if (mp[k] < 0 || mp[k] >= n) return fail(HALMA_ERR_INVALID, "group member outside [0, n)");
    }
    HALMA_CUDA(cudaMemsetAsync(dout, 0, 8ull * G * HALMA_PROP_NFIELDS, st));
    HALMA_LAUNCH(pr_gather_kernel, gN, 256, 0, st, N0, dmem, dx, dy, dz, dvx, dvy, dvz, dm, gbuf);
    HALMA_LAUNCH(pr_fill_kernel, gG, 256, 0, st, G, doff, own);
    HALMA_LAUNCH(pr_bulk_kernel, gG, 256, 0, st, G, doff, gbuf, NM, dcen, dout, about);
    // half-mass radii (3-D with sigma_effective, then x, y, z projections) by the reductions
    const double *gx = gbuf, *gy = gbuf + NM, *gz = gbuf + 2 * NM, *gvx = gbuf + 3 * NM, *gvy = gbuf + 4 * NM,
                 *gvz = gbuf + 5 * NM, *gm = gbuf + 6 * NM, *g0 = gbuf + 7 * NM;
    const double *pos[4][3] = {{gx, gy, gz}, {gy, gz, g0}, {gx, gz, g0}, {gx, gy, g0}};
    for (int r = 0; r < 4; ++r)
        HALMA_TRY(reductions_device(N0, G, doff, pos[r][0], pos[r][1], pos[r][2], gvx, gvy, gvz, gm, nullptr,
                                    about + (int64_t)r * G * HALMA_ABOUT_NFIELDS,
                                    red + (int64_t)r * G * HALMA_RED_NFIELDS, st));
    HALMA_LAUNCH(pr_r05_kernel, gH, 128, 0, st, G, red, dout, res);
    HALMA_CUDA(cudaMemsetAsync(kctr, 0, 4ull * G, st));
    HALMA_LAUNCH(pr_kin1_kernel, G * S, 256, 0, st, G, S, doff, gbuf, NM, dcen, dout, kpart, kctr, jvec);
    HALMA_LAUNCH(pr_kin2_kernel, G * S, 256, 0, st, G, S, doff, gbuf, NM, dcen, dout, kpart, kctr, jvec);
    HALMA_LAUNCH(pr_shape_kernel, gG, 256, 0, st, G, doff, gbuf, NM, dcen, dout);
    if (N0 > 0) {
        HALMA_LAUNCH(pr_pkeys_kernel, gN, 256, 0, st, N0, G, doff, own, gbuf, dcen, linking_length, cbits, kin, vin);
        const int n3 = (int)(3 * N0);
        const int g3 = std::min(sms * 8, grid_for(n3, 256));
        // keys hold (3 group + projection) above cbits of cell index: sort only those bits
        HALMA_TRY(sort_pairs_u64_i32(tmp, sort_b, kin, kout, vin, vout, n3, cbits + nbits((uint64_t)3 * G), st));
        HALMA_LAUNCH(pr_head_kernel, g3, 256, 0, st, n3, kout, head);
        HALMA_TRY(exclusive_sum_i32(tmp, scan_b, head, rpos, n3, st));
        int last[2];
        HALMA_CUDA(cudaMemcpyAsync(&last[0], rpos + n3 - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaMemcpyAsync(&last[1], head + n3 - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        const int ncell = last[0] + last[1];
        int *runstart = vin;   // the sort's input values are no longer needed
        HALMA_LAUNCH(pr_runstart_kernel, g3, 256, 0, st, n3, head, rpos, runstart);
        HALMA_LAUNCH(pr_cells_kernel, sms * 16, 256, 0, st, ncell, N0, runstart, kout, vout, own, gbuf, dout, cellv,
                     cellkey, rid);
        HALMA_LAUNCH(pr_proj_kernel, gG, 256, 0, st, G, N0, doff, gbuf, dcen, linking_length, cbits, rid, cellv,
                     cellkey, ncell, res);
        HALMA_LAUNCH(pr_proj_out_kernel, gH, 128, 0, st, G, res, dout);
    }
    (void)cnt;
    HALMA_TRY(sg.download(st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    return HALMA_OK;
}
