/* ORACLE — test infrastructure, not product code.
 *
 * C restatement of two routines of pyHALMA's fortran_modules/particle_subroutines.f90
 * (gfortran is absent here, so the Fortran cannot be compiled), statement by statement, in
 * the Fortran's precision, run as the main script runs them with one OpenMP thread:
 *
 *   halo_shape            f90:160-214  FP32 inertia tensor sum_p m r_i r_j / sum m (particle
 *                                      order), DIAGONALISE (f90:12-126, Jacobi rotations in
 *                                      REAL*8 on the REAL*4 tensor), SORT_EIGEN (f90:129-157,
 *                                      decreasing), then FP32 sqrt of each eigenvalue;
 *   sigma_projections     f90:217-461  per projection a 2-D grid of cells (nearest grid point,
 *                                      minloc: first index on ties), FP32 per-cell mass,
 *                                      mass-weighted line-of-sight velocity and dispersion,
 *                                      the mean cell dispersion over particles inside the
 *                                      projected half-mass radius, and V/sigma and lambda
 *                                      summed over the cells with R_cell < R05 + 2 ll.
 *
 * Built with gcc -O2 -ffp-contract=off (no FMA contraction, each operation rounded).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static void diagonalise(const float in[3][3], float out[3]) {
    const int n = 3;
    double a[3][3], eig[3], b[3], z[3];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) a[i][j] = (double)in[i][j];
    for (int i = 0; i < n; ++i) {
        b[i] = a[i][i];
        eig[i] = b[i];
        z[i] = 0.0;
    }
    double sum_el = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) sum_el = sum_el + fabs(a[i][j]);
    for (int it = 1; it <= 100; ++it) {
        double suma = 0.0;
        for (int i = 0; i < n - 1; ++i)
            for (int j = i + 1; j < n; ++j) suma = suma + fabs(a[i][j]);
        if (suma < (double)1.e-4f * sum_el) break;
        const double upper = it < 4 ? 0.2 * (suma * suma) : 0.0;
        for (int ip = 0; ip < n - 1; ++ip) {
            for (int iq = ip + 1; iq < n; ++iq) {
                double var1 = 100.0 * fabs(a[ip][iq]);
                if (it > 4 && fabs(eig[ip]) + var1 == fabs(eig[ip]) && fabs(eig[iq]) + var1 == fabs(eig[iq])) {
                    a[ip][iq] = 0.0;
                } else if (fabs(a[ip][iq]) > upper) {
                    double var2 = eig[iq] - eig[ip];
                    double t;
                    if (fabs(var2) + var1 == fabs(var2)) {
                        t = a[ip][iq] / var2;
                    } else {
                        const double theta = 0.5 * var2 / a[ip][iq];
                        t = 1.0 / (fabs(theta) + sqrt(1.0 + theta * theta));
                        if (theta < 0.0) t = -t;
                    }
                    const double c = 1.0 / sqrt(1.0 + t * t);
                    const double s = t * c;
                    const double tau = s / (1.0 + c);
                    var2 = t * a[ip][iq];
                    z[ip] = z[ip] - var2;
                    z[iq] = z[iq] + var2;
                    eig[ip] = eig[ip] - var2;
                    eig[iq] = eig[iq] + var2;
                    a[ip][iq] = 0.0;
                    for (int j = 0; j < ip; ++j) {
                        const double g = a[j][ip], h = a[j][iq];
                        a[j][ip] = g - s * (h + g * tau);
                        a[j][iq] = h + s * (g - h * tau);
                    }
                    for (int j = ip + 1; j < iq; ++j) {
                        const double g = a[ip][j], h = a[j][iq];
                        a[ip][j] = g - s * (h + g * tau);
                        a[j][iq] = h + s * (g - h * tau);
                    }
                    for (int j = iq + 1; j < n; ++j) {
                        const double g = a[ip][j], h = a[iq][j];
                        a[ip][j] = g - s * (h + g * tau);
                        a[iq][j] = h + s * (g - h * tau);
                    }
                }
            }
        }
        for (int i = 0; i < n; ++i) {
            b[i] = b[i] + z[i];
            eig[i] = b[i];
            z[i] = 0.0;
        }
    }
    for (int i = 0; i < n; ++i) out[i] = (float)eig[i];
}

static void sort_eigen(float *e, int n) {
    for (int ii = 0; ii < n - 1; ++ii) {
        int kk = ii;
        float v = e[ii];
        for (int jj = ii + 1; jj < n; ++jj)
            if (e[jj] >= v) {
                kk = jj;
                v = e[jj];
            }
        if (kk != ii) {
            e[kk] = e[ii];
            e[ii] = v;
        }
    }
}

/* x, y, z: float32 positions relative to the centre; out[3] = a >= b >= c. */
void oracle_halo_shape(int npart, const float *x, const float *y, const float *z, const float *mass, float *out) {
    float it[3][3] = {{0}};
    float mtot = 0.f;
    for (int p = 0; p < npart; ++p) {
        const float r[3] = {x[p], y[p], z[p]};
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) it[i][j] = it[i][j] + mass[p] * r[i] * r[j];
        mtot = mtot + mass[p];
    }
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) it[i][j] = it[i][j] / mtot;
    diagonalise((const float(*)[3])it, out);
    sort_eigen(out, 3);
    for (int i = 0; i < 3; ++i) out[i] = sqrtf(out[i]);
}

static int minloc(const float *grid, int n, float v) {
    int best = 0;
    float bd = fabsf(grid[0] - v);
    for (int i = 1; i < n; ++i) {
        const float d = fabsf(grid[i] - v);
        if (d < bd) {
            bd = d;
            best = i;
        }
    }
    return best;
}

/* part_list: 0-based indices into the float32 particle arrays; velocities relative to the
 * bulk velocity.  out[5] = SIG_1D_x_05, SIG_1D_y_05, SIG_1D_z_05, V_sigma, lambda.
 * Returns 0, or -1 when the grid arrays cannot be allocated. */
int oracle_sigma_projections(int npart, const float *grid, int nc, const int64_t *part_list, const float *st_x,
                             const float *st_y, const float *st_z, const float *st_vx, const float *st_vy,
                             const float *st_vz, const float *st_mass, float cx, float cy, float cz, float r05x,
                             float r05y, float r05z, float ll, float *out) {
    const size_t nn = (size_t)nc * nc;
    int *qx = calloc(nn, sizeof(int)), *qy = calloc(nn, sizeof(int)), *qz = calloc(nn, sizeof(int));
    float *vcx = calloc(nn, 4), *vcy = calloc(nn, 4), *vcz = calloc(nn, 4);
    float *sdx = calloc(nn, 4), *sdy = calloc(nn, 4), *sdz = calloc(nn, 4);
    float *sgx = calloc(nn, 4), *sgy = calloc(nn, 4), *sgz = calloc(nn, 4);
    int rc = -1;
    if (!qx || !qy || !qz || !vcx || !vcy || !vcz || !sdx || !sdy || !sdz || !sgx || !sgy || !sgz) goto done;
#define AT(a, i, j) a[(size_t)(i) + (size_t)(j) * nc]   /* Fortran a(i, j) */
    for (int p = 0; p < npart; ++p) {
        const int64_t q = part_list[p];
        const int ix = minloc(grid, nc, st_x[q] - cx), iy = minloc(grid, nc, st_y[q] - cy),
                  iz = minloc(grid, nc, st_z[q] - cz);
        AT(vcx, iy, iz) = AT(vcx, iy, iz) + st_vx[q] * st_mass[q];
        AT(vcy, ix, iz) = AT(vcy, ix, iz) + st_vy[q] * st_mass[q];
        AT(vcz, ix, iy) = AT(vcz, ix, iy) + st_vz[q] * st_mass[q];
        AT(sdx, iy, iz) = AT(sdx, iy, iz) + st_mass[q];
        AT(sdy, ix, iz) = AT(sdy, ix, iz) + st_mass[q];
        AT(sdz, ix, iy) = AT(sdz, ix, iy) + st_mass[q];
        AT(qx, iy, iz) += 1;
        AT(qy, ix, iz) += 1;
        AT(qz, ix, iy) += 1;
    }
    for (size_t k = 0; k < nn; ++k) {
        if (sdx[k] != 0.f) vcx[k] = vcx[k] / sdx[k];
        if (sdy[k] != 0.f) vcy[k] = vcy[k] / sdy[k];
        if (sdz[k] != 0.f) vcz[k] = vcz[k] / sdz[k];
    }
    for (int p = 0; p < npart; ++p) {
        const int64_t q = part_list[p];
        const int ix = minloc(grid, nc, st_x[q] - cx), iy = minloc(grid, nc, st_y[q] - cy),
                  iz = minloc(grid, nc, st_z[q] - cz);
        float d;
        d = st_vx[q] - AT(vcx, iy, iz);
        AT(sgx, iy, iz) = AT(sgx, iy, iz) + d * d;
        d = st_vy[q] - AT(vcy, ix, iz);
        AT(sgy, ix, iz) = AT(sgy, ix, iz) + d * d;
        d = st_vz[q] - AT(vcz, ix, iy);
        AT(sgz, ix, iy) = AT(sgz, ix, iy) + d * d;
    }
    for (size_t k = 0; k < nn; ++k) {
        if (qx[k] != 0) sgx[k] = sqrtf(sgx[k] / (float)qx[k]);
        if (qy[k] != 0) sgy[k] = sqrtf(sgy[k] / (float)qy[k]);
        if (qz[k] != 0) sgz[k] = sqrtf(sgz[k] / (float)qz[k]);
    }
    {
        float s5x = 0.f, s5y = 0.f, s5z = 0.f;
        int cntx = 0, cnty = 0, cntz = 0;
        for (int p = 0; p < npart; ++p) {
            const int64_t q = part_list[p];
            const float dx = st_x[q] - cx, dy = st_y[q] - cy, dz = st_z[q] - cz;
            const int ix = minloc(grid, nc, dx), iy = minloc(grid, nc, dy), iz = minloc(grid, nc, dz);
            const float distx = sqrtf(dy * dy + dz * dz), disty = sqrtf(dx * dx + dz * dz),
                        distz = sqrtf(dx * dx + dy * dy);
            if (distx < r05x) {
                s5x = s5x + AT(sgx, iy, iz);
                cntx += 1;
            }
            if (disty < r05y) {
                s5y = s5y + AT(sgy, ix, iz);
                cnty += 1;
            }
            if (distz < r05z) {
                s5z = s5z + AT(sgz, ix, iy);
                cntz += 1;
            }
        }
        if (cntx > 0) s5x = s5x / (float)cntx;
        if (cnty > 0) s5y = s5y / (float)cnty;
        if (cntz > 0) s5z = s5z / (float)cntz;
        out[0] = s5x;
        out[1] = s5y;
        out[2] = s5z;
    }
    {
        /* planes: (outer, inner, vcm, sig, sd, R05) = XY: (iy, ix, _z, R05z), XZ: (iz, ix, _y,
         * R05y), YZ: (iz, iy, _x, R05x); the cell of (inner, outer) is a(inner, outer) */
        const float *vc[3] = {vcz, vcy, vcx}, *sg[3] = {sgz, sgy, sgx}, *sd[3] = {sdz, sdy, sdx};
        const float rr[3] = {r05z, r05y, r05x};
        float vs[3], lam[3];
        for (int pl = 0; pl < 3; ++pl) {
            float sumV = 0.f, sumS = 0.f, up = 0.f, down = 0.f;
            for (int o = 0; o < nc; ++o)
                for (int i = 0; i < nc; ++i) {
                    const float rbin = sqrtf(grid[i] * grid[i] + grid[o] * grid[o]);
                    if (rbin < rr[pl] + 2.f * ll) {
                        const float v = AT(vc[pl], i, o), s = AT(sg[pl], i, o), w = AT(sd[pl], i, o);
                        sumV = sumV + v * v * w;
                        sumS = sumS + s * s * w;
                        up = up + w * rbin * fabsf(v);
                        down = down + w * rbin * sqrtf(v * v + s * s);
                    }
                }
            vs[pl] = sumS > 0.f ? sqrtf(sumV / sumS) : 0.f;
            lam[pl] = down > 0.f ? up / down : 0.f;
        }
        /* (V_sigma_x + V_sigma_y + V_sigma_z) / 3: x is the YZ plane, z the XY plane */
        out[3] = (vs[2] + vs[1] + vs[0]) / 3.f;
        out[4] = (lam[2] + lam[1] + lam[0]) / 3.f;
    }
#undef AT
    rc = 0;
done:
    free(qx); free(qy); free(qz); free(vcx); free(vcy); free(vcz);
    free(sdx); free(sdy); free(sdz); free(sgx); free(sgy); free(sgz);
    return rc;
}
