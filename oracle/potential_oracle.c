/*
 * ORACLE (test infrastructure only): CPU restatement of pyHALMA's brute-force potential.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this code, as
 * the checker.  It is never part of the product path.
 *
 * oracle_bf_potential_f32 follows fortran_modules/particle_subroutines.f90:466-514
 * (brute_force_binding_energy) statement by statement:
 *   - float32 storage and float32 accumulation (f90:476-481);
 *   - for each test point, the source loop runs j = 1..ntotal in order, so the sum is a
 *     sequential float32 sum in source order (f90:497-510; the OpenMP reduction is over
 *     targets only);
 *   - a source is skipped unless x, y AND z all differ from the test point (f90:499-501);
 *   - r = sqrt((xj-xi)^2 + (yj-yi)^2 + (zj-zi)^2) in float32, summed left to right
 *     (f90:502-504), then phi += m_j / r (f90:505);
 *   - no softening.
 * Built with -ffp-contract=off and no fast-math so that each operation rounds on its own,
 * as the Fortran source reads.  Thread count = the reference's ncores argument (f90:490).
 *
 * oracle_potential_f64 is the FP64 twin: the same loop in double precision, with an
 * optional softening eps2 (phi += m / sqrt(r^2 + eps2)) and a choice of pair mask:
 *   mask 0: the reference's coordinate-inequality mask (f90:499-501);
 *   mask 1: skip only the pair whose source index equals the target index + self_offset
 *           (targets are a sub-range of the sources, as in per-halo unbinding);
 *   mask 2: no mask.
 *
 * oracle_potential_grad_f64 gives the FP64 reference gradient of L = sum_i g_i * phi_i with
 * phi_i = sum_j m_j (r_ij^2 + eps2)^-1/2 (mask 1 or 2):
 *   dL/dm_j   = sum_i g_i (r_ij^2 + eps2)^-1/2
 *   dL/dt_i   = g_i * sum_j m_j (s_j - t_i) (r_ij^2 + eps2)^-3/2       (target positions)
 *   dL/ds_j   = m_j * sum_i g_i (t_i - s_j) (r_ij^2 + eps2)^-3/2       (source positions)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

void oracle_bf_potential_f32(int32_t ncores, int32_t ntotal, const float *total_mass,
                             const float *total_x, const float *total_y, const float *total_z,
                             int32_t ntest, const float *test_x, const float *test_y,
                             const float *test_z, float *binding_energy)
{
#ifdef _OPENMP
    if (ncores > 0) omp_set_num_threads(ncores);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int32_t ip = 0; ip < ntest; ++ip) {
        const float tx = test_x[ip], ty = test_y[ip], tz = test_z[ip];
        float acc = 0.0f;
        for (int32_t j = 0; j < ntotal; ++j) {
            if (total_x[j] != tx && total_y[j] != ty && total_z[j] != tz) {
                const float dx = total_x[j] - tx;
                const float dy = total_y[j] - ty;
                const float dz = total_z[j] - tz;
                float s = dx * dx;
                s = s + dy * dy;
                s = s + dz * dz;
                const float r = sqrtf(s);
                acc = acc + total_mass[j] / r;
            }
        }
        binding_energy[ip] = acc;
    }
}

void oracle_potential_f64(int32_t ncores, int64_t ns, const double *m, const double *sx,
                          const double *sy, const double *sz, int64_t nt, const double *tx,
                          const double *ty, const double *tz, double eps2, int32_t mask,
                          int64_t self_offset, double *out)
{
#ifdef _OPENMP
    if (ncores > 0) omp_set_num_threads(ncores);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t i = 0; i < nt; ++i) {
        const double xi = tx[i], yi = ty[i], zi = tz[i];
        double acc = 0.0;
        for (int64_t j = 0; j < ns; ++j) {
            if (mask == 0) {
                if (!(sx[j] != xi && sy[j] != yi && sz[j] != zi)) continue;
            } else if (mask == 1) {
                if (j == i + self_offset) continue;
            }
            const double dx = sx[j] - xi, dy = sy[j] - yi, dz = sz[j] - zi;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            acc += m[j] / sqrt(r2);
        }
        out[i] = acc;
    }
}

void oracle_potential_grad_f64(int32_t ncores, int64_t ns, const double *m, const double *sx,
                               const double *sy, const double *sz, int64_t nt,
                               const double *tx, const double *ty, const double *tz,
                               const double *g, double eps2, int32_t mask, int64_t self_offset,
                               double *grad_m, double *grad_s /* ns*3 */,
                               double *grad_t /* nt*3 */)
{
#ifdef _OPENMP
    if (ncores > 0) omp_set_num_threads(ncores);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t i = 0; i < nt; ++i) {
        double ax = 0, ay = 0, az = 0;
        for (int64_t j = 0; j < ns; ++j) {
            if (mask == 1 && j == i + self_offset) continue;
            const double dx = sx[j] - tx[i], dy = sy[j] - ty[i], dz = sz[j] - tz[i];
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double ir = 1.0 / sqrt(r2);
            const double ir3 = ir * ir * ir;
            ax += m[j] * dx * ir3;
            ay += m[j] * dy * ir3;
            az += m[j] * dz * ir3;
        }
        grad_t[3 * i + 0] = g[i] * ax;
        grad_t[3 * i + 1] = g[i] * ay;
        grad_t[3 * i + 2] = g[i] * az;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int64_t j = 0; j < ns; ++j) {
        double gm = 0, bx = 0, by = 0, bz = 0;
        for (int64_t i = 0; i < nt; ++i) {
            if (mask == 1 && j == i + self_offset) continue;
            const double dx = tx[i] - sx[j], dy = ty[i] - sy[j], dz = tz[i] - sz[j];
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double ir = 1.0 / sqrt(r2);
            const double ir3 = ir * ir * ir;
            gm += g[i] * ir;
            bx += g[i] * dx * ir3;
            by += g[i] * dy * ir3;
            bz += g[i] * dz * ir3;
        }
        grad_m[j] = gm;
        grad_s[3 * j + 0] = m[j] * bx;
        grad_s[3 * j + 1] = m[j] * by;
        grad_s[3 * j + 2] = m[j] * bz;
    }
}
