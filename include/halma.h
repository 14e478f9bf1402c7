/*
 * halma.h — C ABI of the GB300 (sm_103a) halo-finding hot path.
 *
 * Every entry point returns an int status (HALMA_OK = 0, negative on error) and never
 * throws.  Array arguments are plain pointers that may live in host memory (pageable or
 * pinned) or in device memory of the current CUDA device; the library detects which.
 *   - device pointers: work is queued on `stream` (a cudaStream_t, NULL = legacy default
 *     stream) and the call returns without synchronising unless a count must be returned;
 *   - host pointers: inputs are copied in and outputs copied back on `stream`, and the call
 *     synchronises the stream before returning.
 * The caller owns every buffer it passes.  The library keeps one cached device workspace
 * per device (grown on demand, released by halma_release_workspace) and serialises calls
 * that use it with a mutex.  A human-readable reason for the last failure on the calling
 * thread is returned by halma_last_error().
 *
 * Reference interfaces replaced (pyHALMA, paths inside its repository):
 *   halma_fof / halma_fof_groups  <- python_scripts/fof.py:18-79 friends_of_friends
 *                                    (+ fof.py:87-89 serial wrapper, pyHALMA.py:148-149
 *                                    good_groups for the min-member filter)
 *   halma_bf_potential_f32        <- fortran_modules/particle_subroutines.f90:466-514
 *                                    brute_force_binding_energy, bound by f2py as
 *                                    particle.particle.brute_force_binding_energy(ncores,
 *                                    ntotal, total_mass, total_x, total_y, total_z, ntest,
 *                                    test_x, test_y, test_z) (halo_gas.py:182-186)
 *   halma_potential_f64           <- same loop in FP64 (the plain per-halo GPU comparator)
 *   halma_halo_reductions         <- python_scripts/halo_properties.py:16-60 total_mass,
 *                                    center_of_mass, CM_velocity; :98-111
 *                                    furthest_particle; :365-392 half_mass_radius;
 *                                    :607-625 sigma_effective
 *   halma_unbind_batched          <- halo_properties.py:282-361
 *                                    escape_velocity_unbinding_fortran (single pass),
 *                                    iterated until no particle is removed
 *   halma_potential_grad_f32      <- no reference counterpart (adjoint of the potential)
 *   halma_fof_segmented           <- the per-halo fof.friends_of_friends_serial calls of the
 *                                    substructure loop (pyHALMA.py:716-726), batched
 *   halma_split_bridges           <- the substructure block pyHALMA.py:703-766
 *   halma_amr_to_particles        <- halo_gas.py:9-52 patch_to_particles and :56-141
 *                                    AMRgrid_to_particles (the loop over the box's patches)
 *   halma_ball_gather             <- halo_gas.py:223-277 st_gas_dm_particles_inside range
 *                                    queries (KDTree.query_ball_point, parallel_inside)
 *   halma_phase_space_clean       <- halo_properties.py:113-278 calc_cell / clean_cell and
 *                                    the main script's loop pyHALMA.py:774-843
 *   halma_halo_properties         <- halo_properties.py:45-96, 365-515, 607-625, 781-866 and
 *                                    particle_subroutines.f90:12-461 as called at
 *                                    pyHALMA.py:930-1016
 *   halma_sequential_sum_f64      <- the scalar FP64 accumulation loops of the numba kernels
 *                                    (e.g. halo_properties.py:120-157), exposed on its own
 */
#ifndef HALMA_H
#define HALMA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HALMA_ABI_VERSION 1

#define HALMA_OK                 0
#define HALMA_ERR_INVALID       -1   /* bad argument (size, NaN input, null pointer)   */
#define HALMA_ERR_NOMEM         -2   /* device or pinned allocation failed              */
#define HALMA_ERR_CUDA          -3   /* a CUDA runtime call failed                      */
#define HALMA_ERR_NOT_CONVERGED -4   /* iteration cap reached (union-find, unbinding)   */
#define HALMA_ERR_TIMEOUT       -5   /* a bounded device-side wait ran out              */
#define HALMA_ERR_CAPACITY      -6   /* input exceeds a documented capacity             */
#define HALMA_ERR_NO_DEVICE     -7   /* no CUDA device visible                          */

typedef void *halma_stream_t;        /* cudaStream_t */

int         halma_abi_version(void);
const char *halma_status_string(int status);
const char *halma_last_error(void);
int         halma_release_workspace(void);
/* Number of kernels this library launched since load (all entry points, all devices). */
int64_t     halma_kernel_launch_count(void);
/* Measurement hooks (no reference counterpart).  With profiling on, the unbinding records
 * CUDA events around every pair-kernel launch on the launching stream and the pair count of
 * every pass, and halma_find_haloes times its FoF and unbinding stages.  halma_profile_stats
 * fills out[] with [fof_ms, unbind_ms, n_passes, pairs_0, ms_0, sym_pairs_0, sym_ms_0,
 * pairs_1, ...] for the last call (per pass: pair terms, milliseconds of the pass's pair
 * kernels, the pair terms of the haloes that ran on the symmetric block kernel, where each
 * pair is evaluated once for both particles, and the milliseconds of that kernel alone) and
 * returns the number of values available. */
int         halma_set_profiling(int32_t on);
int         halma_profile_stats(double *out, int32_t cap);
/* With profiling on: milliseconds of the FoF stages of the last halma_find_haloes call
 * (bounding box + keys, key sort, sorted records + sub-cell runs, cell table + hash +
 * one-component cells, work items, linking, roots + labels, groups); returns the count (8). */
int         halma_profile_fof_stages(double *out, int32_t cap);
/* Measurement hook (no reference counterpart): the FP32 FMA rate of the current device, from
 * a kernel of independent FMA chains (packed != 0: fma.rn.f32x2, else fma.rn.f32), iters
 * chain steps per thread, fastest of three timed launches after one warm-up; an FMA counts
 * as two flops.  The roofline denominator of the CUDA-core pair kernels. */
int         halma_measure_fp32_fma_rate(int32_t packed, int32_t iters, double *tflops, double *ms,
                                        halma_stream_t stream);
/* Measurement hook (no reference counterpart): the rate of the pair kernels' arithmetic alone
 * on the current device -- per pair of particles 3 sub + 3 fma + 2 fma as f32x2 instructions
 * and one rsqrt, sources from shared memory, 8 targets per lane, at the occupancy its registers
 * allow -- in pairs per second (each pair gives one term to each particle), fastest of three
 * timed launches after one warm-up.  This mix loads the FP32 pipe and the special-function
 * unit both to their throughput, so its rate, not either peak alone, is the ceiling of the
 * symmetric block kernel. */
int         halma_measure_pair_rate(int32_t iters, double *pairs_per_s, double *ms, halma_stream_t stream);
/* Measurement hook (no reference counterpart): the same for the tile kernel of the incremental
 * passes, whose pair terms are evaluated for one particle each: per term 3 sub + 3 fma + 1 fma
 * as f32x2 instructions and one rsqrt, 4 targets per lane, in pair terms per second. */
int         halma_measure_term_rate(int32_t iters, double *terms_per_s, double *ms, halma_stream_t stream);
/* Debug knob (no reference counterpart): the iteration bound of every union-find loop of the
 * FoF kernels (find walks, CAS retries).  A loop that reaches it stops, and the FoF call
 * returns HALMA_ERR_NOT_CONVERGED with the device still usable.  cap < 0 restores the default
 * (2^26, never reached on real inputs); cap = 0 stops at the first step of any walk.  Applies
 * to all later FoF calls in the process (halma_fof, halma_fof_segmented, halma_find_haloes,
 * halma_split_bridges). */
int         halma_set_union_find_cap(int32_t cap);

/* ------------------------------------------------------------------------------------ */
/* Friends-of-friends                                                                   */
/* ------------------------------------------------------------------------------------ */
/* labels[i] = smallest index of i's FoF component, or -1 if i has no friend.  Pair rule:
 * ((dx*dx + dy*dy) + dz*dz) <= ll*ll in IEEE double (inclusive, non-periodic), exactly the
 * predicate of scipy's KDTree.query_ball_point used by fof.py:40,61.
 * n_groups (optional) receives the number of components with >= 2 members. */
int halma_fof(int64_t n, const double *x, const double *y, const double *z,
              double linking_length, int32_t *labels, int64_t *n_groups,
              halma_stream_t stream);

/* The same in a periodic box (an opt-in option: fof.py:20 itself builds its KDTree without a
 * box size; this is what the same flood fill gives with KDTree(data, boxsize=box)).  Positions must lie in
 * [0, box)^3 (HALMA_ERR_INVALID otherwise) and box must be at least 3 linking lengths.  Two
 * particles are friends when the distance between one and the nearest periodic image of the
 * other passes the same predicate, the image coordinate being x +- box rounded in IEEE
 * double; labels are the smallest index of each component as above. */
int halma_fof_periodic(int64_t n, const double *x, const double *y, const double *z,
                       double linking_length, double box, int32_t *labels, int64_t *n_groups,
                       halma_stream_t stream);

/* Groups in the reference's output order (fof.py:76-77): groups ordered by smallest member,
 * members ascending, only groups with >= min_members members (pyHALMA.py:148-149).
 * members must hold n entries and offsets n+1 entries.  On return *n_groups groups are
 * stored: members[offsets[g] .. offsets[g+1]).  A label outside [-1, n) (checked on the
 * device, so also for device labels) fails the call with HALMA_ERR_INVALID. */
int halma_fof_groups(int64_t n, const int32_t *labels, int32_t min_members,
                     int64_t *offsets, int32_t *members, int64_t *n_groups,
                     halma_stream_t stream);

/* FoF inside segments, all segments in one call: rows seg_offsets[s] .. seg_offsets[s+1]
 * form segment s (offsets from 0 to n, non-decreasing) and two rows link only when they
 * are in the same segment.  Replaces the per-halo calls
 * fof.friends_of_friends_serial(st_x[part_list], st_y[part_list], st_z[part_list], sub_LL)
 * of the substructure loop (pyHALMA.py:716-726): with the members of each halo gathered
 * into consecutive rows, halma_fof_groups on these labels gives every halo's sub-groups in
 * the reference order, halo after halo.  Same pair rule and labels as halma_fof (smallest
 * row index of the component, -1 for rows without a friend in their segment). */
int halma_fof_segmented(int64_t n, const double *x, const double *y, const double *z,
                        int64_t n_segments, const int64_t *seg_offsets, double linking_length,
                        int32_t *labels, int64_t *n_groups, halma_stream_t stream);

/* Bridge splitting of the substructure block (pyHALMA.py:703-766), parameters as read from
 * pyHALMA.dat (pyHALMA.py:96-98; lengths in the unit of the positions). */
typedef struct {
    double  linking_length;  /* LL of the FoF that made the groups                       */
    double  dec_factor;      /* DEC_FACTOR (> 1): sub_LL = LL/DEC, LL/DEC^2, ...         */
    double  min_ll;          /* MIN_LL: levels run while sub_LL > MIN_LL                 */
    double  dist_factor;     /* DIST_FACTOR: a sub-group is cut off when its centre of
                                mass is farther than DIST_FACTOR * r_half from the halo's */
    int32_t minp_sub;        /* MINP_SUB: smallest sub-group considered                  */
    int32_t minp;            /* MINP: smallest group kept at the end                      */
} halma_substructure_params;

/* Input: the FoF groups (after good_groups(MINP)) as CSR over snapshot indices, members
 * ascending, in the reference order.  Output: the groups that pyHALMA.py:703-766 leaves,
 * in its order: the input groups (reduced by the sub-groups cut off; emptied when less than
 * 30 % of their particles remain) followed by the sub-groups cut off (halo by halo, level
 * by level, each level by smallest member), every group with fewer than MINP members
 * dropped.  *n_out receives the number of groups (HALMA_ERR_CAPACITY, with *n_out set,
 * when it exceeds out_capacity); out_offsets holds n_out+1 entries, out_members at most
 * the input's member count.  *n_cut (optional) receives the reference's counter_sub. */
int halma_split_bridges(int64_t n, const double *x, const double *y, const double *z,
                        const double *m, int64_t n_groups, const int64_t *group_offsets,
                        const int32_t *group_members, const halma_substructure_params *params,
                        int64_t *n_out, int64_t out_capacity, int64_t *out_offsets,
                        int32_t *out_members, int64_t *n_cut, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* Phase-space cleaning                                                                 */
/* ------------------------------------------------------------------------------------ */
/* pyHALMA's phase-space cleaning for all groups at once: calc_cell / clean_cell
 * (python_scripts/halo_properties.py:113-278) inside pyHALMA.py's loop over groups
 * (pyHALMA.py:774-843), parameters as read from pyHALMA.dat (pyHALMA.py:71-73, 776). */
typedef struct {
    double  linking_length;  /* LL: grid cells are 2 LL wide                            */
    double  q_fil;           /* Q_FIL: a particle in a cell of <= q_fil particles drops  */
    double  sig_fil;         /* SIG_FIL: drop at |v - v_cell| >= fac_sig*SIG_FIL*sigma    */
    int32_t enabled;         /* PSC_FLAG: 0 keeps every particle (pyHALMA.py's reset)     */
    int32_t min_part;        /* min_part_PSC (50): smaller groups keep every particle     */
    int32_t minp;            /* MINP: groups with fewer kept particles are not kept       */
    int32_t max_passes;      /* bound on the sweeps per group (a safety limit)            */
} halma_psc_params;

enum {
    HALMA_PSC_CX = 0, HALMA_PSC_CY, HALMA_PSC_CZ,  /* centre of mass of the kept particles */
    HALMA_PSC_MASS,      /* their mass                                                   */
    HALMA_PSC_RMAX,      /* furthest kept particle from that centre                      */
    HALMA_PSC_NPART,     /* kept particles                                               */
    HALMA_PSC_NCELL,     /* grid points per axis of the first grid (pyHALMA.py's n_cell)  */
    HALMA_PSC_KEPT,      /* 1 when NPART >= MINP                                         */
    HALMA_PSC_PASSES,    /* sweeps made                                                  */
    HALMA_PSC_NFIELDS
};

/* Groups as CSR over particle indices (group_offsets[n_groups+1], group_members).  Outputs:
 * control[k] (1 = member k kept, pyHALMA.py's part_list[control]); which_cell (optional,
 * 3 x members: the x, y then z cell of every particle of clean_cell's final grid, group g's
 * first n_which[g] entries from group_offsets[g] on, n_which optional); halo_out
 * (n_groups x HALMA_PSC_NFIELDS).  Like the reference, a sweep after the first marks
 * control[ip] with ip the particle's position in the list it sweeps.  HALMA_ERR_NOT_CONVERGED
 * when a group needs more than max_passes sweeps. */
int halma_phase_space_clean(int64_t n, const double *x, const double *y, const double *z,
                            const double *vx, const double *vy, const double *vz, const double *m,
                            int64_t n_groups, const int64_t *group_offsets,
                            const int32_t *group_members, const halma_psc_params *params,
                            uint8_t *control, int32_t *which_cell, int64_t *n_which,
                            double *halo_out, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* O(N) per-halo properties                                                             */
/* ------------------------------------------------------------------------------------ */
enum {
    HALMA_PROP_R05 = 0,   /* half_mass_radius (halo_properties.py:365-392)                  */
    HALMA_PROP_R05X, HALMA_PROP_R05Y, HALMA_PROP_R05Z,   /* half_mass_radius_proj :397-458  */
    HALMA_PROP_VX, HALMA_PROP_VY, HALMA_PROP_VZ,         /* CM_velocity :45-60              */
    HALMA_PROP_JX, HALMA_PROP_JY, HALMA_PROP_JZ,         /* angular_momentum :461-481       */
    HALMA_PROP_J,         /* (jx^2 + jy^2 + jz^2)^0.5 (pyHALMA.py:961-963)                  */
    HALMA_PROP_VTF,       /* tully_fisher_velocity :62-96 (NaN: no particle in 0.9-1.1 R05) */
    HALMA_PROP_KCO,       /* kinematic_morphology :483-515                                  */
    HALMA_PROP_SA, HALMA_PROP_SB, HALMA_PROP_SC,         /* halo_shape_fortran -> f90:160-214 */
    HALMA_PROP_SIG3D,     /* sigma_effective :607-625                                       */
    HALMA_PROP_SIG1DX, HALMA_PROP_SIG1DY, HALMA_PROP_SIG1DZ,  /* sigma_projections_fortran   */
    HALMA_PROP_VSIGMA, HALMA_PROP_LAMBDA,                /* -> f90:217-461                  */
    HALMA_PROP_NFIELDS
};

/* The O(N) properties of pyHALMA's property loop (pyHALMA.py:930-1016) for all groups at
 * once.  Groups as CSR over particle indices; centre: n_groups x 5 rows (cx, cy, cz, mass,
 * rmax), the center_x / masses / rmax arrays the phase-space cleaning leaves; out: n_groups x
 * HALMA_PROP_NFIELDS.  As in the reference, JZ is sum m (rx*vvy - ry*vvz) / M.  The FP32
 * Fortran quantities (shape, projections) are summed in the Fortran's order, every operation
 * rounded on its own. */
int halma_halo_properties(int64_t n, const double *x, const double *y, const double *z,
                          const double *vx, const double *vy, const double *vz, const double *m,
                          int64_t n_groups, const int64_t *group_offsets,
                          const int32_t *group_members, const double *centre,
                          double linking_length, double *out, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* AMR gas cells to particles                                                           */
/* ------------------------------------------------------------------------------------ */
/* Replaces python_scripts/halo_gas.py:56-141 AMRgrid_to_particles (with the numba kernel
 * patch_to_particles, :9-52) for one box: every cell of the n_patches patches given (levels
 * >= 1, in the order to emit) whose centre x0 + i*res (x0 = r - res/2, res = (L/ncoarse)/2^level)
 * lies strictly inside box = [xmin, xmax, ymin, ymax, zmin, zmax] and whose cr0amr and
 * solapst flags are both non-zero becomes one gas particle: the centre, the velocity times
 * 3e5, mass ((1 + delta) * rho_B) * res^3 (comoving) and the temperature.  Patch tables are
 * host arrays: patch_level[p], patch_n[3p..3p+2] = nx, ny, nz, patch_r[3p..3p+2] = the
 * reference's patchrx/ry/rz, cell_offset[p] = first cell of patch p (cell_offset[n] = total).
 * Cell arrays (host or device) hold each patch's cells x-major: cell (ix, iy, iz) of patch p
 * at cell_offset[p] + (ix*ny + iy)*nz + iz.  Particles come out in patch order, x-major, as
 * the reference emits them; *n_out receives the count (HALMA_ERR_CAPACITY when it exceeds
 * capacity). */
int halma_amr_to_particles(int32_t n_patches, const int32_t *patch_level, const int32_t *patch_n,
                           const double *patch_r, const int64_t *cell_offset, const double *delta,
                           const double *vx, const double *vy, const double *vz, const double *temp,
                           const uint8_t *cr0amr, const uint8_t *solapst, double L, int32_t ncoarse,
                           const double *box, double rho_B, int64_t capacity, double *out_x,
                           double *out_y, double *out_z, double *out_vx, double *out_vy,
                           double *out_vz, double *out_mass, double *out_temp, int64_t *n_out,
                           halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* Ball gather                                                                          */
/* ------------------------------------------------------------------------------------ */
/* The particles inside each of n_balls spheres (centre cx/cy/cz[s], radius[s] >= 0), all
 * spheres in one call.  Replaces the per-halo range queries of
 * python_scripts/halo_gas.py:223-277 st_gas_dm_particles_inside:
 *   strict = 0: st_kdtree / dm_kdtree.query_ball_point([cx, cy, cz], R) (halo_gas.py:254,
 *               268), ((dx*dx + dy*dy) + dz*dz) <= R*R in IEEE double;
 *   strict = 1: parallel_inside(x, y, z, R, cx, cy, cz) (halo_gas.py:218-220, 237),
 *               sqrt((dx*dx + dy*dy) + dz*dz) < R.
 * Output as CSR: offsets[n_balls+1] (optional) and indices[offsets[s] .. offsets[s+1]) the
 * particle indices inside sphere s, ascending (KDTree.query_ball_point returns the same set
 * in tree order).  *n_found receives the total.  With indices == NULL only the counts are
 * computed; HALMA_ERR_CAPACITY (with *n_found set) when the total exceeds capacity. */
int halma_ball_gather(int64_t n, const double *x, const double *y, const double *z,
                      int64_t n_balls, const double *cx, const double *cy, const double *cz,
                      const double *radius, int32_t strict, int64_t *offsets, int32_t *indices,
                      int64_t capacity, int64_t *n_found, halma_stream_t stream);

/* Sequential FP64 sums: out[s] = values[offsets[s]] + values[offsets[s]+1] + ... added left to
 * right and rounded after every addition, as the reference's numba loops add (e.g. the
 * per-cell sums of calc_cell, halo_properties.py:120-157).  The GPU adds 32 values at a time
 * in integer ulps of the running sum's binade and falls back to one IEEE add where the sum
 * leaves its binade, changes sign or meets a tie, so the result equals the scalar loop bit
 * for bit for any finite or non-finite input.  offsets[n_segments+1] runs from 0 to n. */
int halma_sequential_sum_f64(int64_t n, const double *values, int64_t n_segments,
                             const int64_t *offsets, double *out, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* Brute-force potential                                                                */
/* ------------------------------------------------------------------------------------ */
#define HALMA_POT_REFERENCE 0   /* per target, float32 sequential sum in source order:
                                   bit-identical to particle_subroutines.f90:497-510
                                   (each operation rounded, no FMA); eps2 must be 0     */
#define HALMA_POT_FAST      1   /* float32 pair terms (rsqrt), compensated summation    */

/* phi_i = sum_j m_j / sqrt(r_ij^2 + eps2), skipping source j unless its x, y and z all
 * differ from target i's (f90:499-501).  Inputs are float32 as the f2py wrapper casts them
 * (halo_gas.py:172-178). */
int halma_bf_potential_f32(int64_t ntotal, const float *total_mass, const float *total_x,
                           const float *total_y, const float *total_z, int64_t ntest,
                           const float *test_x, const float *test_y, const float *test_z,
                           float *binding_energy, int32_t mode, double eps2,
                           halma_stream_t stream);

#define HALMA_MASK_COORD 0   /* the reference's coordinate-inequality mask              */
#define HALMA_MASK_SELF  1   /* skip source j == i + self_offset only                   */
#define HALMA_MASK_NONE  2

/* Allocation-free twin of halma_bf_potential_f32 in HALMA_POT_FAST mode (no counterpart in
 * the reference).  For callers that cannot let a library allocate device memory: host codes
 * (an AMR simulation calling the halo finder between steps) that reserve nearly all device
 * memory in their own pool, and callers that keep several streams busy, for whom the
 * device-wide synchronisation of a cudaFree is a stall.  It takes arrays in the current
 * device's memory only, calls no cudaMalloc/cudaFree, and keeps its scratch (the partial sums
 * of the source slices) in a 16 MiB static device array held by every GPU that loads the
 * library.  Same source split, same kernels and identical results as
 * halma_bf_potential_f32(HALMA_POT_FAST); returns HALMA_ERR_CAPACITY when the split needs more
 * than 2,097,152 partial sums (source slices x targets).  The first call on a device looks up
 * the array's address: make it before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race. */
int halma_bf_potential_f32_noalloc(int64_t ntotal, const float *total_mass, const float *total_x,
                                   const float *total_y, const float *total_z, int64_t ntest,
                                   const float *test_x, const float *test_y, const float *test_z,
                                   float *binding_energy, double eps2, halma_stream_t stream);

/* float32 pair terms (rsqrt) with compensated sums and a selectable mask: the smooth
 * (differentiable) forward of halma_potential_grad_f32 when mask is SELF or NONE.
 * When the targets are the first nt sources (tx == sx, ty == sy, tz == sz, device arrays,
 * nt >= 8192) and the mask is NONE with eps2 > 0 or SELF with self_offset 0, the pairs among
 * those nt particles are evaluated once for both particles (symmetric block kernel) and the
 * other sources per target; the result agrees with the per-target route within the same
 * 1e-6 relative bound, not bit for bit.
 * No reference counterpart beyond the potential above. */
int halma_potential_f32(int64_t ns, const float *m, const float *sx, const float *sy,
                        const float *sz, int64_t nt, const float *tx, const float *ty,
                        const float *tz, double eps2, int32_t mask, int64_t self_offset,
                        float *phi, halma_stream_t stream);

/* FP64 pairs and FP64 sum, one thread per target (the plain comparator path). */
int halma_potential_f64(int64_t ns, const double *m, const double *sx, const double *sy,
                        const double *sz, int64_t nt, const double *tx, const double *ty,
                        const double *tz, double eps2, int32_t mask, int64_t self_offset,
                        double *phi, halma_stream_t stream);

/* Adjoint of phi_i = sum_j m_j (r_ij^2 + eps2)^-1/2 (mask SELF or NONE) for an upstream
 * gradient g_i = dL/dphi_i.  Outputs (any may be NULL):
 *   grad_m[j]          = sum_i g_i (r^2+eps2)^-1/2
 *   grad_src[3j+k]     = m_j sum_i g_i (t_i - s_j)_k (r^2+eps2)^-3/2
 *   grad_tgt[3i+k]     = g_i sum_j m_j (s_j - t_i)_k (r^2+eps2)^-3/2
 * float32 pair terms with compensated sums. */
int halma_potential_grad_f32(int64_t ns, const float *m, const float *sx, const float *sy,
                             const float *sz, int64_t nt, const float *tx, const float *ty,
                             const float *tz, const float *g, double eps2, int32_t mask,
                             int64_t self_offset, float *grad_m, float *grad_src,
                             float *grad_tgt, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* Per-halo reductions (FP64)                                                           */
/* ------------------------------------------------------------------------------------ */
/* Haloes are CSR segments: halo h owns rows offsets[h] .. offsets[h+1] of the particle
 * arrays (halo-contiguous order); the offsets run from 0 to n without decreasing
 * (HALMA_ERR_INVALID otherwise, before any device work).  mask (optional, uint8) selects the particles that take
 * part.  out is n_haloes x HALMA_RED_NFIELDS doubles, row-major. */
enum {
    HALMA_RED_MASS = 0,  /* total_mass                                  */
    HALMA_RED_CX, HALMA_RED_CY, HALMA_RED_CZ,      /* center_of_mass    */
    HALMA_RED_VX, HALMA_RED_VY, HALMA_RED_VZ,      /* CM_velocity       */
    HALMA_RED_RMAX,      /* furthest_particle from the centre of mass  */
    HALMA_RED_R05,       /* half_mass_radius                           */
    HALMA_RED_SIGMA,     /* sigma_effective inside R05                 */
    HALMA_RED_N,         /* members taking part                        */
    HALMA_RED_NFIELDS
};
/* about (optional, n_haloes x HALMA_ABOUT_NFIELDS): per-halo values supplied by the caller
 * in place of the computed ones, as the reference functions take them as arguments
 * (furthest_particle and half_mass_radius take the centre and M, sigma_effective the
 * centre, bulk velocity and R05).  A NaN entry means "use the computed value". */
enum {
    HALMA_ABOUT_CX = 0, HALMA_ABOUT_CY, HALMA_ABOUT_CZ, HALMA_ABOUT_VX, HALMA_ABOUT_VY,
    HALMA_ABOUT_VZ, HALMA_ABOUT_MASS, HALMA_ABOUT_R05, HALMA_ABOUT_NFIELDS
};
int halma_halo_reductions(int64_t n, int64_t n_haloes, const int64_t *offsets,
                          const double *x, const double *y, const double *z,
                          const double *vx, const double *vy, const double *vz,
                          const double *m, const uint8_t *mask, const double *about,
                          double *out, halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* Batched iterative unbinding                                                          */
/* ------------------------------------------------------------------------------------ */
#define HALMA_UNBIND_FP32C 0   /* float32 pair terms, compensated sums, FP64 reductions */
#define HALMA_UNBIND_FP64  1   /* plain FP64 per-halo path: one launch per halo         */

typedef struct {
    double  eps;        /* softening length (position units), must be > 0               */
    double  G;          /* gravitational constant: velocity^2 * length / mass           */
    double  factor_v;   /* potential multiplied by factor_v^2 (halo_properties.py:353)  */
    int32_t max_iter;   /* passes at most (>= 1)                                        */
    int32_t precision;  /* HALMA_UNBIND_FP32C or HALMA_UNBIND_FP64                      */
    int32_t use_graph;  /* FP32C: replay all passes as one captured CUDA graph          */
    int32_t flags;      /* HALMA_UNBIND_FULL_RECOMPUTE or 0                             */
} halma_unbind_params;

/* FP32C passes after the first normally update the potential of the survivors by
 * subtracting the contribution of the particles the previous pass removed (the potential is
 * linear in the sources): O(bound x removed) pairs per pass instead of O(bound^2).  This flag
 * recomputes the full sum every pass instead. */
#define HALMA_UNBIND_FULL_RECOMPUTE 1

enum {
    HALMA_UB_MASS = 0, HALMA_UB_CX, HALMA_UB_CY, HALMA_UB_CZ, HALMA_UB_VX, HALMA_UB_VY,
    HALMA_UB_VZ, HALMA_UB_NBOUND, HALMA_UB_ITER, HALMA_UB_EKIN, HALMA_UB_EPOT,
    HALMA_UB_NFIELDS
};

/* Tile shapes of the FP32C pair kernel per halo size class (no reference counterpart):
 * a halo with nb bound particles uses T = t_per_class[c] targets per lane (1, 2 or 4) for
 * the first class c with nb <= upper[c] (increasing bounds, at most 8 classes), and every
 * work item covers slice_len source slots (a multiple of 32): big haloes are split into
 * (target tile x source slice) items whose partial sums are added in slice order.  Written
 * by the autotuner (pyhalma_gb300.autotune); the default is {32:1, 64:2, inf:4}, 4096. */
int halma_set_tile_table(int32_t n_classes, const int32_t *upper, const int32_t *t_per_class,
                         int32_t slice_len);
int halma_get_tile_table(int32_t *n_classes, int32_t *upper, int32_t *t_per_class,
                         int32_t *slice_len);

/* Particles in halo-contiguous order (CSR offsets, n_haloes+1 entries).  Every pass
 * recomputes each halo's FP64 bound mass, centre and bulk velocity, the potential of the
 * bound particles due to the bound particles (self pair excluded), and removes particles
 * with 1/2|v - v_bulk|^2 - G * factor_v^2 * phi > 0.  Outputs: bound[n] (1 = bound),
 * phi[n] (optional, last pass, FP64; 0 for removed particles), halo_out (n_haloes x
 * HALMA_UB_NFIELDS, row-major; EKIN = sum 1/2 m |v - v_bulk|^2 and EPOT = -1/2 G
 * factor_v^2 sum m phi over the bound particles of the last pass). */
int halma_unbind_batched(int64_t n, int64_t n_haloes, const int64_t *offsets,
                         const double *x, const double *y, const double *z,
                         const double *vx, const double *vy, const double *vz,
                         const double *m, const halma_unbind_params *params,
                         uint8_t *bound, double *phi, double *halo_out,
                         halma_stream_t stream);

/* ------------------------------------------------------------------------------------ */
/* One snapshot end to end                                                              */
/* ------------------------------------------------------------------------------------ */
/* pyHALMA.py's star-particle path (pyHALMA.py:543-592 FoF + good_groups, then the per-halo
 * unbinding above) in one call: halma_fof -> groups with >= min_members members in the
 * reference order -> halma_unbind_batched over those groups.  Outputs (each optional except
 * n_haloes): labels[n] (FoF labels), bound[n] (1 = member of a kept group that survived the
 * unbinding), halo_offsets[cap+1] / members[n] (the groups as CSR over particle indices) and
 * halo_out[cap x HALMA_UB_NFIELDS].  Returns HALMA_ERR_CAPACITY (with *n_haloes set) when
 * more than halo_capacity groups were found and halo_offsets or halo_out was requested. */
int halma_find_haloes(int64_t n, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, const double *m,
                      double linking_length, int32_t min_members,
                      const halma_unbind_params *params, int32_t *labels, uint8_t *bound,
                      int64_t *n_haloes, int64_t halo_capacity, int64_t *halo_offsets,
                      int32_t *members, double *halo_out, halma_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* HALMA_H */
