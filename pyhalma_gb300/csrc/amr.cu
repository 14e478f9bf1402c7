// AMR gas cells to gas particles: python_scripts/halo_gas.py:9-52 (patch_to_particles) and
// :56-141 (AMRgrid_to_particles) for all selected patches of one box in one launch sequence.
//
// Every leaf cell (cr0amr and solapst both non-zero) of a refined patch whose centre lies
// strictly inside the box becomes one particle at the cell centre with the cell's velocity
// (times c = 3e5 km/s) and temperature and the comoving mass (1 + delta) * rho_B * res^3.
// Particles come out in the reference's order: patch by patch in the order given, and inside
// a patch x-major (ix outer, iz inner), the loop order of halo_gas.py:28-48.
//
// Arithmetic, with each operation rounded as written there (no contraction):
//   res  = (L / ncoarse) / 2^level              (halo_gas.py:107, on the host)
//   x0   = rx - res / 2                         (halo_gas.py:24)
//   x    = x0 + ix * res                        (halo_gas.py:29)
//   mass = ((1 + delta) * rho_B) * res^3        (halo_gas.py:45; res^3 from the host's pow)
//   vx   = vx_cell * 3e5                        (halo_gas.py:136)
// Cells are one thread each: a flag pass, an exclusive scan (CUB), a scatter pass.
#include <math.h>

#include "common.cuh"
#include "sort.cuh"

namespace halma {
namespace {

struct PatchGeom {
    double x0, y0, z0, res, res3;
    int nx, ny, nz, pad;
    int64_t first;   // first cell of the patch in the concatenated cell arrays
};

__device__ __forceinline__ int patch_of(const PatchGeom *__restrict__ pg, int np, int64_t c) {
    int lo = 0, hi = np - 1;
    while (lo < hi) {   // last patch whose first cell is <= c
        const int mid = (lo + hi + 1) >> 1;
        if (pg[mid].first <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool cell_centre(const PatchGeom &p, int64_t local, const double *box, double &x,
                                            double &y, double &z) {
    const int64_t nyz = (int64_t)p.ny * p.nz;
    const int ix = (int)(local / nyz);
    const int64_t r = local - (int64_t)ix * nyz;
    const int iy = (int)(r / p.nz), iz = (int)(r - (int64_t)iy * p.nz);
    x = __dadd_rn(p.x0, __dmul_rn((double)ix, p.res));
    y = __dadd_rn(p.y0, __dmul_rn((double)iy, p.res));
    z = __dadd_rn(p.z0, __dmul_rn((double)iz, p.res));
    return x > box[0] && x < box[1] && y > box[2] && y < box[3] && z > box[4] && z < box[5];
}

__global__ void amr_flag_kernel(int np, const PatchGeom *__restrict__ pg, int64_t ncell, const double *__restrict__ boxp,
                                const unsigned char *__restrict__ cr0amr, const unsigned char *__restrict__ solapst,
                                int *__restrict__ flag) {
    double box[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = boxp[k];
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
        const PatchGeom &p = pg[patch_of(pg, np, c)];
        double x, y, z;
        const bool in = cell_centre(p, c - p.first, box, x, y, z);
        flag[c] = (in && cr0amr[c] && solapst[c]) ? 1 : 0;
    }
}

__global__ void amr_emit_kernel(int np, const PatchGeom *__restrict__ pg, int64_t ncell, const double *__restrict__ boxp,
                                const int *__restrict__ flag, const int *__restrict__ pos,
                                const double *__restrict__ delta, const double *__restrict__ vx,
                                const double *__restrict__ vy, const double *__restrict__ vz,
                                const double *__restrict__ temp, double rho_B, double *__restrict__ ox,
                                double *__restrict__ oy, double *__restrict__ oz, double *__restrict__ ovx,
                                double *__restrict__ ovy, double *__restrict__ ovz, double *__restrict__ om,
                                double *__restrict__ ot) {
    double box[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) box[k] = boxp[k];
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
        if (!flag[c]) continue;
        const PatchGeom &p = pg[patch_of(pg, np, c)];
        double x, y, z;
        cell_centre(p, c - p.first, box, x, y, z);
        const int k = pos[c];
        ox[k] = x;
        oy[k] = y;
        oz[k] = z;
        ovx[k] = __dmul_rn(vx[c], 3e5);
        ovy[k] = __dmul_rn(vy[c], 3e5);
        ovz[k] = __dmul_rn(vz[c], 3e5);
        om[k] = __dmul_rn(__dmul_rn(__dadd_rn(1.0, delta[c]), rho_B), p.res3);
        ot[k] = temp[c];
    }
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_amr_to_particles(int32_t n_patches, const int32_t *patch_level, const int32_t *patch_n,
                                      const double *patch_r, const int64_t *cell_offset, const double *delta,
                                      const double *vx, const double *vy, const double *vz, const double *temp,
                                      const uint8_t *cr0amr, const uint8_t *solapst, double L, int32_t ncoarse,
                                      const double *box, double rho_B, int64_t capacity, double *out_x,
                                      double *out_y, double *out_z, double *out_vx, double *out_vy, double *out_vz,
                                      double *out_mass, double *out_temp, int64_t *n_out, halma_stream_t stream) {
    if (!n_out || !box || (n_patches > 0 && (!patch_level || !patch_n || !patch_r || !cell_offset)))
        return fail(HALMA_ERR_INVALID, "null pointer argument");
    if (n_patches < 0 || capacity < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (ncoarse <= 0 || !(L > 0.0) || !isfinite(L)) return fail(HALMA_ERR_INVALID, "L and ncoarse must be > 0");
    *n_out = 0;
    if (n_patches == 0) return HALMA_OK;
    // patch geometry on the host, in the reference's operations
    std::vector<PatchGeom> pg(n_patches);
    const int64_t ncell = cell_offset[n_patches];
    if (cell_offset[0] != 0 || ncell < 0) return fail(HALMA_ERR_INVALID, "cell_offset must start at 0");
    if (ncell >= (1ll << 31)) return fail(HALMA_ERR_CAPACITY, "at most 2^31-1 cells per call");
    const double cell0 = L / (double)ncoarse;
    for (int p = 0; p < n_patches; ++p) {
        const int l = patch_level[p];
        const int nx = patch_n[3 * p], ny = patch_n[3 * p + 1], nz = patch_n[3 * p + 2];
        if (l < 0 || l > 60) return fail(HALMA_ERR_INVALID, "patch %d: level %d out of range", p, l);
        if (nx < 0 || ny < 0 || nz < 0) return fail(HALMA_ERR_INVALID, "patch %d: negative extent", p);
        if (cell_offset[p + 1] - cell_offset[p] != (int64_t)nx * ny * nz)
            return fail(HALMA_ERR_INVALID, "patch %d: cell_offset does not match nx * ny * nz", p);
        PatchGeom &g = pg[p];
        g.res = cell0 / (double)(1ll << l);
        g.x0 = patch_r[3 * p] - g.res / 2;
        g.y0 = patch_r[3 * p + 1] - g.res / 2;
        g.z0 = patch_r[3 * p + 2] - g.res / 2;
        g.res3 = pow(g.res, 3.0);
        g.nx = nx;
        g.ny = ny;
        g.nz = nz;
        g.first = cell_offset[p];
    }
    if (ncell > 0 && (!delta || !vx || !vy || !vz || !temp || !cr0amr || !solapst))
        return fail(HALMA_ERR_INVALID, "null cell array");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *d_delta = nullptr, *d_vx = nullptr, *d_vy = nullptr, *d_vz = nullptr, *d_t = nullptr;
    const unsigned char *d_cr = nullptr, *d_so = nullptr;
    sg.add(delta, ncell, true, false, &d_delta);
    sg.add(vx, ncell, true, false, &d_vx);
    sg.add(vy, ncell, true, false, &d_vy);
    sg.add(vz, ncell, true, false, &d_vz);
    sg.add(temp, ncell, true, false, &d_t);
    sg.add(cr0amr, ncell, true, false, &d_cr);
    sg.add(solapst, ncell, true, false, &d_so);
    double *o[8] = {};
    double *user_out[8] = {out_x, out_y, out_z, out_vx, out_vy, out_vz, out_mass, out_temp};
    for (int k = 0; k < 8; ++k) sg.add((const double *)user_out[k], capacity, false, true, &o[k]);
    Layout Lw;
    sg.plan(Lw);
    const size_t o_pg = Lw.add(sizeof(PatchGeom) * n_patches), o_box = Lw.add(sizeof(double) * 6);
    const size_t o_flag = Lw.add(sizeof(int) * std::max<int64_t>(ncell, 1));
    const size_t o_pos = Lw.add(sizeof(int) * std::max<int64_t>(ncell, 1));
    const size_t scan_b = exclusive_sum_i32_bytes((int)std::max<int64_t>(ncell, 1));
    const size_t o_tmp = Lw.add(scan_b);
    void *base = nullptr;
    HALMA_TRY(workspace(Lw.total, &base, st));
    HALMA_TRY(sg.bind_and_upload(base, st));
    auto *dpg = at<PatchGeom>(base, o_pg);
    auto *dbox = at<double>(base, o_box);
    int *flag = at<int>(base, o_flag), *pos = at<int>(base, o_pos);
    HALMA_CUDA(cudaMemcpyAsync(dpg, pg.data(), sizeof(PatchGeom) * n_patches, cudaMemcpyHostToDevice, st));
    HALMA_CUDA(cudaMemcpyAsync(dbox, box, sizeof(double) * 6, cudaMemcpyHostToDevice, st));
    if (ncell == 0) return HALMA_OK;
    const int g = std::min(device_sm_count() * 8, grid_for(ncell, 256));
    HALMA_LAUNCH(amr_flag_kernel, g, 256, 0, st, n_patches, dpg, ncell, dbox, d_cr, d_so, flag);
    HALMA_TRY(exclusive_sum_i32(at<void>(base, o_tmp), scan_b, flag, pos, (int)ncell, st));
    int last[2];
    HALMA_CUDA(cudaMemcpyAsync(&last[0], pos + ncell - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaMemcpyAsync(&last[1], flag + ncell - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    const int64_t count = (int64_t)last[0] + last[1];
    *n_out = count;
    if (count > capacity)
        return fail(HALMA_ERR_CAPACITY, "%lld gas particles, capacity %lld", (long long)count, (long long)capacity);
    if (count == 0) return HALMA_OK;
    for (int k = 0; k < 8; ++k)
        if (!o[k]) return fail(HALMA_ERR_INVALID, "null output array");
    HALMA_LAUNCH(amr_emit_kernel, g, 256, 0, st, n_patches, dpg, ncell, dbox, flag, pos, d_delta, d_vx, d_vy, d_vz,
                 d_t, rho_B, o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7]);
    return sg.download(st);
}
