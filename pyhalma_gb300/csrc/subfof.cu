// Batched substructure identification: pyHALMA's bridge-splitting loop (pyHALMA.py:703-766)
// for every FoF group at once.
//
// The reference walks the groups one by one and, for sub_LL = LL/DEC, LL/DEC^2, ... while
// sub_LL > MIN_LL, (1) takes the centre of mass and half-mass radius of the group's current
// particle list (halo_properties.py:26-43, 365-392), (2) runs a KDTree FoF on that list at
// sub_LL (fof.py:87-89) and keeps sub-groups with >= MINP_SUB members (pyHALMA.py:148-149),
// (3) accepts a sub-group when 0.6 > its share of the list > 0.01 and its centre of mass lies
// farther than DIST_FACTOR * r_half from the group's, (4) removes the accepted sub-groups'
// particles from the list.  A group that lost more than 70 % of its particles is emptied;
// accepted sub-groups are appended after all groups; finally groups with fewer than MINP
// members are dropped.
//
// Here one level of that loop runs for all groups in a fixed number of launches: the current
// lists are gathered into group-contiguous FP64 arrays, the FP64 reductions run per group,
// the FoF runs once over all groups with links confined to each group (segmented cell
// list), the sub-groups' reductions run per sub-group, one thread per sub-group applies the
// two cuts, and the survivors are compacted in order.  The host only sees per-level counts
// and, at the end, the small table of accepted sub-groups, which it orders as the reference
// appends them.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

__global__ void gather4_kernel(int64_t nm, const int *__restrict__ idx, const double *__restrict__ x,
                               const double *__restrict__ y, const double *__restrict__ z,
                               const double *__restrict__ m, double *__restrict__ gx, double *__restrict__ gy,
                               double *__restrict__ gz, double *__restrict__ gm) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = idx[k];
        gx[k] = x[i];
        gy[k] = y[i];
        gz[k] = z[i];
        gm[k] = m[i];
    }
}

__device__ __forceinline__ int owner_of(const int64_t *__restrict__ off, int nseg, int64_t row) {
    int lo = 0, hi = nseg - 1;   // last segment whose start is <= row
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= row) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Input check before any gather: every member is a particle index, members ascend strictly
// inside each group.  bad |= 1 (out of range), |= 2 (order).
__global__ void check_members_kernel(int64_t nm, const int *__restrict__ mem, const int64_t *__restrict__ off, int nh,
                                     int64_t n, int *__restrict__ bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x) {
        const int v = mem[k];
        if (v < 0 || (int64_t)v >= n) atomicOr(bad, 1);
        if (k > 0 && owner_of(off, nh, k) == owner_of(off, nh, k - 1) && mem[k - 1] >= v) atomicOr(bad, 2);
    }
}

// One thread per sub-group: the share and distance cuts of pyHALMA.py:733-740.
//   part_fraction = len(group) / len(part_list);  0.6 > part_fraction > 0.01
//   dist_sub = sqrt((cx-cx_sub)**2 + (cy-cy_sub)**2 + (cz-cz_sub)**2) > DIST_FACTOR * r12
// (each operation rounded on its own, as NumPy evaluates the expression).
__global__ void cut_kernel(int ng, const int64_t *__restrict__ soff, const int *__restrict__ smem,
                           const int64_t *__restrict__ cur_off, int nh, const double *__restrict__ hred,
                           const double *__restrict__ sred, double dist_factor, int *__restrict__ acc,
                           int *__restrict__ acc_size, int *__restrict__ owner) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
        const int64_t b = soff[g], e = soff[g + 1];
        const int h = owner_of(cur_off, nh, smem[b]);
        const double frac = (double)(e - b) / (double)(cur_off[h + 1] - cur_off[h]);
        bool ok = 0.6 > frac && frac > 0.01;
        if (ok) {
            const double *H = hred + (int64_t)h * HALMA_RED_NFIELDS;
            const double *S = sred + (int64_t)g * HALMA_RED_NFIELDS;
            const double dx = __dsub_rn(H[HALMA_RED_CX], S[HALMA_RED_CX]);
            const double dy = __dsub_rn(H[HALMA_RED_CY], S[HALMA_RED_CY]);
            const double dz = __dsub_rn(H[HALMA_RED_CZ], S[HALMA_RED_CZ]);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            ok = __dsqrt_rn(d2) > __dmul_rn(dist_factor, H[HALMA_RED_R05]);
        }
        acc[g] = ok ? 1 : 0;
        acc_size[g] = ok ? (int)(e - b) : 0;
        owner[g] = h;
    }
}

// Accepted sub-groups: their members (as snapshot indices, ascending) appended to the new
// groups' store and marked removed; one record {halo, level, rank in level, size, start}
// per accepted sub-group.
__global__ void take_kernel(int ng, const int64_t *__restrict__ soff, const int *__restrict__ smem,
                            const int *__restrict__ cur_mem, const int *__restrict__ acc,
                            const int *__restrict__ apos, const int *__restrict__ mpos,
                            const int *__restrict__ owner, int level, int rec_base, int64_t mem_base,
                            int *__restrict__ newmem, unsigned char *__restrict__ removed,
                            long long *__restrict__ rec) {
    for (int g = blockIdx.x; g < ng; g += gridDim.x) {
        if (!acc[g]) continue;
        const int64_t b = soff[g], e = soff[g + 1];
        const int64_t dst = mem_base + mpos[g];
        for (int64_t k = b + threadIdx.x; k < e; k += blockDim.x) {
            const int r = smem[k];
            newmem[dst + (k - b)] = cur_mem[r];
            removed[r] = 1;
        }
        if (threadIdx.x == 0) {
            long long *o = rec + 5ll * (rec_base + apos[g]);
            o[0] = owner[g];
            o[1] = level;
            o[2] = apos[g];
            o[3] = e - b;
            o[4] = dst;
        }
    }
}

__global__ void keepflag_kernel(int64_t n, const unsigned char *__restrict__ removed, int *__restrict__ keep) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        keep[k] = removed[k] ? 0 : 1;
}

// Survivors in order: next_mem[pos[k]] = cur_mem[k]; next_off[h] = pos at the group's first
// row (the exclusive scan of the keep flags), next_off[nh] = survivors in total.
__global__ void compact_kernel(int64_t n, int nh, const int *__restrict__ keep, const int *__restrict__ pos,
                               const int *__restrict__ cur_mem, const int64_t *__restrict__ cur_off,
                               int *__restrict__ next_mem, int64_t *__restrict__ next_off) {
    const int64_t total = n > 0 ? (int64_t)pos[n - 1] + keep[n - 1] : 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        if (keep[k]) next_mem[pos[k]] = cur_mem[k];
    for (int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; h <= nh; h += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = cur_off[h];
        next_off[h] = r < n ? (int64_t)pos[r] : total;
    }
}

// Output assembly: plan entry q copies len ints from src (0 = survivors, 1 = new groups)
// at src_off to the output at dst_off.
__global__ void assemble_kernel(int nplan, const long long *__restrict__ plan, const int *__restrict__ cur_mem,
                                const int *__restrict__ newmem, int *__restrict__ out) {
    for (int q = blockIdx.x; q < nplan; q += gridDim.x) {
        const long long *p = plan + 4ll * q;
        const int *src = p[0] == 0 ? cur_mem : newmem;
        const long long so = p[1], d = p[2], len = p[3];
        for (long long k = threadIdx.x; k < len; k += blockDim.x) out[d + k] = src[so + k];
    }
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_fof_segmented(int64_t n, const double *x, const double *y, const double *z,
                                   int64_t n_segments, const int64_t *seg_offsets, double linking_length,
                                   int32_t *labels, int64_t *n_groups, halma_stream_t stream) {
    if (n < 0 || n_segments < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= INT32_MAX || n_segments >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles per call");
    if (!(linking_length >= 0.0) || !isfinite(linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and >= 0");
    if (!seg_offsets || (n > 0 && (!x || !y || !z || !labels))) return fail(HALMA_ERR_INVALID, "null pointer");
    if (n == 0 || n_segments == 0) {
        if (n > 0) return fail(HALMA_ERR_INVALID, "particles given but no segments");
        if (n_groups) *n_groups = 0;
        return HALMA_OK;
    }
    // the offsets must cover the rows exactly, in non-decreasing order (checked on the host)
    std::vector<int64_t> hoff(n_segments + 1);
    if (is_device_pointer(seg_offsets)) {
        HALMA_CUDA(cudaMemcpy(hoff.data(), seg_offsets, 8ull * (n_segments + 1), cudaMemcpyDeviceToHost));
    } else {
        memcpy(hoff.data(), seg_offsets, 8ull * (n_segments + 1));
    }
    if (hoff[0] != 0 || hoff[n_segments] != n) return fail(HALMA_ERR_INVALID, "segment offsets must run from 0 to n");
    for (int64_t s = 0; s < n_segments; ++s)
        if (hoff[s + 1] < hoff[s]) return fail(HALMA_ERR_INVALID, "segment offsets must not decrease");
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr;
    const int64_t *doff = nullptr;
    int32_t *dl = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(seg_offsets, n_segments + 1, true, false, &doff);
    sg.add((const int32_t *)labels, n, false, true, &dl);
    void *stage = nullptr;
    if (sg.any_host) {
        Layout L;
        sg.plan(L);
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
    }
    int s = sg.bind_and_upload(stage, st);
    if (s == HALMA_OK) s = fof_segmented_device((int)n, (int)n_segments, doff, dx, dy, dz, linking_length, dl, n_groups, st);
    if (s == HALMA_OK) s = sg.download(st);
    if (stage) {
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
    }
    return s;
}

extern "C" int halma_split_bridges(int64_t n, const double *x, const double *y, const double *z, const double *m,
                                   int64_t n_groups, const int64_t *group_offsets, const int32_t *group_members,
                                   const halma_substructure_params *params, int64_t *n_out, int64_t out_capacity,
                                   int64_t *out_offsets, int32_t *out_members, int64_t *n_cut,
                                   halma_stream_t stream) {
    if (!params || !n_out) return fail(HALMA_ERR_INVALID, "params and n_out must not be NULL");
    if (n < 0 || n_groups < 0 || out_capacity < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= INT32_MAX || n_groups >= INT32_MAX) return fail(HALMA_ERR_CAPACITY, "at most 2^31-2 particles per call");
    const halma_substructure_params p = *params;
    if (!(p.linking_length > 0.0) || !isfinite(p.linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and > 0");
    if (!(p.dec_factor > 1.0) || !isfinite(p.dec_factor)) return fail(HALMA_ERR_INVALID, "dec_factor must be > 1");
    if (!(p.min_ll >= 0.0) || !isfinite(p.min_ll)) return fail(HALMA_ERR_INVALID, "min_ll must be finite and >= 0");
    if (!isfinite(p.dist_factor)) return fail(HALMA_ERR_INVALID, "dist_factor must be finite");
    if (!group_offsets || (n_groups > 0 && !group_members) || (n > 0 && (!x || !y || !z || !m)))
        return fail(HALMA_ERR_INVALID, "null pointer");
    *n_out = 0;
    if (n_cut) *n_cut = 0;
    // group table on the host: validity and the starting sizes
    std::vector<int64_t> h_goff(n_groups + 1);
    if (is_device_pointer(group_offsets)) {
        HALMA_CUDA(cudaMemcpy(h_goff.data(), group_offsets, 8ull * (n_groups + 1), cudaMemcpyDeviceToHost));
    } else {
        memcpy(h_goff.data(), group_offsets, 8ull * (n_groups + 1));
    }
    if (h_goff[0] != 0) return fail(HALMA_ERR_INVALID, "group offsets must start at 0");
    for (int64_t g = 0; g < n_groups; ++g)
        if (h_goff[g + 1] < h_goff[g]) return fail(HALMA_ERR_INVALID, "group offsets must not decrease");
    const int64_t N0 = h_goff[n_groups];
    if (N0 > n) return fail(HALMA_ERR_INVALID, "groups hold more members than there are particles");
    const int nh = (int)n_groups;
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dm = nullptr;
    const int64_t *dgoff = nullptr;
    const int32_t *dgmem = nullptr;
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(m, n, true, false, &dm);
    sg.add(group_offsets, n_groups + 1, true, false, &dgoff);
    sg.add(group_members, N0, true, false, &dgmem);
    // level state (workspace slot 3; the FoF and reductions use slots 0 and 2)
    const int64_t NM = std::max<int64_t>(N0, 1);
    Layout L;
    sg.plan(L);
    const size_t o_off0 = L.add(8ull * (nh + 1)), o_off1 = L.add(8ull * (nh + 1));
    const size_t o_mem0 = L.add(4ull * NM), o_mem1 = L.add(4ull * NM), o_new = L.add(4ull * NM);
    const size_t o_g4 = L.add(32ull * NM), o_s4 = L.add(32ull * NM);
    const size_t o_lab = L.add(4ull * NM), o_soff = L.add(8ull * (NM + 1)), o_smem = L.add(4ull * NM);
    const size_t o_hred = L.add(8ull * HALMA_RED_NFIELDS * std::max(nh, 1));
    const size_t o_sred = L.add(8ull * HALMA_RED_NFIELDS * NM);
    const size_t o_acc = L.add(4ull * NM), o_asz = L.add(4ull * NM), o_own = L.add(4ull * NM);
    const size_t o_apos = L.add(4ull * NM), o_mpos = L.add(4ull * NM);
    const size_t o_rm = L.add(1ull * NM), o_keep = L.add(4ull * NM), o_pos = L.add(4ull * NM);
    const size_t o_rec = L.add(40ull * NM), o_out = L.add(4ull * NM);
    const size_t scan_b = exclusive_sum_i32_bytes((int)NM);
    const size_t o_tmp = L.add(scan_b);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 3));
    HALMA_TRY(sg.bind_and_upload(base, st));
    int64_t *off[2] = {at<int64_t>(base, o_off0), at<int64_t>(base, o_off1)};
    int *mem[2] = {at<int>(base, o_mem0), at<int>(base, o_mem1)};
    int *newmem = at<int>(base, o_new);
    double *g4 = at<double>(base, o_g4), *s4 = at<double>(base, o_s4);
    int *lab = at<int>(base, o_lab);
    int64_t *soff = at<int64_t>(base, o_soff);
    int *smem = at<int>(base, o_smem);
    double *hred = at<double>(base, o_hred), *sred = at<double>(base, o_sred);
    int *acc = at<int>(base, o_acc), *asz = at<int>(base, o_asz), *own = at<int>(base, o_own);
    int *apos = at<int>(base, o_apos), *mpos = at<int>(base, o_mpos);
    unsigned char *removed = at<unsigned char>(base, o_rm);
    int *keep = at<int>(base, o_keep), *pos = at<int>(base, o_pos);
    long long *rec = at<long long>(base, o_rec);
    int *dout = at<int>(base, o_out);
    void *tmp = at<void>(base, o_tmp);
    const int sms = device_sm_count();

    HALMA_CUDA(cudaMemcpyAsync(off[0], dgoff, 8ull * (nh + 1), cudaMemcpyDeviceToDevice, st));
    if (N0 > 0) {
        HALMA_CUDA(cudaMemcpyAsync(mem[0], dgmem, 4ull * N0, cudaMemcpyDeviceToDevice, st));
        int *bad = keep;   // scratch flag, the keep flags are written later
        HALMA_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
        HALMA_LAUNCH(check_members_kernel, std::min(sms * 8, grid_for(N0, 256)), 256, 0, st, N0, mem[0], off[0], nh,
                     n, bad);
        int hbad = 0;
        HALMA_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        if (hbad & 1) return fail(HALMA_ERR_INVALID, "group member outside [0, n)");
        if (hbad & 2) return fail(HALMA_ERR_INVALID, "group members must ascend strictly inside each group");
    }
    int cur = 0;
    int64_t ncur = N0, nnew = 0;
    int nrec = 0;
    const int minp_sub = std::max(p.minp_sub, 2);   // FoF groups have at least two members
    int level = 0;
    for (double sub_ll = p.linking_length / p.dec_factor; sub_ll > p.min_ll && ncur > 0 && nh > 0;
         sub_ll /= p.dec_factor, ++level) {
        const int g = std::min(sms * 8, grid_for(ncur, 256));
        double *gx = g4, *gy = g4 + ncur, *gz = g4 + 2 * ncur, *gm = g4 + 3 * ncur;
        HALMA_LAUNCH(gather4_kernel, g, 256, 0, st, ncur, mem[cur], dx, dy, dz, dm, gx, gy, gz, gm);
        // centre of mass and half-mass radius of every current list (velocities unused)
        HALMA_TRY(reductions_device(ncur, nh, off[cur], gx, gy, gz, gx, gy, gz, gm, nullptr, nullptr, hred, st));
        HALMA_TRY(fof_segmented_device((int)ncur, nh, off[cur], gx, gy, gz, sub_ll, lab, nullptr, st));
        int64_t ng = 0, nsm = 0;
        HALMA_TRY(fof_groups_device((int)ncur, lab, minp_sub, soff, smem, &ng, &nsm, st));
        if (ng == 0) continue;
        const int gs = std::min(sms * 8, grid_for(nsm, 256));
        double *qx = s4, *qy = s4 + nsm, *qz = s4 + 2 * nsm, *qm = s4 + 3 * nsm;
        HALMA_LAUNCH(gather4_kernel, gs, 256, 0, st, nsm, smem, gx, gy, gz, gm, qx, qy, qz, qm);
        HALMA_TRY(reductions_device(nsm, (int)ng, soff, qx, qy, qz, qx, qy, qz, qm, nullptr, nullptr, sred, st));
        HALMA_LAUNCH(cut_kernel, grid_for(ng, 128), 128, 0, st, (int)ng, soff, smem, off[cur], nh, hred, sred,
                     p.dist_factor, acc, asz, own);
        HALMA_TRY(exclusive_sum_i32(tmp, scan_b, acc, apos, (int)ng, st));
        HALMA_TRY(exclusive_sum_i32(tmp, scan_b, asz, mpos, (int)ng, st));
        int last[4];
        HALMA_CUDA(cudaMemcpyAsync(&last[0], apos + ng - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaMemcpyAsync(&last[1], acc + ng - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaMemcpyAsync(&last[2], mpos + ng - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaMemcpyAsync(&last[3], asz + ng - 1, 4, cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
        const int nacc = last[0] + last[1];
        const int64_t macc = (int64_t)last[2] + last[3];
        if (nacc == 0) continue;
        HALMA_CUDA(cudaMemsetAsync(removed, 0, ncur, st));
        HALMA_LAUNCH(take_kernel, (int)std::min<int64_t>(ng, sms * 8), 128, 0, st, (int)ng, soff, smem, mem[cur], acc,
                     apos, mpos, own, level, nrec, nnew, newmem, removed, rec);
        nrec += nacc;
        nnew += macc;
        HALMA_LAUNCH(keepflag_kernel, g, 256, 0, st, ncur, removed, keep);
        HALMA_TRY(exclusive_sum_i32(tmp, scan_b, keep, pos, (int)ncur, st));
        HALMA_LAUNCH(compact_kernel, g, 256, 0, st, ncur, nh, keep, pos, mem[cur], off[cur], mem[cur ^ 1],
                     off[cur ^ 1]);
        cur ^= 1;
        ncur -= macc;
    }

    // final lists and the accepted sub-groups, in the order the reference builds its list
    std::vector<int64_t> h_cur(nh + 1);
    std::vector<long long> h_rec(5ull * nrec);
    HALMA_CUDA(cudaMemcpyAsync(h_cur.data(), off[cur], 8ull * (nh + 1), cudaMemcpyDeviceToHost, st));
    if (nrec) HALMA_CUDA(cudaMemcpyAsync(h_rec.data(), rec, 40ull * nrec, cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    std::vector<int> order(nrec);
    for (int r = 0; r < nrec; ++r) order[r] = r;
    // records were appended level by level, each level in group order: a stable sort by
    // group keeps (level, rank) order inside a group
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return h_rec[5ull * a] < h_rec[5ull * b]; });
    std::vector<long long> plan;
    std::vector<int64_t> h_out{0};
    for (int h = 0; h < nh; ++h) {
        const int64_t len = h_cur[h + 1] - h_cur[h], start = h_goff[h + 1] - h_goff[h];
        // pyHALMA.py:751-755: emptied when less than 30 % of the particles are left
        if (start == 0 || (double)len / (double)start < 0.3) continue;
        if (len < p.minp) continue;   // good_groups(groups, MINP)
        plan.insert(plan.end(), {0, (long long)h_cur[h], (long long)h_out.back(), (long long)len});
        h_out.push_back(h_out.back() + len);
    }
    for (int r : order) {
        const long long *q = &h_rec[5ull * r];
        if (q[3] < p.minp) continue;
        plan.insert(plan.end(), {1, q[4], (long long)h_out.back(), q[3]});
        h_out.push_back(h_out.back() + q[3]);
    }
    const int64_t G = (int64_t)h_out.size() - 1;
    *n_out = G;
    if (n_cut) *n_cut = nrec;
    if (G > out_capacity) return fail(HALMA_ERR_CAPACITY, "%lld groups out, capacity %lld", (long long)G,
                                      (long long)out_capacity);
    if (!out_offsets || (h_out.back() > 0 && !out_members)) return fail(HALMA_ERR_INVALID, "null output pointer");
    const int nplan = (int)(plan.size() / 4);
    if (nplan > 0) {
        // the plan goes up in the group-record buffer (no longer needed)
        if (plan.size() > 5ull * NM) return fail(HALMA_ERR_CAPACITY, "assembly plan exceeds its buffer");
        HALMA_CUDA(cudaMemcpyAsync(rec, plan.data(), 8ull * plan.size(), cudaMemcpyHostToDevice, st));
        HALMA_LAUNCH(assemble_kernel, std::min(nplan, sms * 8), 256, 0, st, nplan, rec, mem[cur], newmem, dout);
    }
    HALMA_CUDA(cudaMemcpyAsync(out_offsets, h_out.data(), 8ull * (G + 1), cudaMemcpyDefault, st));
    if (h_out.back() > 0)
        HALMA_CUDA(cudaMemcpyAsync(out_members, dout, 4ull * h_out.back(), cudaMemcpyDefault, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    return HALMA_OK;
}
