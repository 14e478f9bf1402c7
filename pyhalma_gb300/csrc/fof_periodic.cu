// Friends-of-friends in a periodic box (opt-in; the reference's fof.py builds its KDTree
// without a box size, so halma_fof is non-periodic like it).  Positions lie in [0, box)^3 and
// two particles are friends when their nearest-image distance is within the linking length.
//
// Images: every particle within the linking length (plus a rounding margin) of a face gets a
// copy shifted by +box or -box across it, one per combination of the faces it is near (up to
// 7 at a corner).  The plain exact FoF (fof_device) of the originals and their images then
// sees every pair that links across a face as an original-image pair, inside the box's
// non-periodic cell grid.  The components of that extended set are merged through the image
// map: a lock-free union-find over the original indices (the larger root hooked under the
// smaller, so a root is its tree's smallest index) joins the original of every extended
// particle with the original of its component's label.  A particle's label is its root when
// it or one of its images had a friend, else -1.  A particle cannot be its own image's friend
// because the box must be at least three linking lengths wide.
#include <math.h>
#include <limits.h>

#include "common.cuh"
#include "sort.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

constexpr int kMergeCap = 1 << 26;   // bound on any union-find loop here (never reached)

// Image flags per axis: bit 0 an image at v + box (v near 0), bit 1 at v - box (v near box).
__device__ __forceinline__ int face_flags(double v, double lim_lo, double lim_hi) {
    return (v < lim_lo ? 1 : 0) | (v >= lim_hi ? 2 : 0);
}

__device__ __forceinline__ int image_count(int fx, int fy, int fz) {
    return (fx ? 2 : 1) * (fy ? 2 : 1) * (fz ? 2 : 1) - 1;
}

// Images per particle (count[i]), and err[0] set when a position lies outside [0, box).
__global__ void image_count_kernel(int n, const double *__restrict__ x, const double *__restrict__ y,
                                   const double *__restrict__ z, double box, double lim_lo, double lim_hi,
                                   int *__restrict__ count, int *__restrict__ err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
        bool bad = false;
#pragma unroll
        for (int d = 0; d < 3; ++d) bad |= !(v[d] >= 0.0 && v[d] < box);
        if (bad) atomicOr(err, 1);
        count[i] = bad ? 0
                       : image_count(face_flags(v[0], lim_lo, lim_hi), face_flags(v[1], lim_lo, lim_hi),
                                     face_flags(v[2], lim_lo, lim_hi));
    }
}

// The extended set: originals at 0..n-1, particle i's images from n + pos[i] on (axis shifts
// in a fixed order: every non-empty subset of the flagged axes), orig[] = the original index
// of each image.
__global__ void image_emit_kernel(int n, const double *__restrict__ x, const double *__restrict__ y,
                                  const double *__restrict__ z, double box, double lim_lo, double lim_hi,
                                  const int *__restrict__ pos, double *__restrict__ ex, double *__restrict__ ey,
                                  double *__restrict__ ez, int *__restrict__ orig) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
        ex[i] = v[0];
        ey[i] = v[1];
        ez[i] = v[2];
        int f[3];
        double s[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            f[d] = face_flags(v[d], lim_lo, lim_hi);
            s[d] = (f[d] & 1) ? v[d] + box : v[d] - box;
        }
        int k = n + pos[i];
        for (int m = 1; m < 8; ++m) {   // subsets of the axes: bit d shifts axis d
            if (((m & 1) && !f[0]) || ((m & 2) && !f[1]) || ((m & 4) && !f[2])) continue;
            ex[k] = (m & 1) ? s[0] : v[0];
            ey[k] = (m & 2) ? s[1] : v[1];
            ez[k] = (m & 4) ? s[2] : v[2];
            orig[k - n] = i;
            ++k;
        }
    }
}

__device__ __forceinline__ int merge_find(int *parent, int v, int *err) {
    int p = __ldcg(parent + v);
    int guard = 0;
    while (p != v) {
        const int gp = __ldcg(parent + p);
        if (gp != p) __stcg(parent + v, gp);
        v = p;
        p = gp;
        if (++guard > kMergeCap) {
            atomicOr(err, 2);
            break;
        }
    }
    return v;
}

__device__ __forceinline__ void merge_union(int *parent, int a, int b, int *err) {
    a = merge_find(parent, a, err);
    b = merge_find(parent, b, err);
    int guard = 0;
    while (a != b) {
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicCAS(parent + a, a, b);
        if (old == a) return;
        a = merge_find(parent, old, err);
        b = merge_find(parent, b, err);
        if (++guard > kMergeCap) {
            atomicOr(err, 2);
            return;
        }
    }
}

__global__ void merge_init_kernel(int n, int *__restrict__ parent, unsigned char *__restrict__ has) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        parent[i] = i;
        has[i] = 0;
    }
}

// Every extended particle with a friend joins its original to the original of its label.
__global__ void merge_kernel(int n, int ne, const int *__restrict__ elabel, const int *__restrict__ orig,
                             int *parent, unsigned char *__restrict__ has, int *err) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int l = elabel[e];
        if (l < 0) continue;
        const int a = e < n ? e : orig[e - n];
        const int b = l < n ? l : orig[l - n];
        has[a] = 1;
        if (a != b) merge_union(parent, a, b, err);
    }
}

__global__ void merge_label_kernel(int n, int *parent, const unsigned char *__restrict__ has,
                                   int *__restrict__ labels, int *__restrict__ ngroups, int *err) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int r = merge_find(parent, i, err);
        labels[i] = has[i] ? r : -1;
        if (has[i] && r == i) atomicAdd(ngroups, 1);
    }
}

// Periodic FoF on device arrays.  The image counts live in workspace slot 11, the extended set
// and the merge state in slot 12 (fof_device uses slots 0 and 10).
int fof_periodic_device(int n, const double *x, const double *y, const double *z, double ll, double box,
                        int *labels, int64_t *n_groups, cudaStream_t st) {
    // images for every particle within ll of a face, with a margin far above the rounding of
    // v +- box (a pair that links across a face has both particles within ll of it)
    const double margin = ll * 1e-9 + box * 0x1p-40;
    const double lim_lo = ll + margin, lim_hi = box - ll - margin;
    const size_t scan_b = exclusive_sum_i32_bytes(n);
    Layout L;
    const size_t o_cnt = L.add(4ull * n), o_pos = L.add(4ull * n), o_flags = L.add(64), o_tmp = L.add(scan_b);
    void *base = nullptr;
    HALMA_TRY(workspace(L.total, &base, st, 11));
    int *cnt = at<int>(base, o_cnt), *pos = at<int>(base, o_pos), *flags = at<int>(base, o_flags);
    const int g1 = std::min(device_sm_count() * 8, grid_for(n, 256));
    HALMA_CUDA(cudaMemsetAsync(flags, 0, 64, st));
    HALMA_LAUNCH(image_count_kernel, g1, 256, 0, st, n, x, y, z, box, lim_lo, lim_hi, cnt, flags);
    HALMA_TRY(exclusive_sum_i32(at<void>(base, o_tmp), scan_b, cnt, pos, n, st));
    int h[3] = {0, 0, 0};
    HALMA_CUDA(cudaMemcpyAsync(h, pos + (n - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaMemcpyAsync(h + 1, cnt + (n - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaMemcpyAsync(h + 2, flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    if (h[2]) return fail(HALMA_ERR_INVALID, "periodic FoF: every position must lie in [0, box)");
    const int64_t images = (int64_t)h[0] + h[1], ne = n + images;
    if (ne >= INT_MAX) return fail(HALMA_ERR_CAPACITY, "periodic FoF: %lld particles with images", (long long)ne);
    Layout E;
    const size_t o_ex = E.add(8ull * ne), o_ey = E.add(8ull * ne), o_ez = E.add(8ull * ne);
    const size_t o_orig = E.add(4ull * std::max<int64_t>(images, 1)), o_elab = E.add(4ull * ne);
    const size_t o_par = E.add(4ull * n), o_has = E.add(1ull * n);
    void *ebase = nullptr;
    HALMA_TRY(workspace(E.total, &ebase, st, 12));
    double *ex = at<double>(ebase, o_ex), *ey = at<double>(ebase, o_ey), *ez = at<double>(ebase, o_ez);
    int *orig = at<int>(ebase, o_orig), *elab = at<int>(ebase, o_elab), *parent = at<int>(ebase, o_par);
    unsigned char *has = at<unsigned char>(ebase, o_has);
    HALMA_LAUNCH(image_emit_kernel, g1, 256, 0, st, n, x, y, z, box, lim_lo, lim_hi, pos, ex, ey, ez, orig);
    HALMA_TRY(fof_device((int)ne, ex, ey, ez, ll, elab, nullptr, st));
    HALMA_CUDA(cudaMemsetAsync(flags, 0, 64, st));
    HALMA_LAUNCH(merge_init_kernel, g1, 256, 0, st, n, parent, has);
    HALMA_LAUNCH(merge_kernel, std::min(device_sm_count() * 8, grid_for(ne, 256)), 256, 0, st, n, (int)ne, elab,
                 orig, parent, has, flags);
    HALMA_LAUNCH(merge_label_kernel, g1, 256, 0, st, n, parent, has, labels, flags + 1, flags);
    int r[2] = {0, 0};
    HALMA_CUDA(cudaMemcpyAsync(r, flags, sizeof(r), cudaMemcpyDeviceToHost, st));
    HALMA_CUDA(cudaStreamSynchronize(st));
    if (r[0]) return fail(HALMA_ERR_NOT_CONVERGED, "periodic FoF: union-find iteration cap reached");
    if (n_groups) *n_groups = r[1];
    return HALMA_OK;
}

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_fof_periodic(int64_t n, const double *x, const double *y, const double *z,
                                  double linking_length, double box, int32_t *labels, int64_t *n_groups,
                                  halma_stream_t stream) {
    if (n < 0) return fail(HALMA_ERR_INVALID, "negative particle count");
    if (!(linking_length >= 0.0) || !isfinite(linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and >= 0");
    if (!(box > 0.0) || !isfinite(box)) return fail(HALMA_ERR_INVALID, "box must be finite and > 0");
    if (box < 3.0 * linking_length)
        return fail(HALMA_ERR_INVALID, "the periodic box must be at least three linking lengths wide");
    if (n > 0 && (!x || !y || !z || !labels)) return fail(HALMA_ERR_INVALID, "null pointer");
    if (n >= INT_MAX / 8) return fail(HALMA_ERR_CAPACITY, "at most 2^28-1 particles per periodic call");
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
        Layout L;
        sg.plan(L);
        void *stage = nullptr;
        HALMA_CUDA(cudaMallocAsync(&stage, L.total, st));
        int s = sg.bind_and_upload(stage, st);
        if (s == HALMA_OK) s = fof_periodic_device((int)n, dx, dy, dz, linking_length, box, dl, n_groups, st);
        if (s == HALMA_OK) s = sg.download(st);
        cudaFreeAsync(stage, st);
        cudaStreamSynchronize(st);
        return s;
    }
    HALMA_TRY(sg.bind_and_upload(nullptr, st));
    return fof_periodic_device((int)n, dx, dy, dz, linking_length, box, dl, n_groups, st);
}
