// End-to-end halo finding for one snapshot: FoF -> groups with >= min_members members in the
// reference order (pyHALMA.py:555-592) -> members gathered into halo-contiguous FP64 arrays
// -> batched iterative unbinding -> bound flags scattered back to the snapshot order.
#include <math.h>
#include <string.h>

#include <map>
#include <string>
#include <thread>

#include "common.cuh"
#include "unbind.cuh"

namespace halma {
namespace {

// Members gathered into halo-contiguous arrays: field f of member k goes to
// out[col[f] * nm + k] (the 7 x nm array x, y, z, vx, vy, vz, m).
template <int NF>
struct GatherSrc {
    const double *src[NF];
    int col[NF];
};

template <int NF>
__global__ void gather_kernel(int64_t nm, const int *__restrict__ members, GatherSrc<NF> g,
                              double *__restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x) {
        const int i = members[k];
        double v[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) v[f] = g.src[f][i];
#pragma unroll
        for (int f = 0; f < NF; ++f) out[g.col[f] * nm + k] = v[f];
    }
}

__global__ void scatter_bound_kernel(int64_t nm, const int *__restrict__ members, const unsigned char *__restrict__ bs,
                                     unsigned char *__restrict__ bound) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nm; k += (int64_t)gridDim.x * blockDim.x)
        bound[members[k]] = bs[k];
}

// A second stream per device, for the host-to-device copies of the masses and velocities,
// which overlap the FoF stage (it reads positions only), for the gather of the velocities,
// which overlaps the first unbinding pass's pair kernels, and for the copies of the labels and
// the groups to the caller, which overlap the unbinding.
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t pos = nullptr;       // the positions' uploads have been issued on the main stream
    cudaEvent_t mass = nullptr;      // the masses are on the device
    cudaEvent_t done = nullptr;      // all uploads are done
    cudaEvent_t members = nullptr;   // the groups' member lists are final (main stream)
    cudaEvent_t vel = nullptr;       // the members' velocities are gathered
    cudaEvent_t groups = nullptr;    // labels and groups final, the halo offsets read
};

int side_stream(SideStream **out) {
    static std::map<int, SideStream> m;
    SideStream &ss = m[current_device()];
    if (!ss.s) {
        HALMA_CUDA(cudaStreamCreateWithFlags(&ss.s, cudaStreamNonBlocking));
        for (cudaEvent_t *e : {&ss.pos, &ss.mass, &ss.done, &ss.members, &ss.vel, &ss.groups})
            HALMA_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    *out = &ss;
    return HALMA_OK;
}

// One output of the early copies: caller's destination, device source, bytes.
struct OutCopy {
    void *user;
    const void *dev;
    size_t bytes;
};

// The labels and the groups to the caller's buffers (host or device) on the side stream once
// `groups` has fired, waiting for the copies to end.  Runs on a helper thread while the
// calling thread drives the unbinding: a copy to pageable host memory returns only when it is
// complete.  (Staging them through pinned memory and a CPU memcpy measured far slower: the
// CUDA driver's own pageable path writes fresh pages much faster than a memcpy that faults them in.)
int copy_groups_out(int dev, SideStream *side, const OutCopy *outs, int nout) {
    HALMA_CUDA(cudaSetDevice(dev));
    HALMA_CUDA(cudaStreamWaitEvent(side->s, side->groups, 0));
    for (int k = 0; k < nout; ++k)
        if (outs[k].user && outs[k].bytes)
            HALMA_CUDA(cudaMemcpyAsync(outs[k].user, outs[k].dev, outs[k].bytes, cudaMemcpyDefault, side->s));
    HALMA_CUDA(cudaStreamSynchronize(side->s));
    return HALMA_OK;
}

// Joins a helper thread on every way out of the scope that started it.
struct JoinOnExit {
    std::thread &t;
    ~JoinOnExit() {
        if (t.joinable()) t.join();
    }
};

// Waits for a stream on every way out of a scope (no copy from the caller's host buffers
// outlives the call that was given them, whatever error ended it).
struct SyncOnExit {
    cudaStream_t s;
    ~SyncOnExit() { cudaStreamSynchronize(s); }
};

}  // namespace
}  // namespace halma

using namespace halma;

extern "C" int halma_find_haloes(int64_t n, const double *x, const double *y, const double *z, const double *vx,
                                 const double *vy, const double *vz, const double *m, double linking_length,
                                 int32_t min_members, const halma_unbind_params *params, int32_t *labels,
                                 uint8_t *bound, int64_t *n_haloes, int64_t halo_capacity, int64_t *halo_offsets,
                                 int32_t *members, double *halo_out, halma_stream_t stream) {
    if (!params || !n_haloes) return fail(HALMA_ERR_INVALID, "params and n_haloes must not be NULL");
    if (n < 0 || halo_capacity < 0) return fail(HALMA_ERR_INVALID, "negative size");
    if (n >= (1ll << 31) - 64) return fail(HALMA_ERR_CAPACITY, "at most 2^31-65 particles per call");
    if (!(linking_length >= 0.0) || !isfinite(linking_length))
        return fail(HALMA_ERR_INVALID, "linking length must be finite and >= 0");
    const halma_unbind_params p = *params;
    if (!(p.eps > 0.0) || !isfinite(p.eps)) return fail(HALMA_ERR_INVALID, "eps must be finite and > 0");
    if (p.max_iter < 1 || p.max_iter > 1000) return fail(HALMA_ERR_INVALID, "max_iter must be in [1, 1000]");
    if (p.precision != HALMA_UNBIND_FP32C && p.precision != HALMA_UNBIND_FP64)
        return fail(HALMA_ERR_INVALID, "unknown precision %d", p.precision);
    if (n > 0 && (!x || !y || !z || !vx || !vy || !vz || !m)) return fail(HALMA_ERR_INVALID, "null input pointer");
    *n_haloes = 0;
    if (n == 0) {
        if (halo_offsets) {
            int64_t zero = 0;
            if (is_device_pointer(halo_offsets)) HALMA_CUDA(cudaMemcpy(halo_offsets, &zero, 8, cudaMemcpyHostToDevice));
            else halo_offsets[0] = 0;
        }
        return HALMA_OK;
    }
    std::lock_guard<std::mutex> guard(api_mutex());
    cudaStream_t st = (cudaStream_t)stream;
    Stager sg;
    const double *dx = nullptr, *dy = nullptr, *dz = nullptr, *dvx = nullptr, *dvy = nullptr, *dvz = nullptr,
                 *dm = nullptr;
    SideStream *side = nullptr;
    HALMA_TRY(side_stream(&side));
    SyncOnExit side_idle{side->s};
    sg.add(x, n, true, false, &dx);
    sg.add(y, n, true, false, &dy);
    sg.add(z, n, true, false, &dz);
    sg.add(m, n, true, false, &dm, true);
    sg.add_mark(side->mass, true);
    sg.add(vx, n, true, false, &dvx, true);
    sg.add(vy, n, true, false, &dvy, true);
    sg.add(vz, n, true, false, &dvz, true);
    // private scratch for everything that must outlive the individual stages
    Layout L;
    sg.plan(L);
    const size_t o_lab = L.add(4ull * n), o_off = L.add(8ull * (n + 1)), o_mem = L.add(4ull * n);
    const size_t o_g7 = L.add(8ull * 7 * n), o_bs = L.add(1ull * n), o_bnd = L.add(1ull * n);
    const size_t o_halo = L.add(8ull * HALMA_UB_NFIELDS * (size_t)std::max<int64_t>(n / 2 + 1, 1));
    // cached across calls: no allocation in the steady state, and stable addresses let the
    // unbinding stage replay its captured graph
    struct {
        void *p = nullptr;
    } buf;
    HALMA_TRY(workspace(L.total, &buf.p, st, 1));
    // masses and velocities from host memory are copied on a side stream while FoF runs, after
    // the positions (so that the positions, which FoF waits for, have the link to themselves);
    // the masses first, which the first unbinding pass needs from its start
    HALMA_TRY(sg.bind_and_upload(buf.p, st, side->s, side->pos));
    HALMA_CUDA(cudaEventRecord(side->done, side->s));
    int *dlab = at<int>(buf.p, o_lab);
    int64_t *doff = at<int64_t>(buf.p, o_off);
    int *dmem = at<int>(buf.p, o_mem);
    double *g7 = at<double>(buf.p, o_g7);
    unsigned char *bs = at<unsigned char>(buf.p, o_bs), *dbnd = at<unsigned char>(buf.p, o_bnd);
    double *dhalo = at<double>(buf.p, o_halo);

    Profile &prof = profile();
    cudaEvent_t ev[4] = {};
    if (prof.enabled) {
        for (auto &e : ev) HALMA_CUDA(cudaEventCreate(&e));
        HALMA_CUDA(cudaEventRecord(ev[0], st));
    }
    HALMA_TRY(fof_device((int)n, dx, dy, dz, linking_length, dlab, nullptr, st));
    int64_t ng = 0, nm = 0;
    HALMA_TRY(fof_groups_device((int)n, dlab, std::max(min_members, 1), doff, dmem, &ng, &nm, st));
    HALMA_TRY(prof.fof_mark(Profile::kFofStages, st));
    if (prof.enabled) HALMA_CUDA(cudaEventRecord(ev[1], st));
    *n_haloes = ng;
    // the labels and the groups are final: their copies to the caller run during the unbinding
    const bool fits = !(ng > halo_capacity && (halo_offsets || halo_out));
    int early_status = HALMA_OK;
    std::string early_msg;
    std::thread early;
    JoinOnExit join_early{early};
    const OutCopy outs[3] = {{labels, dlab, 4ull * n}, {halo_offsets, doff, 8ull * (ng + 1)}, {members, dmem, 4ull * nm}};
    HALMA_CUDA(cudaMemsetAsync(dbnd, 0, n, st));
    // Velocities copied from host memory are waited for only by the first pass's energy
    // kernel (FP32C path): on a slow host link their upload then overlaps the first pass's
    // pair kernels instead of delaying the unbinding's start.
    const bool defer_vel = p.precision == HALMA_UNBIND_FP32C &&
                           (!is_device_pointer(vx) || !is_device_pointer(vy) || !is_device_pointer(vz));
    HALMA_CUDA(cudaStreamWaitEvent(st, defer_vel ? side->mass : side->done, 0));
    const int g = std::min(device_sm_count() * 8, grid_for(std::max<int64_t>(nm, 1), 256));
    std::vector<int64_t> h_off(ng + 1);
    if (ng > 0) {
        if (defer_vel) {
            HALMA_LAUNCH(gather_kernel<4>, g, 256, 0, st, nm, dmem, (GatherSrc<4>{{dx, dy, dz, dm}, {0, 1, 2, 6}}), g7);
            HALMA_CUDA(cudaEventRecord(side->members, st));
            HALMA_CUDA(cudaStreamWaitEvent(side->s, side->members, 0));
            HALMA_LAUNCH(gather_kernel<3>, g, 256, 0, side->s, nm, dmem, (GatherSrc<3>{{dvx, dvy, dvz}, {3, 4, 5}}),
                         g7);
            HALMA_CUDA(cudaEventRecord(side->vel, side->s));
        } else {
            HALMA_LAUNCH(gather_kernel<7>, g, 256, 0, st, nm, dmem,
                         (GatherSrc<7>{{dx, dy, dz, dvx, dvy, dvz, dm}, {0, 1, 2, 3, 4, 5, 6}}), g7);
        }
        HALMA_CUDA(cudaMemcpyAsync(h_off.data(), doff, 8ull * (ng + 1), cudaMemcpyDeviceToHost, st));
        HALMA_CUDA(cudaStreamSynchronize(st));
    }
    // started only now, so that the halo offsets above did not queue behind them on the
    // device-to-host copy engine
    if (fits) {
        HALMA_CUDA(cudaEventRecord(side->groups, st));
        const int dev = current_device();
        early = std::thread([&, dev]() {
            early_status = copy_groups_out(dev, side, outs, 3);
            if (early_status != HALMA_OK) early_msg = halma_last_error();
        });
    }
    if (ng > 0) {
        if (prof.enabled) HALMA_CUDA(cudaEventRecord(ev[2], st));
        HALMA_TRY(unbind_device(nm, (int)ng, doff, h_off.data(), g7, g7 + nm, g7 + 2 * nm, g7 + 3 * nm, g7 + 4 * nm,
                                g7 + 5 * nm, g7 + 6 * nm, p, bs, nullptr, dhalo, st, defer_vel ? side->vel : nullptr));
        if (prof.enabled) HALMA_CUDA(cudaEventRecord(ev[3], st));
        HALMA_LAUNCH(scatter_bound_kernel, g, 256, 0, st, nm, dmem, bs, dbnd);
    }
    if (prof.enabled) {
        HALMA_CUDA(cudaStreamSynchronize(st));
        float a = 0.f, b = 0.f;
        HALMA_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
        if (ng > 0) HALMA_CUDA(cudaEventElapsedTime(&b, ev[2], ev[3]));
        prof.fof_ms = a;
        prof.unbind_ms = b;
        for (int k = 0; k < Profile::kFofStages; ++k) {
            float t = 0.f;
            HALMA_CUDA(cudaEventElapsedTime(&t, prof.fev[k], prof.fev[k + 1]));
            prof.fof_stage_ms[k] = t;
        }
        for (auto &e : ev) cudaEventDestroy(e);
    }
    // outputs (host or device)
    auto put = [&](void *user, const void *dev, size_t bytes) -> int {
        if (!user || bytes == 0) return HALMA_OK;
        HALMA_CUDA(cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDefault, st));
        return HALMA_OK;
    };
    HALMA_TRY(put(bound, dbnd, 1ull * n));
    if (!fits) {
        HALMA_TRY(put(labels, dlab, 4ull * n));
        HALMA_CUDA(cudaStreamSynchronize(st));
        return fail(HALMA_ERR_CAPACITY, "%lld haloes found, capacity %lld", (long long)ng, (long long)halo_capacity);
    }
    HALMA_TRY(put(halo_out, dhalo, 8ull * HALMA_UB_NFIELDS * ng));
    HALMA_CUDA(cudaStreamSynchronize(st));
    early.join();
    if (early_status != HALMA_OK) return fail(early_status, "%s", early_msg.c_str());
    return HALMA_OK;
}

extern "C" int halma_set_profiling(int32_t on) {
    std::lock_guard<std::mutex> guard(api_mutex());
    profile().enabled = on != 0;
    return HALMA_OK;
}

extern "C" int halma_profile_fof_stages(double *out, int32_t cap) {
    std::lock_guard<std::mutex> guard(api_mutex());
    const Profile &p = profile();
    for (int i = 0; out && i < cap && i < Profile::kFofStages; ++i) out[i] = p.fof_stage_ms[i];
    return Profile::kFofStages;
}

extern "C" int halma_profile_stats(double *out, int32_t cap) {
    std::lock_guard<std::mutex> guard(api_mutex());
    const Profile &p = profile();
    std::vector<double> v = {p.fof_ms, p.unbind_ms, (double)p.passes.size()};
    for (const auto &q : p.passes) {
        v.push_back(q.pairs);
        v.push_back(q.ms);
        v.push_back(q.sym_pairs);
        v.push_back(q.sym_ms);
    }
    if (out)
        for (int i = 0; i < cap && i < (int)v.size(); ++i) out[i] = v[i];
    return (int)v.size();
}
