// Shared host/device helpers for libhalma_gb300: status handling, the cached device
// workspace, host/device pointer staging and launch accounting.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include <mutex>
#include <type_traits>
#include <vector>

#include "halma.h"

namespace halma {

// Records a formatted failure reason for halma_last_error() on this thread; returns status.
int fail(int status, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define HALMA_CUDA(expr)                                                          \
    do {                                                                          \
        cudaError_t _e = (expr);                                                  \
        if (_e != cudaSuccess) return ::halma::cuda_fail(_e, #expr, __FILE__, __LINE__); \
    } while (0)

#define HALMA_TRY(expr)                                                           \
    do {                                                                          \
        int _s = (expr);                                                          \
        if (_s != HALMA_OK) return _s;                                            \
    } while (0)

// Every kernel launch of this library goes through HALMA_LAUNCH so that the number of
// launches is known (halma_kernel_launch_count) and launch errors are caught at once.
void count_launch();
void add_launches(int64_t k);   // graph replays: one count per captured kernel node
#define HALMA_LAUNCH(kernel, grid, block, smem, stream, ...)                      \
    do {                                                                          \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);               \
        ::halma::count_launch();                                                  \
        HALMA_CUDA(cudaGetLastError());                                           \
    } while (0)

int device_sm_count();          // SMs of the current device (cached per device)
int current_device();

// One process-wide lock serialises the entry points that use the cached workspace.
std::mutex &api_mutex();

// Bump layout: collect sizes first, then carve one workspace allocation.
struct Layout {
    size_t total = 0;
    size_t add(size_t bytes, size_t align = 256) {
        total = (total + align - 1) / align * align;
        size_t off = total;
        total += bytes;
        return off;
    }
};

// Returns a device buffer of at least `bytes`, cached per device and slot and grown on
// demand.  Slot 0 is the scratch of one stage (FoF, unbinding, potentials); slot 1 holds what
// the one-call pipeline keeps across its stages.  The others: 2 segmented-FoF geometry, 3
// bridge splitting, 4 / 5 / 8 ball gather, 6 phase-space cleaning, 7 properties, 9 symmetric
// potentials, 10 the FoF neighbour table, 11 / 12 the periodic FoF's images.  Slot 0 is reused by consecutive stages; what must
// survive a call into another stage lives in a slot that no stage it calls uses.
int workspace(size_t bytes, void **ptr, cudaStream_t stream, int slot = 0);

template <class T>
inline T *at(void *base, size_t off) { return reinterpret_cast<T *>(static_cast<char *>(base) + off); }

bool is_device_pointer(const void *p);

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Collects the caller's arrays of one call.  Host arrays get a slice of the workspace
// (planned into the same Layout as the call's scratch), inputs are uploaded before the
// kernels and outputs downloaded after them; device arrays are used in place.
struct Stager {
    struct Item {
        const void *user;
        size_t bytes;
        bool in, out, host;
        size_t off;
        void **slot;
        bool late;   // uploaded on the late stream of bind_and_upload, when one is given
        cudaEvent_t mark = nullptr;   // a marker, not an array: the event recorded at this point
    };
    std::vector<Item> items;
    bool any_host = false;

    // `slot` receives the device pointer the kernels must use.
    template <class T, class U>
    void add(const T *user, size_t count, bool in, bool out, U **slot, bool late = false) {
        Item it{user, count * sizeof(T), in, out, false, 0,
                reinterpret_cast<void **>(const_cast<typename std::remove_const<U>::type **>(slot)), late};
        if (user && count > 0) it.host = !is_device_pointer(user);
        any_host |= it.host;
        items.push_back(it);
    }
    // Records ev on the stream of the copies before it (s, or late_s for late), once those
    // copies have been issued.
    void add_mark(cudaEvent_t ev, bool late = false) {
        Item it{nullptr, 0, false, false, false, 0, nullptr, late};
        it.mark = ev;
        items.push_back(it);
    }
    void plan(Layout &L) {
        for (auto &it : items)
            if (it.host) it.off = L.add(it.bytes);
    }
    // Host inputs are copied on s, or (items added as late) on late_s, which the caller makes
    // s wait for before their first use.  With after_ev, the late copies start once the copies
    // on s have been done (after_ev is recorded on s and late_s waits for it).
    int bind_and_upload(void *base, cudaStream_t s, cudaStream_t late_s = nullptr, cudaEvent_t after_ev = nullptr) {
        for (int pass = 0; pass < 2; ++pass) {   // the items on s first, then the late ones
            if (pass == 1 && late_s && after_ev) {
                HALMA_CUDA(cudaEventRecord(after_ev, s));
                HALMA_CUDA(cudaStreamWaitEvent(late_s, after_ev, 0));
            }
            for (auto &it : items) {
                const bool late = it.late && late_s;
                if (late != (pass == 1)) continue;
                if (it.mark) {
                    HALMA_CUDA(cudaEventRecord(it.mark, late ? late_s : s));
                    continue;
                }
                if (!it.user || it.bytes == 0) {
                    *it.slot = const_cast<void *>(it.user);
                    continue;
                }
                if (it.host) {
                    *it.slot = at<void>(base, it.off);
                    if (it.in)
                        HALMA_CUDA(cudaMemcpyAsync(*it.slot, it.user, it.bytes, cudaMemcpyHostToDevice,
                                                   late ? late_s : s));
                } else {
                    *it.slot = const_cast<void *>(it.user);
                }
            }
        }
        return HALMA_OK;
    }
    int download(cudaStream_t s) {
        for (auto &it : items)
            if (it.host && it.out && it.bytes)
                HALMA_CUDA(cudaMemcpyAsync(const_cast<void *>(it.user), *it.slot, it.bytes,
                                           cudaMemcpyDeviceToHost, s));
        if (any_host) HALMA_CUDA(cudaStreamSynchronize(s));
        return HALMA_OK;
    }
};

inline int grid_for(int64_t n, int block, int cap = 1 << 30) {
    int64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

}  // namespace halma
