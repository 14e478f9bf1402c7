// Status strings, per-thread error text, cached workspace and launch accounting.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>
#include <map>

#include "common.cuh"

namespace halma {

static thread_local char g_last_error[512] = "";
static std::atomic<int64_t> g_launches{0};

int fail(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    int st = (e == cudaErrorMemoryAllocation) ? HALMA_ERR_NOMEM
             : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? HALMA_ERR_NO_DEVICE
                                                                             : HALMA_ERR_CUDA;
    return fail(st, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(int64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

std::mutex &api_mutex() {
    static std::mutex m;
    return m;
}

int current_device() {
    int d = 0;
    cudaGetDevice(&d);
    return d;
}

int device_sm_count() {
    static std::mutex m;
    static std::map<int, int> cache;
    int d = current_device();
    std::lock_guard<std::mutex> g(m);
    auto it = cache.find(d);
    if (it != cache.end()) return it->second;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || sms <= 0)
        sms = 148;
    cache[d] = sms;
    return sms;
}

struct WsEntry {
    void *ptr = nullptr;
    size_t bytes = 0;
};
static std::map<std::pair<int, int>, WsEntry> &ws_map() {   // (device, slot)
    static std::map<std::pair<int, int>, WsEntry> m;
    return m;
}

int workspace(size_t bytes, void **ptr, cudaStream_t stream, int slot) {
    int d = current_device();
    WsEntry &e = ws_map()[{d, slot}];
    if (bytes == 0) bytes = 256;
    if (e.bytes < bytes) {
        if (e.ptr) {
            // earlier work on any stream may still read the old buffer
            HALMA_CUDA(cudaDeviceSynchronize());
            HALMA_CUDA(cudaFree(e.ptr));
            e.ptr = nullptr;
            e.bytes = 0;
        }
        size_t want = bytes + bytes / 8;
        void *p = nullptr;
        cudaError_t err = cudaMalloc(&p, want);
        if (err != cudaSuccess) {
            cudaGetLastError();
            return fail(HALMA_ERR_NOMEM, "workspace allocation of %zu bytes failed: %s", want,
                        cudaGetErrorString(err));
        }
        e.ptr = p;
        e.bytes = want;
    }
    (void)stream;
    *ptr = e.ptr;
    return HALMA_OK;
}

bool is_device_pointer(const void *p) {
    if (!p) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace halma

extern "C" {

int halma_abi_version(void) { return HALMA_ABI_VERSION; }

const char *halma_status_string(int s) {
    switch (s) {
        case HALMA_OK: return "ok";
        case HALMA_ERR_INVALID: return "invalid argument";
        case HALMA_ERR_NOMEM: return "out of memory";
        case HALMA_ERR_CUDA: return "CUDA error";
        case HALMA_ERR_NOT_CONVERGED: return "not converged";
        case HALMA_ERR_TIMEOUT: return "device wait timed out";
        case HALMA_ERR_CAPACITY: return "capacity exceeded";
        case HALMA_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

const char *halma_last_error(void) { return halma::g_last_error; }

int64_t halma_kernel_launch_count(void) { return halma::g_launches.load(); }

int halma_release_workspace(void) {
    std::lock_guard<std::mutex> g(halma::api_mutex());
    for (auto &kv : halma::ws_map()) {
        if (kv.second.ptr) {
            cudaSetDevice(kv.first.first);
            cudaDeviceSynchronize();
            cudaFree(kv.second.ptr);
        }
    }
    halma::ws_map().clear();
    return HALMA_OK;
}

}  // extern "C"
