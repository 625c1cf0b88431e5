// Library-wide C ABI helpers: version string and per-thread last CUDA error.
#include <stdio.h>

#include <atomic>
#include <mutex>

#include "common.cuh"

namespace fvgb {
namespace {
thread_local char g_last_error[256] = "";
std::atomic<unsigned long long> g_launches{0};
}

void record_message(const char *msg) { snprintf(g_last_error, sizeof(g_last_error), "%s", msg); }

void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

int record_cuda(cudaError_t e) {
    if (e == cudaSuccess) return FVGB_OK;
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
    return FVGB_ECUDA;
}

int device_sm_count() {
    static std::mutex mu;
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

}  // namespace fvgb

extern "C" const char *fvgb_version(void) { return "fvdb_gb300 0.1.0 (sm_103a)"; }

extern "C" const char *fvgb_last_error(void) { return fvgb::g_last_error; }

extern "C" uint64_t fvgb_launch_count(void) { return fvgb::g_launches.load(std::memory_order_relaxed); }
