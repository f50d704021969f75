// Per-kernel-family timing with CUDA events on the launching stream.
//
// When enabled (tags_gpu_profile), the library brackets each launch of the
// hot kernels with an event pair on the stream it launches on and records the
// algorithmic flops and bytes of that launch; tags_gpu_profile_read returns
// launches, device time and work per family. Disabled, it costs one branch.
#include <atomic>
#include <cstring>
#include <mutex>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

struct Family {
    const char* name;
    long long launches = 0;
    double flops = 0.0, bytes = 0.0;
    std::vector<cudaEvent_t> ev;     // start/end pairs
    size_t used = 0;                 // events in use (even)
};

const char* kNames[TAGS_PROF_N] = {"fill_fp64", "fill_mixed", "ldl_diag", "ldl_panel_gemm", "ldl_trailing_gemm",
                                   "ldl_solve", "residual_fp64", "build_fp32", "lu_fp64_gemm", "lu_fp64_other",
                                   "fields"};
Family g_fam[TAGS_PROF_N];
std::atomic<int> g_on{0};
std::mutex g_pm;

}  // namespace

int tags_prof_begin(int fam, cudaStream_t st) {
    if (!g_on.load(std::memory_order_relaxed)) return -1;
    // launches captured into a graph are not timed per family
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return -1;
    std::lock_guard<std::mutex> lk(g_pm);
    Family& f = g_fam[fam];
    if (f.used + 2 > f.ev.size()) {
        for (int q = 0; q < 2; ++q) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            f.ev.push_back(e);
        }
    }
    int slot = (int)f.used;
    f.used += 2;
    cudaEventRecord(f.ev[slot], st);
    return slot;
}

void tags_prof_end(int fam, int slot, cudaStream_t st, double flops, double bytes) {
    if (slot < 0) return;
    std::lock_guard<std::mutex> lk(g_pm);
    Family& f = g_fam[fam];
    cudaEventRecord(f.ev[slot + 1], st);
    f.launches++;
    f.flops += flops;
    f.bytes += bytes;
}

extern "C" int tags_gpu_profile(int enable) {
    std::lock_guard<std::mutex> lk(g_pm);
    for (auto& f : g_fam) {
        f.launches = 0;
        f.flops = f.bytes = 0.0;
        f.used = 0;
    }
    g_on.store(enable ? 1 : 0);
    return 0;
}

extern "C" int tags_gpu_profile_read(int family, long long* launches, double* ms, double* flops, double* bytes,
                                     char* name, int name_len) {
    if (family < 0 || family >= TAGS_PROF_N) return TAGS_E_ARG;
    std::lock_guard<std::mutex> lk(g_pm);
    Family& f = g_fam[family];
    double tot = 0.0;
    for (size_t q = 0; q + 1 < f.used; q += 2) {
        float t = 0.f;
        if (cudaEventSynchronize(f.ev[q + 1]) != cudaSuccess) return TAGS_E_CUDA;
        if (cudaEventElapsedTime(&t, f.ev[q], f.ev[q + 1]) == cudaSuccess) tot += t;
    }
    if (launches) *launches = f.launches;
    if (ms) *ms = tot;
    if (flops) *flops = f.flops;
    if (bytes) *bytes = f.bytes;
    if (name && name_len > 0) {
        strncpy(name, kNames[family], name_len - 1);
        name[name_len - 1] = 0;
    }
    return 0;
}
