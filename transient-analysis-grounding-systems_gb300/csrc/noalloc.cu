// Solve of the immittance system for callers that cannot allocate device memory.
//
// Some host programs run where they may not call cudaMalloc themselves and may
// not let a library do it either: code embedded in a larger GPU application
// that owns a fixed memory pool or a pre-sized arena, and code that must not
// allocate after start-up. They already hold device buffers for their own data;
// what they cannot provide is the solver's scratch. This entry point keeps that
// scratch (row interchanges and the status word) in one file-scope device array
// of fixed size, so a call allocates nothing.
//
// Limits and sharing: at most TAGS_NOALLOC_MAX_N unknowns; every GPU that loads
// the library holds the array (about 128 KiB) until the process exits; all
// calls on a device share it and it keeps the previous call's contents, so
// calls that overlap on the GPU (other host threads, other streams) race.
// The first call on each device looks up the array's device address; make that
// first call before any stream capture. The address is kept for the life of
// the process, so after cudaDeviceReset on a device the entry point must not
// be called on that device again (the cached address belongs to the context
// the reset destroyed).
#include <cstdio>
#include <mutex>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

constexpr size_t kMaxN = TAGS_NOALLOC_MAX_N;
// row interchanges (kMaxN ints) followed by the factorisation status word
static __device__ __align__(256) int g_noalloc_scratch[kMaxN + 64];

struct NoallocSetup {
    bool done = false;
    int* scratch = nullptr;     // device address of g_noalloc_scratch
};
NoallocSetup g_noalloc[64];
std::mutex g_noalloc_mutex;

}  // namespace

extern "C" int tags_solve_immittance_noalloc(tags_cdouble* d_wg, tags_cdouble* d_ie, size_t num_electrodes,
                                             size_t num_nodes, void* stream) {
    const size_t N = 2 * num_electrodes + num_nodes;
    if (N == 0) return 0;
    if (!d_wg || !d_ie) return tags_fail(TAGS_E_ARG, "tags_solve_immittance_noalloc: null pointer argument");
    if (N > kMaxN) {
        char msg[160];
        snprintf(msg, sizeof(msg),
                 "tags_solve_immittance_noalloc: %zu unknowns exceed the fixed scratch of %zu unknowns", N, kMaxN);
        return tags_fail(TAGS_E_ARG, msg);
    }
    int dev = 0;
    TAGS_CUDA_OK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return tags_fail(TAGS_E_ARG, "tags_solve_immittance_noalloc: device index out of range");
    int* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mutex);
        NoallocSetup& su = g_noalloc[dev];
        if (!su.done) {
            // the host-side name of the array is not a device address
            TAGS_CUDA_OK(cudaGetSymbolAddress((void**)&su.scratch, g_noalloc_scratch));
            su.done = true;
        }
        scratch = su.scratch;
    }
    cudaStream_t st = (cudaStream_t)stream;
    double2* W = reinterpret_cast<double2*>(d_wg);
    double2* x = reinterpret_cast<double2*>(d_ie);
    int* ipiv = scratch;
    int* info_d = scratch + kMaxN;
    const int n = (int)N;
    // factorise the caller's W_G in place (the reference's zsysv also
    // overwrites it), lower half read as in zsysv('L')
    int err = tags_symmetrize_lower(W, n, (long long)N, 0, 1, st);
    if (!err) err = tags_lu_z(W, n, (long long)N, 0, 1, 1, ipiv, info_d, st);
    if (err) return err;
    int info = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(&info, info_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (info > 0) return info;      // singular: ie left unchanged
    err = tags_lu_solve_z(W, n, (long long)N, 0, 1, ipiv, x, 1, (long long)N, 0, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}
