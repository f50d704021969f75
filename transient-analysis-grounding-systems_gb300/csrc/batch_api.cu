// One-call batched entry points of the C-ABI (host code):
//   tags_gpu_solve_batch  many grids x many Laplace samples: one grid batch
//                         (grid_batch.cu: every grid a branch of one CUDA
//                         graph); grids too large to be resident together run
//                         as plans from a few host threads instead (each plan
//                         owns its stream, workspaces and graphs);
//   tags_gpu_inlt         the batched inverse Laplace transform.
// They replace the per-grid, per-sample OpenMP loops the reference's examples
// write around the library (examples/three_grids.c:286-465).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tags_gpu.h"

extern "C" int tags_gpu_solve_batch(const tags_grid_job* jobs, size_t njobs, int precision, double mur,
                                    size_t max_batch, int workers) {
    if (njobs == 0) return 0;
    if (!jobs) return TAGS_E_ARG;
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        if (!j.electrodes || !j.nodes || (j.ns && (!j.s || !j.kappa)) || j.num_electrodes == 0 || j.num_nodes == 0)
            return TAGS_E_ARG;
        if (!j.ie && j.inj_node >= j.num_nodes) return TAGS_E_ARG;
    }
    {
        // all grids in one graph when they fit in device memory together
        std::vector<tags_grid_job> live;
        for (size_t q = 0; q < njobs; ++q)
            if (jobs[q].ns) live.push_back(jobs[q]);
        if (live.empty()) return 0;
        tags_batch b = nullptr;
        int e = tags_batch_create(&b, live.data(), live.size(), precision, mur, max_batch);
        if (e == 0) {
            e = tags_batch_run(b, live.data(), live.size(), nullptr);
            tags_batch_destroy(b);
            return e;
        }
        if (e != TAGS_E_NOMEM) return e;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return TAGS_E_CUDA;
    const int nw = (int)std::max<size_t>(1, std::min<size_t>(njobs, workers > 0 ? (size_t)workers : 4));
    std::atomic<size_t> next{0};
    std::atomic<int> first_err{0};
    auto worker = [&]() {
        // the calling thread's device, in every worker
        if (cudaSetDevice(device) != cudaSuccess) {
            int z = 0;
            first_err.compare_exchange_strong(z, TAGS_E_CUDA);
            return;
        }
        for (size_t q = next++; q < njobs; q = next++) {
            const tags_grid_job& j = jobs[q];
            if (j.ns == 0) continue;
            tags_plan plan = nullptr;
            const size_t batch = max_batch ? max_batch : std::min<size_t>(j.ns, 256);
            int e = tags_plan_create(&plan, j.electrodes, j.images, j.num_electrodes, j.nodes, j.num_nodes, precision,
                                     batch);
            if (!e) e = tags_plan_run(plan, j.s, j.kappa, mur, j.ns, j.ie, j.inj_node, j.sol, j.info, 0, nullptr);
            if (plan) tags_plan_destroy(plan);
            if (e) {
                int z = 0;
                first_err.compare_exchange_strong(z, e);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 1; w < nw; ++w) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    return first_err.load();
}

extern "C" int tags_gpu_inlt(double* f, const tags_cdouble* g, const tags_cdouble* s, double tmax, size_t nt,
                             size_t nseries, int filter, int flags) {
    return tags_inv_laplace_batch(f, g, s, tmax, nt, nseries, filter, flags);
}
