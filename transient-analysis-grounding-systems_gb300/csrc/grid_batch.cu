// Many grids of uneven size x many Laplace samples as ONE CUDA graph.
//
// The reference's examples loop over grids and, inside, over samples with
// OpenMP (examples/three_grids.c:286-443). Here a grid batch builds, once, a
// plan per grid (geometry, incidence, pair plan, workspaces) and device-
// resident input and output arrays for all of its samples, with the number of
// samples resident per grid admitted against the free device memory. One
// stream capture then records every grid's passes: each grid is a branch of
// the graph (its passes in sequence on its plan's buffers), the branches are
// independent, so the GPU runs grids of different sizes side by side; a pass
// is the plan's usual sequence (coefficients, right-hand sides, fill,
// factorisation, and for the mixed form the refinement as a conditional
// while-node), followed by copies of its solutions and its refinement state
// out of the plan. A run is the input copies, one cudaGraphLaunch, and the
// output copies; samples whose refinement did not converge (or whose
// tensor-core factorisation reported an error) are re-solved in plain FP64
// afterwards, from the snapshots of their pass.
#include <algorithm>
#include <numeric>
#include <vector>

#include <cuda_runtime.h>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

int tags_plan_coef(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur, int nb, cudaStream_t st);
int tags_plan_rhs(tags_plan_s* p, double2* d_X, const double2* d_ie, int inj_node, int nb, cudaStream_t st);

namespace {

struct GridSlot {
    tags_plan_s* plan = nullptr;
    int ns = 0, n = 0, m = 0, N = 0, per_pass = 0, passes = 0;
    int has_ie = 0;
    size_t inj = 0;
    double2* d_s = nullptr;      // ns
    double2* d_k = nullptr;      // ns
    double2* d_ie = nullptr;     // ns x n (or null)
    double2* d_sol = nullptr;    // ns x N
    int* d_info = nullptr;       // ns
    int* d_snap_i = nullptr;     // passes x (3 b + 2): active, converged, iterations, step, continue
    double* d_snap_d = nullptr;  // passes x 3 b: previous correction, max row sum, backward error
    int* d_snap_err = nullptr;   // passes x 2: tensor-core error words
};

struct Body {
    tags_plan_s* plan;
    int nb;
    cudaGraphConditionalHandle cond;
    cudaGraph_t graph;
};

}  // namespace

struct tags_batch_s {
    int device = 0;
    int precision = 0;
    double mur = 1.0;
    cudaStream_t stream = nullptr;
    std::vector<GridSlot> grids;
    std::vector<cudaEvent_t> events;
    cudaGraphExec_t exec = nullptr;
    long long launches_fixed = 0, launches_step = 0;
};

static void batch_free(tags_batch_s* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    for (auto& g : b->grids) {
        void* ptrs[] = {g.d_s, g.d_k, g.d_ie, g.d_sol, g.d_info, g.d_snap_i, g.d_snap_d, g.d_snap_err};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        if (g.plan) tags_plan_destroy(g.plan);
    }
    for (cudaEvent_t e : b->events) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

// Device bytes one resident sample of a plan needs (the estimate plan
// creation uses to size its batch).
static double bytes_per_sample(int m, int n, int precision) {
    const double N = (double)n + 2.0 * m, NN = N * N;
    return precision == TAGS_PLAIN_FP64 ? 16.0 * NN + 40.0 * N
                                        : 8.0 * NN + 32.0 * (double)m * m + 80.0 * N +
                                              (double)tags_ldl_tc_workspace((int)N, 1);
}

// One capture of every grid's passes (see the file comment).
static int capture_batch(tags_batch_s* b) {
    cudaStream_t s0 = b->stream;
    const long long l0 = tags_thread_launch_count();
    std::vector<Body> bodies;
    TAGS_CUDA_OK(cudaStreamBeginCapture(s0, cudaStreamCaptureModeRelaxed));
    int err = 0;
    cudaError_t ce = cudaEventRecord(b->events[0], s0);
    if (ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaEventRecord (fork)", __FILE__, __LINE__);
    // largest grids first: their branches are the longest
    std::vector<int> order(b->grids.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->grids[x].N > b->grids[y].N; });
    for (int gi : order) {
        if (err) break;
        GridSlot& g = b->grids[gi];
        tags_plan_s* p = g.plan;
        cudaStream_t st = p->stream;
        ce = cudaStreamWaitEvent(st, b->events[0], 0);
        if (ce != cudaSuccess) { err = tags_fail_cuda(ce, "cudaStreamWaitEvent (fork)", __FILE__, __LINE__); break; }
        const int bcap = p->batch;
        for (int q = 0; q < g.passes && !err; ++q) {
            const int k0 = q * g.per_pass, nb = std::min(g.per_pass, g.ns - k0);
            err = tags_plan_coef(p, g.d_s + k0, g.d_k + k0, b->mur, nb, st);
            if (!err) err = tags_plan_rhs(p, p->d_x, g.has_ie ? g.d_ie + (size_t)k0 * g.n : nullptr, (int)g.inj, nb, st);
            if (err) break;
            if (b->precision == TAGS_PLAIN_FP64) {
                err = tags_plan_run_plain(p, nullptr, nb, st);
            } else {
                Body bd{p, nb, 0, nullptr};
                err = tags_mixed_factor(p, nb, st);
                if (!err) err = tags_mixed_ir_setup(p, nb, st);
                if (!err) err = tags_plan_add_while_node(st, &bd.cond, &bd.graph);
                if (!err) bodies.push_back(bd);
            }
            if (err) break;
            ce = cudaMemcpyAsync(g.d_sol + (size_t)k0 * g.N, p->d_x, sizeof(double2) * (size_t)nb * g.N,
                                 cudaMemcpyDeviceToDevice, st);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(g.d_info + k0, p->d_info, sizeof(int) * nb, cudaMemcpyDeviceToDevice, st);
            if (ce == cudaSuccess && b->precision != TAGS_PLAIN_FP64) {
                ce = cudaMemcpyAsync(g.d_snap_i + (size_t)q * (3 * bcap + 2), p->d_iri, sizeof(int) * (3 * bcap + 2),
                                     cudaMemcpyDeviceToDevice, st);
                if (ce == cudaSuccess)
                    ce = cudaMemcpyAsync(g.d_snap_d + (size_t)q * 3 * bcap, p->d_ird, sizeof(double) * 3 * bcap,
                                         cudaMemcpyDeviceToDevice, st);
                if (ce == cudaSuccess)
                    ce = cudaMemcpyAsync(g.d_snap_err + 2 * q, p->d_ldlerr, sizeof(int) * 2, cudaMemcpyDeviceToDevice,
                                         st);
                // the next pass starts with a clear error word, as after a plan's pass
                if (ce == cudaSuccess) ce = cudaMemsetAsync(p->d_ldlerr, 0, sizeof(int) * 2, st);
            }
            if (ce != cudaSuccess) err = tags_fail_cuda(ce, "pass output copies", __FILE__, __LINE__);
        }
        if (err) break;
        ce = cudaEventRecord(b->events[1 + gi], st);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(s0, b->events[1 + gi], 0);
        if (ce != cudaSuccess) err = tags_fail_cuda(ce, "join", __FILE__, __LINE__);
    }
    cudaGraph_t graph = nullptr;
    ce = cudaStreamEndCapture(s0, &graph);
    if (!err && ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    const long long l1 = tags_thread_launch_count();
    // the refinement step of every while-node, captured into its body
    for (const Body& bd : bodies) {
        if (err) break;
        cudaStream_t st = bd.plan->stream;
        ce = cudaStreamBeginCaptureToGraph(st, bd.graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (ce != cudaSuccess) {
            err = tags_fail_cuda(ce, "cudaStreamBeginCaptureToGraph", __FILE__, __LINE__);
            break;
        }
        err = tags_mixed_ir_step(bd.plan, bd.nb, st, bd.cond, 1);
        cudaGraph_t g2 = nullptr;
        ce = cudaStreamEndCapture(st, &g2);
        if (!err && ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaStreamEndCapture (body)", __FILE__, __LINE__);
    }
    const long long l2 = tags_thread_launch_count();
    tags_note_launch(-(l2 - l0));      // captured, not launched
    if (!err) {
        ce = cudaGraphInstantiate(&b->exec, graph, 0);
        if (ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    if (graph) cudaGraphDestroy(graph);
    if (err) {
        cudaGetLastError();
        b->exec = nullptr;
        return err;
    }
    b->launches_fixed = l1 - l0;
    b->launches_step = bodies.empty() ? 0 : (l2 - l1) / (long long)bodies.size();
    return 0;
}

extern "C" int tags_batch_create(tags_batch* out, const tags_grid_job* jobs, size_t njobs, int precision, double mur,
                                 size_t max_batch) {
    if (!out || !jobs || njobs == 0) return tags_fail(TAGS_E_ARG, "tags_batch_create: invalid argument");
    if (precision != TAGS_PLAIN_FP64 && precision != TAGS_MIXED)
        return tags_fail(TAGS_E_ARG, "tags_batch_create: unknown precision");
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        if (!j.electrodes || !j.nodes || j.ns == 0 || !j.s || !j.kappa || j.num_electrodes == 0 || j.num_nodes == 0)
            return tags_fail(TAGS_E_ARG, "tags_batch_create: invalid job");
        if (!j.ie && j.inj_node >= j.num_nodes) return tags_fail(TAGS_E_ARG, "tags_batch_create: inj_node out of range");
    }
    *out = nullptr;
    DeviceCtx* ctx = tags_ctx();
    if (!ctx) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    tags_batch_s* b = new tags_batch_s();
    b->device = ctx->device;
    b->precision = precision;
    b->mur = mur;
    b->grids.resize(njobs);
    int err = 0;
#define BATCH_CHECK(expr)                                            \
    do {                                                             \
        cudaError_t _e = (expr);                                     \
        if (_e != cudaSuccess) {                                     \
            err = tags_fail_cuda(_e, #expr, __FILE__, __LINE__);     \
            batch_free(b);                                           \
            return err;                                              \
        }                                                            \
    } while (0)
    BATCH_CHECK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->events.resize(njobs + 1, nullptr);
    for (auto& e : b->events) BATCH_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // memory admission: samples resident per grid (at most max_batch, or 256),
    // halving the largest consumer until all plans fit in 60 % of free memory
    size_t freeb = 0;
    BATCH_CHECK(tags_free_memory(&freeb));
    double io = 0.0;
    std::vector<double> per(njobs);
    std::vector<long long> res(njobs);
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        const double N = (double)j.num_nodes + 2.0 * j.num_electrodes;
        io += (double)j.ns * (16.0 * (N + 2.0 + (j.ie ? (double)j.num_nodes : 0.0)) + 4.0);
        per[q] = bytes_per_sample((int)j.num_electrodes, (int)j.num_nodes, precision);
        res[q] = (long long)std::min<size_t>(j.ns, max_batch ? max_batch : 256);
    }
    const double budget = 0.6 * (double)freeb - io;
    for (;;) {
        double tot = 0.0;
        size_t worst = 0;
        for (size_t q = 0; q < njobs; ++q) {
            tot += per[q] * res[q];
            if (per[q] * res[q] > per[worst] * res[worst]) worst = q;
        }
        if (tot <= budget) break;
        if (res[worst] <= 1) {
            batch_free(b);
            return tags_fail(TAGS_E_NOMEM, "tags_batch_create: the grids do not fit in device memory");
        }
        res[worst] = (res[worst] + 1) / 2;
    }
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        GridSlot& g = b->grids[q];
        tags_plan p = nullptr;
        err = tags_plan_create(&p, j.electrodes, j.images, j.num_electrodes, j.nodes, j.num_nodes, precision,
                               (size_t)res[q]);
        if (err) {
            batch_free(b);
            return err;
        }
        g.plan = p;
        g.ns = (int)j.ns;
        g.n = (int)j.num_nodes;
        g.m = (int)j.num_electrodes;
        g.N = p->N;
        g.per_pass = p->batch;
        g.passes = (g.ns + g.per_pass - 1) / g.per_pass;
        g.has_ie = j.ie != nullptr;
        g.inj = j.inj_node;
        BATCH_CHECK(cudaMalloc(&g.d_s, sizeof(double2) * g.ns));
        BATCH_CHECK(cudaMalloc(&g.d_k, sizeof(double2) * g.ns));
        if (g.has_ie) BATCH_CHECK(cudaMalloc(&g.d_ie, sizeof(double2) * (size_t)g.ns * g.n));
        BATCH_CHECK(cudaMalloc(&g.d_sol, sizeof(double2) * (size_t)g.ns * g.N));
        BATCH_CHECK(cudaMalloc(&g.d_info, sizeof(int) * g.ns));
        if (precision != TAGS_PLAIN_FP64) {
            BATCH_CHECK(cudaMalloc(&g.d_snap_i, sizeof(int) * (size_t)g.passes * (3 * p->batch + 2)));
            BATCH_CHECK(cudaMalloc(&g.d_snap_d, sizeof(double) * (size_t)g.passes * 3 * p->batch));
            BATCH_CHECK(cudaMalloc(&g.d_snap_err, sizeof(int) * 2 * g.passes));
        }
    }
#undef BATCH_CHECK
    err = capture_batch(b);
    if (err) {
        batch_free(b);
        return err;
    }
    *out = b;
    return 0;
}

extern "C" int tags_batch_run(tags_batch batch, const tags_grid_job* jobs, size_t njobs, tags_run_stats* stats) {
    TagsRange range("tags grid batch");
    tags_batch_s* b = batch;
    if (!b || !jobs || njobs != b->grids.size()) return tags_fail(TAGS_E_ARG, "tags_batch_run: invalid argument");
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        const GridSlot& g = b->grids[q];
        if ((int)j.ns != g.ns || (int)j.num_nodes != g.n || (int)j.num_electrodes != g.m || !j.s || !j.kappa ||
            (j.ie != nullptr) != (g.has_ie != 0) || (!j.ie && j.inj_node != g.inj))
            return tags_fail(TAGS_E_ARG, "tags_batch_run: a job differs from the one the batch was built for");
    }
    TAGS_CUDA_OK(cudaSetDevice(b->device));
    cudaStream_t s0 = b->stream;
    for (size_t q = 0; q < njobs; ++q)
        if (!tags_all_finite(jobs[q].s, jobs[q].ns) || !tags_all_finite(jobs[q].kappa, jobs[q].ns))
            return tags_fail(TAGS_E_NONFINITE, "tags_batch_run: a job's s or kappa is not finite");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TAGS_CUDA_OK(cudaEventCreate(&e0));
    TAGS_CUDA_OK(cudaEventCreate(&e1));
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        GridSlot& g = b->grids[q];
        TAGS_CUDA_OK(cudaMemsetAsync(g.plan->d_status, 0, sizeof(int) * 4, s0));
        TAGS_CUDA_OK(cudaMemcpyAsync(g.d_s, j.s, sizeof(double2) * g.ns, cudaMemcpyHostToDevice, s0));
        TAGS_CUDA_OK(cudaMemcpyAsync(g.d_k, j.kappa, sizeof(double2) * g.ns, cudaMemcpyHostToDevice, s0));
        if (g.has_ie)
            TAGS_CUDA_OK(cudaMemcpyAsync(g.d_ie, j.ie, sizeof(double2) * (size_t)g.ns * g.n, cudaMemcpyHostToDevice, s0));
    }
    TAGS_CUDA_OK(cudaEventRecord(e0, s0));
    TAGS_CUDA_OK(cudaGraphLaunch(b->exec, s0));
    TAGS_CUDA_OK(cudaEventRecord(e1, s0));
    TAGS_CUDA_OK(cudaStreamSynchronize(s0));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tags_run_stats acc{};
    acc.seconds = 1e-3 * ms;
    acc.split = b->precision == TAGS_PLAIN_FP64 ? 0 : TAGS_SPLIT_F16;
    long long launched = b->launches_fixed;
    int first_err = 0, all_status = 0;
    for (size_t q = 0; q < njobs; ++q) {
        const tags_grid_job& j = jobs[q];
        GridSlot& g = b->grids[q];
        tags_plan_s* p = g.plan;
        // the fill's status word: a degenerate pair or a rejected sample
        // fails the run (no FP64 re-solves for that grid)
        int gst = 0;
        TAGS_CUDA_OK(cudaMemcpy(&gst, p->d_status, sizeof(int), cudaMemcpyDeviceToHost));
        all_status |= gst;
        if (b->precision != TAGS_PLAIN_FP64 && !gst) {
            const int bc = p->batch;
            std::vector<int> si((size_t)g.passes * (3 * bc + 2)), se(2 * (size_t)g.passes);
            std::vector<double> sd((size_t)g.passes * 3 * bc);
            TAGS_CUDA_OK(cudaMemcpy(si.data(), g.d_snap_i, sizeof(int) * si.size(), cudaMemcpyDeviceToHost));
            TAGS_CUDA_OK(cudaMemcpy(sd.data(), g.d_snap_d, sizeof(double) * sd.size(), cudaMemcpyDeviceToHost));
            TAGS_CUDA_OK(cudaMemcpy(se.data(), g.d_snap_err, sizeof(int) * se.size(), cudaMemcpyDeviceToHost));
            for (int pass = 0; pass < g.passes; ++pass) {
                const int k0 = pass * g.per_pass, nb = std::min(g.per_pass, g.ns - k0);
                const int* pi = si.data() + (size_t)pass * (3 * bc + 2);
                const double* pd = sd.data() + (size_t)pass * 3 * bc;
                launched += (long long)pi[3 * bc] * b->launches_step;
                if (se[2 * pass + 1] && !se[2 * pass]) {
                    // an fp16 split value left its range: this grid's plan re-solves
                    // the pass through its own run path (three bf16 pieces from then on)
                    auto cz = [](const double2* v) { return reinterpret_cast<const tags_cdouble*>(v); };
                    tags_run_stats rs{};
                    int e = tags_plan_run(p, cz(g.d_s + k0), cz(g.d_k + k0), b->mur, nb,
                                          g.has_ie ? cz(g.d_ie + (size_t)k0 * g.n) : nullptr, g.inj,
                                          reinterpret_cast<tags_cdouble*>(g.d_sol + (size_t)k0 * g.N), g.d_info + k0,
                                          TAGS_RUN_DEVICE_PTRS, &rs);
                    if (e) return e;
                    acc.max_iterations = std::max(acc.max_iterations, rs.max_iterations);
                    acc.max_backward_error = std::max(acc.max_backward_error, rs.max_backward_error);
                    acc.fallbacks += rs.fallbacks;
                    continue;
                }
                for (int s = 0; s < nb; ++s) {
                    acc.max_iterations = std::max(acc.max_iterations, pi[2 * bc + s]);
                    acc.max_backward_error = std::max(acc.max_backward_error, pd[2 * bc + s]);
                    if (pi[bc + s] && !se[2 * pass]) continue;
                    // not converged, or the pass's tensor-core factorisation
                    // reported an error: plain FP64 re-solve of this sample
                    acc.fallbacks++;
                    const int k = k0 + s;
                    int e = tags_mixed_fallback_one(p, g.d_s + k, g.d_k + k, b->mur,
                                                    g.has_ie ? g.d_ie + (size_t)k * g.n : nullptr, (int)g.inj,
                                                    g.d_sol + (size_t)k * g.N, g.d_info + k, p->stream);
                    if (e) return e;
                }
            }
            TAGS_CUDA_OK(cudaStreamSynchronize(p->stream));
        }
        if (j.sol)
            TAGS_CUDA_OK(cudaMemcpy(j.sol, g.d_sol, sizeof(double2) * (size_t)g.ns * g.N, cudaMemcpyDeviceToHost));
        if (j.info) {
            TAGS_CUDA_OK(cudaMemcpy(j.info, g.d_info, sizeof(int) * g.ns, cudaMemcpyDeviceToHost));
            for (int s = 0; s < g.ns && !first_err; ++s)
                if (j.info[s] < 0) first_err = j.info[s];
        }
    }
    tags_note_launch(launched);
    if (stats) *stats = acc;
    if (all_status & TAGS_ST_DEGENERATE_PAIR)
        return tags_fail(TAGS_E_GEOMETRY, "coincident or overlapping segments: the pair integral diverges");
    if (all_status & TAGS_ST_NONFINITE) return tags_fail(TAGS_E_NONFINITE, "non-finite value in the impedance fill");
    if (all_status & TAGS_ST_BAD_ARG)
        return tags_fail(TAGS_E_ARG, "a sample's propagation constant is outside the supported range (|gamma| > 1e5 / m)");
    return first_err;
}

extern "C" int tags_batch_destroy(tags_batch batch) {
    batch_free(batch);
    return 0;
}
