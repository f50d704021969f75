// Batched plan API (include/tags_gpu.h, part 2): geometry, incidence and
// workspaces stay on the device; every pass handles `batch` Laplace samples:
//   plain FP64: W_G assembled in place (incidence + fused direct/image fill,
//               both triangles), LU with partial pivoting, triangular solves;
//   mixed:      see mixed.cu.
// The per-sample medium terms follow examples/three_grids.c:326-333
// (gamma = sqrt(s mur mu0 kappa), ref_t = (kappa - s eps0)/(kappa + s eps0),
// ref_l = 1) and the right-hand side is [I_E; 0; 0] (src/linalg.h:61-68).
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

// principal square root of a complex number
TAGS_D double2 csqrt_d(double2 z) {
    double a = hypot(z.x, z.y);
    if (a == 0.0) return make_double2(0.0, 0.0);
    double re = sqrt(0.5 * (a + fabs(z.x)));
    double im = 0.5 * z.y / re;
    if (z.x >= 0.0) return make_double2(re, im);
    return make_double2(fabs(im), z.y >= 0.0 ? re : -re);
}

// |gamma| above this (1/m) is outside any soil and frequency the model serves;
// the quadrature orders derived from |gamma| L stay far from integer range.
constexpr double GAMMA_MAX = 1e5;

__global__ void k_coef(const double2* __restrict__ s, const double2* __restrict__ kappa, double mur, int nb,
                       SampleCoef* __restrict__ coef, int* __restrict__ status) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nb) return;
    double2 sk = s[k], kp = kappa[k];
    double2 smu = cscale(sk, mur * TAGS_MU0);
    double2 gamma = csqrt_d(cmul(smu, kp));
    double2 se = cscale(sk, TAGS_EPS0);
    double2 ref_t = cdiv(csub(kp, se), cadd(kp, se));
    double2 cL = cscale(smu, 1.0 / TAGS_FOUR_PI);
    double2 cT = cdiv(make_double2(1.0, 0.0), cscale(kp, TAGS_FOUR_PI));
    SampleCoef c;
    c.gamma = gamma;
    c.cL = cL;
    c.cT = cT;
    c.cLi = cL;                 // ref_l = 1
    c.cTi = cmul(ref_t, cT);
    const bool finite = isfinite(c.gamma.x) && isfinite(c.gamma.y) && isfinite(c.cL.x) && isfinite(c.cL.y) &&
                        isfinite(c.cT.x) && isfinite(c.cT.y) && isfinite(c.cTi.x) && isfinite(c.cTi.y);
    if (!finite || !(cabs2(c.gamma) <= GAMMA_MAX * GAMMA_MAX)) {
        // the run reports the sample (non-finite, or out of range); the
        // kernels that follow see finite, small coefficients
        atomicOr(status, finite ? TAGS_ST_BAD_ARG : TAGS_ST_NONFINITE);
        c.gamma = make_double2(1e-3, 0.0);
        c.cL = c.cT = c.cLi = c.cTi = make_double2(1.0, 0.0);
    }
    coef[k] = c;
}

// X (batch x N, sample-major): [ie; 0; 0] or a unit current at inj_node.
__global__ void k_rhs(double2* __restrict__ X, int N, int n, const double2* __restrict__ ie, int inj_node) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (r >= N) return;
    double2 v = make_double2(0.0, 0.0);
    if (r < n) {
        if (ie) v = ie[(long long)b * n + r];
        else if (r == inj_node) v = make_double2(1.0, 0.0);
    }
    X[(long long)b * N + r] = v;
}

}  // namespace

int tags_plan_coef(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur, int nb, cudaStream_t st) {
    k_coef<<<(nb + 127) / 128, 128, 0, st>>>(d_s, d_kappa, mur, nb, p->d_coef, p->d_status);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_plan_rhs(tags_plan_s* p, double2* d_X, const double2* d_ie, int inj_node, int nb, cudaStream_t st) {
    k_rhs<<<dim3((p->N + 255) / 256, nb), 256, 0, st>>>(d_X, p->N, p->n, d_ie, inj_node);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

static int build_incidence(tags_plan_s* p, cudaStream_t st) {
    const int m = p->m, n = p->n;
    std::vector<signed char> cond((size_t)n * m);
    int err = tags_incidence_codes(p->d_elec, m, reinterpret_cast<const double*>(p->d_W), n, p->d_cond, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaMemcpyAsync(cond.data(), p->d_cond, cond.size(), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    std::vector<int> nptr(n + 1, 0), sptr(m + 1, 0), nseg, snode;
    std::vector<signed char> na, sa;
    long long suma = 0, nb = 0;
    for (int nd = 0; nd < n; ++nd) {
        bool any = false;
        for (int e = 0; e < m; ++e) {
            int c = cond[(size_t)nd * m + e];
            if (!c) continue;
            any = true;
            nseg.push_back(e);
            na.push_back(c == 1 ? 1 : -1);
            suma += c == 1 ? 1 : -1;
            ++nb;
            sptr[e + 1]++;
        }
        nptr[nd + 1] = (int)nseg.size();
        if (!any) {
            char msg[96];
            snprintf(msg, sizeof(msg), "No electrode is connected to node[%i]", nd);
            return tags_fail(TAGS_E_ARG, msg);
        }
    }
    if (suma != 0 || nb != 2LL * m) return tags_fail(TAGS_E_ARG, "incidence checksum failed (sum(A) != 0 or sum(B) != m)");
    for (int e = 0; e < m; ++e) sptr[e + 1] += sptr[e];
    snode.resize(nseg.size());
    sa.resize(nseg.size());
    std::vector<int> fillp(sptr.begin(), sptr.end() - 1);
    for (int nd = 0; nd < n; ++nd)
        for (int q = nptr[nd]; q < nptr[nd + 1]; ++q) {
            int e = nseg[q];
            snode[fillp[e]] = nd;
            sa[fillp[e]] = na[q];
            fillp[e]++;
        }
    Incidence& I = p->inc;
    I.nnz = (int)nseg.size();
    size_t nnz = std::max<size_t>(1, nseg.size());
    TAGS_CUDA_OK(cudaMalloc(&I.node_ptr, sizeof(int) * (n + 1)));
    TAGS_CUDA_OK(cudaMalloc(&I.node_seg, sizeof(int) * nnz));
    TAGS_CUDA_OK(cudaMalloc(&I.node_a, nnz));
    TAGS_CUDA_OK(cudaMalloc(&I.seg_ptr, sizeof(int) * (m + 1)));
    TAGS_CUDA_OK(cudaMalloc(&I.seg_node, sizeof(int) * nnz));
    TAGS_CUDA_OK(cudaMalloc(&I.seg_a, nnz));
    TAGS_CUDA_OK(cudaMemcpy(I.node_ptr, nptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
    TAGS_CUDA_OK(cudaMemcpy(I.seg_ptr, sptr.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice));
    if (!nseg.empty()) {
        TAGS_CUDA_OK(cudaMemcpy(I.node_seg, nseg.data(), sizeof(int) * nseg.size(), cudaMemcpyHostToDevice));
        TAGS_CUDA_OK(cudaMemcpy(I.node_a, na.data(), na.size(), cudaMemcpyHostToDevice));
        TAGS_CUDA_OK(cudaMemcpy(I.seg_node, snode.data(), sizeof(int) * snode.size(), cudaMemcpyHostToDevice));
        TAGS_CUDA_OK(cudaMemcpy(I.seg_a, sa.data(), sa.size(), cudaMemcpyHostToDevice));
    }
    return 0;
}

static void plan_free(tags_plan_s* p) {
    if (!p) return;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    void* ptrs[] = {p->d_elec, p->d_img, p->d_cond, p->d_coef, p->d_status, p->d_info, p->d_ipiv, p->d_W, p->d_x,
                    p->inc.node_ptr, p->inc.node_seg, p->inc.node_a, p->inc.seg_ptr, p->inc.seg_node, p->inc.seg_a};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    tags_mixed_free(p);
    tags_plan_drop_graphs(p);
    if (p->d_sin) cudaFree(p->d_sin);
    if (p->d_stage) cudaFree(p->d_stage);
    if (p->d_fbW) cudaFree(p->d_fbW);
    if (p->d_fbpiv) cudaFree(p->d_fbpiv);
    if (p->d_pot) cudaFree(p->d_pot);
    if (p->d_coef1) cudaFree(p->d_coef1);
    if (p->d_iein) cudaFree(p->d_iein);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    tags_plan_s* tw = p->twin;
    delete p;
    plan_free(tw);
}

extern "C" int tags_plan_create(tags_plan* out, const Electrode* electrodes, const Electrode* images,
                                size_t num_electrodes, const double* nodes, size_t num_nodes, int precision,
                                size_t max_batch) {
    if (!out || !electrodes || !nodes || num_electrodes == 0 || num_nodes == 0)
        return tags_fail(TAGS_E_ARG, "tags_plan_create: invalid argument");
    if (precision != TAGS_PLAIN_FP64 && precision != TAGS_MIXED)
        return tags_fail(TAGS_E_ARG, "tags_plan_create: unknown precision");
    const long long N = (long long)num_nodes + 2LL * (long long)num_electrodes;
    if (N > 60000) return tags_fail(TAGS_E_ARG, "tags_plan_create: system larger than 60000 unknowns");
    *out = nullptr;
    DeviceCtx* ctx = tags_ctx();
    if (!ctx) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    tags_plan_s* p = new tags_plan_s();
    p->device = ctx->device;
    {
        const double* e = reinterpret_cast<const double*>(electrodes);
        p->h_elec.assign(e, e + 11 * num_electrodes);
        if (images) {
            const double* im = reinterpret_cast<const double*>(images);
            p->h_img.assign(im, im + 11 * num_electrodes);
        }
        p->h_nodes.assign(nodes, nodes + 3 * num_nodes);
    }
    p->precision = precision;
    p->m = (int)num_electrodes;
    p->n = (int)num_nodes;
    p->N = (int)N;
    p->has_images = images != nullptr;
    int err = 0;
#define PLAN_CHECK(expr)                      \
    do {                                      \
        cudaError_t _e = (expr);              \
        if (_e != cudaSuccess) {              \
            err = tags_fail_cuda(_e, #expr, __FILE__, __LINE__); \
            plan_free(p);                     \
            return err;                       \
        }                                     \
    } while (0)
    PLAN_CHECK(cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking));
    PLAN_CHECK(cudaEventCreate(&p->ev0));
    PLAN_CHECK(cudaEventCreate(&p->ev1));
    const size_t eb = sizeof(Electrode) * num_electrodes;
    PLAN_CHECK(cudaMalloc(&p->d_elec, eb));
    PLAN_CHECK(cudaMalloc(&p->d_img, eb));
    PLAN_CHECK(cudaMemcpy(p->d_elec, electrodes, eb, cudaMemcpyHostToDevice));
    PLAN_CHECK(cudaMemcpy(p->d_img, images ? (const void*)images : (const void*)electrodes, eb, cudaMemcpyHostToDevice));
    PLAN_CHECK(cudaMalloc(&p->d_cond, (size_t)p->n * p->m));
    PLAN_CHECK(cudaMalloc(&p->d_status, sizeof(int) * 4));
    // nodes go through a temporary buffer (d_W is reused as staging here)
    PLAN_CHECK(cudaMalloc(&p->d_W, sizeof(double) * 3 * num_nodes));
    PLAN_CHECK(cudaMemcpy(p->d_W, nodes, sizeof(double) * 3 * num_nodes, cudaMemcpyHostToDevice));
    err = build_incidence(p, p->stream);
    cudaFree(p->d_W);
    p->d_W = nullptr;
    if (err) { plan_free(p); return err; }
    // batch size from free device memory
    size_t freeb = 0;
    PLAN_CHECK(tags_free_memory(&freeb));
    const double NN = (double)N * (double)N;
    double per = precision == TAGS_PLAIN_FP64
                     ? 16.0 * NN + 40.0 * N
                     : 8.0 * NN + 32.0 * (double)p->m * p->m + 80.0 * N + (double)tags_ldl_tc_workspace((int)N, 1);
    long long cap = (long long)(0.45 * (double)freeb / per);
    long long b = max_batch ? (long long)max_batch : std::min<long long>(cap, 64);
    if (b > cap) b = cap;
    if (b < 1) { plan_free(p); return tags_fail(TAGS_E_NOMEM, "not enough device memory for one sample"); }
    p->batch = (int)b;
    PLAN_CHECK(cudaMalloc(&p->d_coef, sizeof(SampleCoef) * b));
    PLAN_CHECK(cudaMalloc(&p->d_info, sizeof(int) * b));
    PLAN_CHECK(cudaMalloc(&p->d_x, sizeof(double2) * N * b));
    PLAN_CHECK(cudaMalloc(&p->d_sin, sizeof(double2) * 2 * b));
    if (precision == TAGS_PLAIN_FP64) {
        PLAN_CHECK(cudaMalloc(&p->d_ipiv, sizeof(int) * N * b));
        PLAN_CHECK(cudaMalloc(&p->d_W, sizeof(double2) * (size_t)NN * b));
        err = tags_lu_prepare();
        if (err) { plan_free(p); return err; }
    } else {
        err = tags_mixed_alloc(p);
        if (err) { plan_free(p); return err; }
    }
#undef PLAN_CHECK
    *out = p;
    return 0;
}

extern "C" int tags_plan_destroy(tags_plan plan) {
    plan_free(plan);
    return 0;
}

int tags_plan_fill_fp64(tags_plan_s* p, const SampleCoef* d_coef, int nb, const FillOut& out, cudaStream_t st) {
    if (p->fill_model == TAGS_INTG_MHEM)
        return tags_launch_mhem_fp64(p->d_elec, p->d_img, p->m, p->has_images, p->d_pot, d_coef, nb, out, p->d_status,
                                     st);
    return tags_launch_fill_fp64(p->d_elec, p->d_img, p->m, d_coef, nb, out,
                                 p->has_images ? TAGS_FILL_BOTH : TAGS_FILL_DIRECT, TAGS_INTG_DOUBLE, 1, p->d_status, st);
}

extern "C" int tags_plan_set_fill(tags_plan plan, int integration_type) {
    tags_plan_s* p = plan;
    if (!p) return tags_fail(TAGS_E_ARG, "tags_plan_set_fill: invalid plan");
    if (integration_type != TAGS_INTG_DOUBLE && integration_type != TAGS_INTG_MHEM)
        return tags_fail(TAGS_E_ARG, "tags_plan_set_fill: INTG_DOUBLE (2) or INTG_MHEM (4)");
    if (integration_type == p->fill_model) return 0;
    TAGS_CUDA_OK(cudaSetDevice(p->device));
    if (integration_type == TAGS_INTG_MHEM && !p->d_pot) {
        // the static potentials, once per geometry
        TAGS_CUDA_OK(cudaMalloc(&p->d_pot, sizeof(double2) * 4 * (size_t)p->m * p->m));
        TAGS_CUDA_OK(cudaMalloc(&p->d_coef1, sizeof(SampleCoef)));
        int err = tags_launch_mhem_potentials(p->d_elec, p->d_img, p->m, p->has_images, p->d_pot, p->d_coef1,
                                              p->d_status, p->stream);
        if (err) return err;
        TAGS_CUDA_OK(cudaStreamSynchronize(p->stream));
    }
    p->fill_model = integration_type;
    tags_plan_drop_graphs(p);
    return 0;
}

// Plain FP64 pass over nb samples whose coefficients and right-hand sides are
// already in p->d_coef and p->d_x.
int tags_plan_run_plain(tags_plan_s* p, const double2*, int nb, cudaStream_t st) {
    const long long N = p->N, NN = N * N;
    TagsRange range("tags assemble");
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_W, 0, sizeof(double2) * NN * nb, st));
    int err = tags_wg_incidence(p->d_W, N, NN, nb, p->d_cond, p->n, p->m, st);
    if (err) return err;
    FillOut out{};
    out.zl = p->d_W;
    out.zt = p->d_W;
    out.ld = N;
    out.batch_stride = NN;
    out.row0_l = out.col0_l = p->n;
    out.row0_t = out.col0_t = p->n + p->m;
    out.sign = -1.0;
    out.mirror = 1;
    out.accumulate = 0;
    range.next("tags fill");
    err = tags_plan_fill_fp64(p, p->d_coef, nb, out, st);
    if (err) return err;
    range.next("tags factor");
    err = tags_lu_z(p->d_W, (int)N, N, NN, nb, 1, p->d_ipiv, p->d_info, st);
    if (err) return err;
    range.next("tags solve");
    return tags_lu_solve_z(p->d_W, (int)N, N, NN, nb, p->d_ipiv, p->d_x, 1, N, N, st);
}

// ---- graph passes ------------------------------------------------------------------

// Add a while-node after the work captured so far on `st`; its body graph is
// returned for a separate capture, its condition starts at 1 on every launch.
int tags_plan_add_while_node(cudaStream_t st, cudaGraphConditionalHandle* cond, cudaGraph_t* body) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    const cudaGraphNode_t* deps_rt = nullptr;
    size_t ndeps = 0;
    TAGS_CUDA_OK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps_rt, nullptr, &ndeps));
    if (cs != cudaStreamCaptureStatusActive) return tags_fail(TAGS_E_CUDA, "stream is not capturing");
    std::vector<cudaGraphNode_t> deps(deps_rt, deps_rt + ndeps);
    TAGS_CUDA_OK(cudaGraphConditionalHandleCreate(cond, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = *cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    TAGS_CUDA_OK(cudaGraphAddNode(&node, g, deps.data(), nullptr, deps.size(), &cp));
    *body = cp.conditional.phGraph_out[0];
    TAGS_CUDA_OK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    return 0;
}

// Capture one pass of nb samples into an executable graph: sample
// coefficients and right-hand sides from the plan's staging buffers, then the
// plain FP64 fill + LU + solve, or the mixed factorisation, the refinement
// set-up and a while-node repeating the refinement step until the device
// clears the condition. Nothing runs during the capture.
static int capture_pass(tags_plan_s* p, int nb, double mur, int has_ie, int inj, tags_plan_s::GraphPass* gp) {
    TagsRange range("tags capture pass");
    cudaStream_t st = p->stream;
    const long long l0 = tags_thread_launch_count();
    TAGS_CUDA_OK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    int err = tags_plan_coef(p, p->d_sin, p->d_sin + p->batch, mur, nb, st);
    if (!err) err = tags_plan_rhs(p, p->d_x, has_ie ? p->d_iein : nullptr, inj, nb, st);
    cudaGraph_t body = nullptr;
    cudaGraphConditionalHandle cond = 0;
    if (!err) {
        if (p->precision == TAGS_PLAIN_FP64) {
            err = tags_plan_run_plain(p, nullptr, nb, st);
        } else {
            err = tags_mixed_factor(p, nb, st);
            if (!err) err = tags_mixed_ir_setup(p, nb, st);
            if (!err) err = tags_plan_add_while_node(st, &cond, &body);
        }
    }
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (!err && ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaStreamEndCapture", __FILE__, __LINE__);
    const long long l1 = tags_thread_launch_count();
    if (!err && body) {
        ce = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (ce != cudaSuccess) {
            err = tags_fail_cuda(ce, "cudaStreamBeginCaptureToGraph", __FILE__, __LINE__);
        } else {
            err = tags_mixed_ir_step(p, nb, st, cond, 1);
            cudaGraph_t b2 = nullptr;
            ce = cudaStreamEndCapture(st, &b2);
            if (!err && ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaStreamEndCapture (body)", __FILE__, __LINE__);
        }
    }
    const long long l2 = tags_thread_launch_count();
    tags_note_launch(-(l2 - l0));      // captured, not launched
    if (!err) {
        ce = cudaGraphInstantiate(&gp->exec, g, 0);
        if (ce != cudaSuccess) err = tags_fail_cuda(ce, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    if (g) cudaGraphDestroy(g);
    if (err) {
        cudaGetLastError();
        gp->exec = nullptr;
        return err;
    }
    gp->nb = nb;
    gp->mur = mur;
    gp->has_ie = has_ie;
    gp->inj = inj;
    gp->launches_fixed = l1 - l0;
    gp->launches_step = l2 - l1;
    return 0;
}

static tags_plan_s::GraphPass* graph_for(tags_plan_s* p, int nb, double mur, int has_ie, int inj, int* err) {
    *err = 0;
    for (auto& g : p->graphs)
        if (g.nb == nb && g.mur == mur && g.has_ie == has_ie && (has_ie || g.inj == inj)) return &g;
    tags_plan_s::GraphPass gp;
    *err = capture_pass(p, nb, mur, has_ie, has_ie ? 0 : inj, &gp);
    if (*err) return nullptr;
    if (p->graphs.size() >= 8) {        // a few pass shapes per plan: drop the oldest
        cudaGraphExecDestroy(p->graphs.front().exec);
        p->graphs.erase(p->graphs.begin());
    }
    p->graphs.push_back(gp);
    return &p->graphs.back();
}

void tags_plan_drop_graphs(tags_plan_s* p) {
    for (auto& g : p->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    p->graphs.clear();
}

extern "C" int tags_plan_set_panels(tags_plan plan, int panels) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_panels: invalid plan");
    if (panels < 0 || panels > 6) return tags_fail(TAGS_E_ARG, "tags_plan_set_panels: panels must be 0 .. 6");
    const int v = panels == 0 ? 6 : panels;
    if (plan->group_panels != v) {
        plan->group_panels = v;
        tags_plan_drop_graphs(plan);
    }
    return 0;
}

extern "C" int tags_plan_set_split(tags_plan plan, int pieces) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_split: invalid plan");
    if (pieces != 2 && pieces != 3 && pieces != TAGS_SPLIT_F16)
        return tags_fail(TAGS_E_ARG, "tags_plan_set_split: pieces must be 2, 3 or 16");
    if (plan->split_pieces != pieces) {
        plan->split_pieces = pieces;
        tags_plan_drop_graphs(plan);
    }
    return 0;
}

extern "C" int tags_plan_set_refine_tol(tags_plan plan, double tol) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_refine_tol: invalid plan");
    if (!(tol >= 0.0) || tol > 1e-3) return tags_fail(TAGS_E_ARG, "tags_plan_set_refine_tol: tol must be 0 .. 1e-3");
    const double v = tol == 0.0 ? 1e-9 : tol;
    if (plan->ir_tol != v) {
        plan->ir_tol = v;
        tags_plan_drop_graphs(plan);     // the tolerance is an argument of the captured refinement kernels
    }
    return 0;
}

extern "C" int tags_plan_set_tc_pairs(tags_plan plan, int on) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_tc_pairs: invalid plan");
    if (on < 0 || on > 2) return tags_fail(TAGS_E_ARG, "tags_plan_set_tc_pairs: 0, 1 or 2");
    const int v = on;
    if (plan->tc_pairs != v) {
        plan->tc_pairs = v;
        tags_plan_drop_graphs(plan);
    }
    return 0;
}

extern "C" int tags_plan_set_max_steps(tags_plan plan, int steps) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_max_steps: invalid plan");
    if (steps < 0 || steps > 40) return tags_fail(TAGS_E_ARG, "tags_plan_set_max_steps: steps must be 0 .. 40");
    const int v = steps == 0 ? 40 : steps;
    if (plan->max_steps != v) {
        plan->max_steps = v;
        tags_plan_drop_graphs(plan);     // the step cap is an argument of the captured decision kernel
    }
    return 0;
}

// forward declaration: the tuner times the public run path
extern "C" int tags_plan_run(tags_plan plan, const tags_cdouble* s, const tags_cdouble* kappa, double mur, size_t ns,
                             const tags_cdouble* ie, size_t inj_node, tags_cdouble* sol, int* info, int flags,
                             tags_run_stats* stats);

// ---- autotuner cache ---------------------------------------------------------------
// A text file, one line per timed tune:
//   tags-tune 1 N=.. m=.. prec=.. fill=.. cap=.. pipes=.. pairs=.. gpu=<name>/<SMs>/sm<cc> | <pass> <panels> <split> <rate>
// The key holds what the candidates' timings depend on: the system's size, the
// precision and impedance model, the samples the tuner may put in one pass,
// the pipelines and pair setting, and the GPU. A lookup takes the last line
// with the plan's key; a line is appended by one write to a file opened for
// appending, so processes may share the file.
static std::mutex g_tune_mutex;
static std::string g_tune_path;

extern "C" int tags_gpu_set_tune_cache(const char* path) {
    std::lock_guard<std::mutex> lk(g_tune_mutex);
    if (!path || !*path) {
        g_tune_path.clear();
        return 0;
    }
    FILE* f = fopen(path, "a");
    if (!f) return tags_fail(TAGS_E_ARG, "tags_gpu_set_tune_cache: the file cannot be opened for appending");
    fclose(f);
    g_tune_path = path;
    return 0;
}

static std::string tune_key(const tags_plan_s* p, int cap) {
    std::string gpu = "unknown";
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, p->device) == cudaSuccess) {
        gpu = prop.name;
        for (char& ch : gpu)
            if (ch == ' ' || ch == '|' || ch == '\t' || ch == '\n' || ch == '\r') ch = '_';
        gpu += "/" + std::to_string(prop.multiProcessorCount) + "/sm" + std::to_string(prop.major * 10 + prop.minor);
    } else {
        cudaGetLastError();
    }
    char buf[160];
    snprintf(buf, sizeof buf, "tags-tune 1 N=%d m=%d prec=%d fill=%d cap=%d pipes=%d pairs=%d gpu=", p->N, p->m,
             p->precision, p->fill_model, cap, p->pipelines, p->tc_pairs);
    return std::string(buf) + gpu;
}

// The last entry for `key` that is valid for this plan, if any.
static bool tune_lookup(const std::string& path, const std::string& key, const tags_plan_s* p, int cap,
                        tags_tune_result* r) {
    FILE* f = fopen(path.c_str(), "r");
    if (!f) return false;
    const bool mixed = p->precision != TAGS_PLAIN_FP64;
    char line[1024];
    bool hit = false;
    while (fgets(line, sizeof line, f)) {
        const char* bar = strstr(line, " | ");
        if (!bar || (size_t)(bar - line) != key.size() || strncmp(line, key.c_str(), key.size()) != 0) continue;
        tags_tune_result t{};
        if (sscanf(bar + 3, "%d %d %d %lf", &t.samples_per_pass, &t.panels_per_update, &t.split,
                   &t.solves_per_second) != 4)
            continue;
        const int g = t.panels_per_update;
        const bool ok = t.samples_per_pass >= 1 && t.samples_per_pass <= cap &&
                        (mixed ? (g == 1 || g == 2 || g == 4 || g == 6) && (t.split == TAGS_SPLIT_F16 || t.split == 3)
                               : g == 0 && t.split == 0);
        if (ok) {
            *r = t;
            hit = true;
        }
    }
    fclose(f);
    return hit;
}

static void tune_store(const std::string& path, const std::string& key, const tags_tune_result& r) {
    FILE* f = fopen(path.c_str(), "a");
    if (!f) return;
    char line[1024];
    const int len = snprintf(line, sizeof line, "%s | %d %d %d %.6g\n", key.c_str(), r.samples_per_pass,
                             r.panels_per_update, r.split, r.solves_per_second);
    if (len > 0 && len < (int)sizeof line) fwrite(line, 1, (size_t)len, f);
    fclose(f);
}

extern "C" int tags_plan_tune(tags_plan plan, const tags_cdouble* s, const tags_cdouble* kappa, double mur, size_t ns,
                              size_t inj_node, int flags, tags_tune_result* out) {
    TagsRange range("tags tune");
    tags_plan_s* p = plan;
    if (!p || !s || !kappa || ns == 0) return tags_fail(TAGS_E_ARG, "tags_plan_tune: invalid argument");
    const int cap = (int)std::min<size_t>(p->batch, ns);
    const bool refresh = (flags & TAGS_TUNE_REFRESH) != 0;
    flags &= ~TAGS_TUNE_REFRESH;
    std::string cache;
    {
        std::lock_guard<std::mutex> lk(g_tune_mutex);
        cache = g_tune_path;
    }
    const std::string key = cache.empty() ? std::string() : tune_key(p, cap);
    if (!cache.empty() && !refresh) {
        tags_tune_result hit{};
        if (tune_lookup(cache, key, p, cap, &hit)) {
            p->pass_batch = hit.samples_per_pass;
            if (p->precision != TAGS_PLAIN_FP64) {
                p->group_panels = hit.panels_per_update;
                p->split_pieces = hit.split;
            }
            tags_plan_drop_graphs(p);
            hit.candidates = 0;                 // nothing timed
            if (out) *out = hit;
            return 0;
        }
    }
    std::vector<int> sizes;
    for (int b = 16; b < cap; b *= 2) sizes.push_back(b);
    sizes.push_back(cap);
    const bool mixed = p->precision != TAGS_PLAIN_FP64;
    const int groups[4] = {6, 4, 2, 1};
    const int splits[2] = {TAGS_SPLIT_F16, 3};
    tags_tune_result best{};
    best.solves_per_second = -1.0;
    const int saved_pass = p->pass_batch, saved_group = p->group_panels, saved_split = p->split_pieces;
    int count = 0;
    for (int b : sizes)
        for (int ip = 0; ip < (mixed ? 4 : 1); ++ip)
            for (int is = 0; is < (mixed ? 2 : 1); ++is) {
                p->pass_batch = b;
                if (mixed) {
                    p->group_panels = groups[ip];
                    p->split_pieces = splits[is];
                }
                tags_plan_drop_graphs(p);
                tags_run_stats st{};
                // the first pass captures the graph of this shape; the second is timed
                int rc = tags_plan_run(p, s, kappa, mur, (size_t)b, nullptr, inj_node, nullptr, nullptr, flags, &st);
                if (!rc) rc = tags_plan_run(p, s, kappa, mur, (size_t)b, nullptr, inj_node, nullptr, nullptr, flags, &st);
                if (rc) {
                    // a candidate that fails is skipped; the error stays in tags_gpu_last_error
                    cudaGetLastError();
                    continue;
                }
                ++count;
                const double rate = st.seconds > 0 ? b / st.seconds : 0.0;
                // the fp16 split may have fallen back to three pieces inside the run
                const int used_split = mixed ? st.split : 0;
                if (rate > best.solves_per_second) {
                    best.samples_per_pass = b;
                    best.panels_per_update = mixed ? p->group_panels : 0;
                    best.split = used_split;
                    best.solves_per_second = rate;
                }
            }
    if (best.solves_per_second < 0) {
        p->pass_batch = saved_pass;
        p->group_panels = saved_group;
        p->split_pieces = saved_split;
        tags_plan_drop_graphs(p);
        return tags_fail(TAGS_E_CUDA, "tags_plan_tune: no candidate ran");
    }
    p->pass_batch = best.samples_per_pass;
    if (mixed) {
        p->group_panels = best.panels_per_update;
        p->split_pieces = best.split;
    }
    tags_plan_drop_graphs(p);
    best.candidates = count;
    if (!cache.empty()) tune_store(cache, key, best);
    if (out) *out = best;
    return 0;
}

extern "C" int tags_plan_set_graphs(tags_plan plan, int enable) {
    if (!plan) return tags_fail(TAGS_E_ARG, "tags_plan_set_graphs: invalid plan");
    plan->use_graphs = enable ? 1 : 0;
    return 0;
}

// The passes of a run that plan p takes from the shared counter `next` (pass q
// covers samples q * per_pass onwards), on p's stream; per-sample statistics
// folded into *acc.
static int run_passes(tags_plan_s* p, const tags_cdouble* s, const tags_cdouble* kappa, double mur, size_t ns,
                      const tags_cdouble* ie, size_t inj_node, tags_cdouble* sol, int* info, int flags, size_t per_pass,
                      std::atomic<size_t>* next, tags_run_stats* acc) {
    cudaStream_t st = p->stream;
    const bool dev = (flags & TAGS_RUN_DEVICE_PTRS) != 0;
    const long long N = p->N;
    // staging for host inputs
    double2* d_in = nullptr;
    if (!dev && !p->use_graphs) {
        size_t need = sizeof(double2) * (2 * (size_t)p->batch + (ie ? (size_t)p->batch * p->n : 0));
        if (need > p->stage_bytes) {
            if (p->d_stage) cudaFree(p->d_stage);
            p->d_stage = nullptr;
            p->stage_bytes = 0;
            TAGS_CUDA_OK(cudaMalloc(&p->d_stage, need));
            p->stage_bytes = need;
        }
        d_in = p->d_stage;
    }
    // passes are taken in order from a counter shared with the other pipeline
    // (if any): a pipeline takes the next pass once its last one has finished
    for (size_t k0 = next->fetch_add(1) * per_pass; k0 < ns; k0 = next->fetch_add(1) * per_pass) {
        const int nb = (int)std::min<size_t>(per_pass, ns - k0);
        TagsRange range("tags pass");
        const double2 *ds, *dk, *die = nullptr;
        if (p->use_graphs) {
            // inputs go to the plan's staging buffers, which the graph reads
            const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
            TAGS_CUDA_OK(cudaMemcpyAsync(p->d_sin, s + k0, sizeof(double2) * nb, kind, st));
            TAGS_CUDA_OK(cudaMemcpyAsync(p->d_sin + p->batch, kappa + k0, sizeof(double2) * nb, kind, st));
            ds = p->d_sin;
            dk = p->d_sin + p->batch;
            if (ie) {
                if (!p->d_iein) TAGS_CUDA_OK(cudaMalloc(&p->d_iein, sizeof(double2) * p->batch * p->n));
                TAGS_CUDA_OK(cudaMemcpyAsync(p->d_iein, ie + k0 * p->n, sizeof(double2) * nb * p->n, kind, st));
                die = p->d_iein;
            }
        } else if (dev) {
            ds = reinterpret_cast<const double2*>(s) + k0;
            dk = reinterpret_cast<const double2*>(kappa) + k0;
            if (ie) die = reinterpret_cast<const double2*>(ie) + k0 * p->n;
        } else {
            TAGS_CUDA_OK(cudaMemcpyAsync(d_in, s + k0, sizeof(double2) * nb, cudaMemcpyHostToDevice, st));
            TAGS_CUDA_OK(cudaMemcpyAsync(d_in + p->batch, kappa + k0, sizeof(double2) * nb, cudaMemcpyHostToDevice, st));
            ds = d_in;
            dk = d_in + p->batch;
            if (ie) {
                TAGS_CUDA_OK(cudaMemcpyAsync(d_in + 2 * p->batch, ie + k0 * p->n, sizeof(double2) * nb * p->n,
                                             cudaMemcpyHostToDevice, st));
                die = d_in + 2 * p->batch;
            }
        }
        int err = 0;
        std::vector<int> iters(nb), conv(nb);
        std::vector<double> berr(nb);
        if (p->use_graphs) {
            tags_plan_s::GraphPass* gp = graph_for(p, nb, mur, die != nullptr, (int)inj_node, &err);
            if (err) return err;
            TAGS_CUDA_OK(cudaGraphLaunch(gp->exec, st));
            long long launched = gp->launches_fixed;
            if (p->precision != TAGS_PLAIN_FP64) {
                int steps = 0;
                err = tags_mixed_finish(p, nb, st, iters.data(), berr.data(), conv.data(), &steps);
                if (err) return err;
                launched += (long long)steps * gp->launches_step;
            }
            tags_note_launch(launched);
        } else {
            err = tags_plan_coef(p, ds, dk, mur, nb, st);
            if (!err) err = tags_plan_rhs(p, p->d_x, die, (int)inj_node, nb, st);
            if (err) return err;
            if (p->precision == TAGS_PLAIN_FP64) err = tags_plan_run_plain(p, ds, nb, st);
            else err = tags_mixed_solve_batch(p, nb, nullptr, iters.data(), berr.data(), conv.data(), st);
            if (err) return err;
        }
        if (p->precision != TAGS_PLAIN_FP64) {
            for (int q = 0; q < nb; ++q) {
                acc->max_iterations = std::max(acc->max_iterations, iters[q]);
                acc->max_backward_error = std::max(acc->max_backward_error, berr[q]);
                if (!conv[q]) acc->fallbacks++;
            }
        }
        if (sol) {
            TAGS_CUDA_OK(cudaMemcpyAsync(sol + k0 * N, p->d_x, sizeof(double2) * N * nb,
                                         dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        }
        if (info) {
            TAGS_CUDA_OK(cudaMemcpyAsync(info + k0, p->d_info, sizeof(int) * nb,
                                         dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        }
        if (!dev) TAGS_CUDA_OK(cudaStreamSynchronize(st));   // staging buffer reused by the next pass
    }
    return 0;
}

// The twins (the plan's further pipelines, a chain p->twin->twin) follow the
// plan's settings (split, panels per update, samples per pass, graphs, fill
// model) before they take passes.
static int sync_twin(tags_plan_s* p) {
    for (tags_plan_s* t = p->twin; t; t = t->twin) {
        if (t->split_pieces != p->split_pieces || t->group_panels != p->group_panels ||
            t->pass_batch != p->pass_batch || t->max_steps != p->max_steps || t->ir_tol != p->ir_tol ||
            t->tc_pairs != p->tc_pairs) {
            t->split_pieces = p->split_pieces;
            t->group_panels = p->group_panels;
            t->pass_batch = p->pass_batch;
            t->max_steps = p->max_steps;
            t->ir_tol = p->ir_tol;
            t->tc_pairs = p->tc_pairs;
            tags_plan_drop_graphs(t);
        }
        t->use_graphs = p->use_graphs;
        if (t->fill_model != p->fill_model)
            if (int e = tags_plan_set_fill(t, p->fill_model)) return e;
    }
    return 0;
}

extern "C" int tags_plan_set_pipelines(tags_plan plan, int pipelines) {
    tags_plan_s* p = plan;
    if (!p || p->twin == p) return tags_fail(TAGS_E_ARG, "tags_plan_set_pipelines: invalid plan");
    if (pipelines < 1 || pipelines > TAGS_MAX_PIPELINES)
        return tags_fail(TAGS_E_ARG, "tags_plan_set_pipelines: 1, 2 or 3");
    TAGS_CUDA_OK(cudaSetDevice(p->device));
    // twins beyond the count asked for are kept for a later switch back
    tags_plan_s* last = p;
    for (int k = 1; k < pipelines; ++k) {
        if (!last->twin) {
            tags_plan t = nullptr;
            const size_t m = (size_t)p->m, n = (size_t)p->n;
            int err = tags_plan_create(&t, reinterpret_cast<const Electrode*>(p->h_elec.data()),
                                       p->h_img.empty() ? nullptr : reinterpret_cast<const Electrode*>(p->h_img.data()),
                                       m, p->h_nodes.data(), n, p->precision, (size_t)p->batch);
            if (err) return err;
            if (t->batch != p->batch) {
                plan_free(t);
                return tags_fail(TAGS_E_NOMEM,
                                 "tags_plan_set_pipelines: no room for another pipeline of the same batch");
            }
            last->twin = t;
        }
        last = last->twin;
    }
    if (int err = sync_twin(p)) return err;
    p->pipelines = pipelines;
    return 0;
}

extern "C" int tags_plan_run(tags_plan plan, const tags_cdouble* s, const tags_cdouble* kappa, double mur, size_t ns,
                             const tags_cdouble* ie, size_t inj_node, tags_cdouble* sol, int* info, int flags,
                             tags_run_stats* stats) {
    tags_plan_s* p = plan;
    if (!p || !s || !kappa) return tags_fail(TAGS_E_ARG, "tags_plan_run: invalid argument");
    if (!ie && inj_node >= (size_t)p->n) return tags_fail(TAGS_E_ARG, "tags_plan_run: inj_node out of range");
    if (ns == 0) return 0;
    // host inputs are checked here; device inputs by k_coef, which reports a
    // non-finite sample and hands the kernels finite coefficients instead
    if (!(flags & TAGS_RUN_DEVICE_PTRS) && (!tags_all_finite(s, ns) || !tags_all_finite(kappa, ns)))
        return tags_fail(TAGS_E_NONFINITE, "tags_plan_run: s or kappa is not finite");
    TAGS_CUDA_OK(cudaSetDevice(p->device));
    cudaStream_t st = p->stream;
    DeviceCtx* ctx = tags_ctx();
    if (!ctx) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    if (stats) memset(stats, 0, sizeof(*stats));
    tags_run_stats acc{}, acc2{};
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_status, 0, sizeof(int) * 4, st));
    const size_t per_pass = p->pass_batch > 0 && p->pass_batch < p->batch ? p->pass_batch : p->batch;
    const size_t passes = (ns + per_pass - 1) / per_pass;
    // the pipelines that take passes: the plan and its first twins
    std::vector<tags_plan_s*> pl{p};
    for (tags_plan_s* t = p->twin; t && (int)pl.size() < p->pipelines && pl.size() < passes; t = t->twin)
        pl.push_back(t);
    if (pl.size() > 1) {
        if (int e = sync_twin(p)) return e;
        for (size_t k = 1; k < pl.size(); ++k)
            TAGS_CUDA_OK(cudaMemsetAsync(pl[k]->d_status, 0, sizeof(int) * 4, pl[k]->stream));
    }
    TAGS_CUDA_OK(cudaEventRecord(p->ev0, st));
    int err = 0;
    std::atomic<size_t> next{0};
    if (pl.size() > 1) {
        // each twin takes passes on its own stream from its own host thread;
        // they start after ev0 so the run's device time spans them all
        std::vector<tags_run_stats> accs(pl.size());
        std::vector<int> errs(pl.size(), 0);
        std::vector<std::thread> th;
        for (size_t k = 1; k < pl.size(); ++k) {
            tags_plan_s* t = pl[k];
            TAGS_CUDA_OK(cudaStreamWaitEvent(t->stream, p->ev0, 0));
        }
        for (size_t k = 1; k < pl.size(); ++k) {
            tags_plan_s* t = pl[k];
            th.emplace_back([&, k, t] {
                if (cudaSetDevice(t->device) != cudaSuccess) {
                    errs[k] = TAGS_E_CUDA;
                    return;
                }
                errs[k] = run_passes(t, s, kappa, mur, ns, ie, inj_node, sol, info, flags, per_pass, &next, &accs[k]);
                if (!errs[k] && cudaEventRecord(t->ev1, t->stream) != cudaSuccess) errs[k] = TAGS_E_CUDA;
            });
        }
        err = run_passes(p, s, kappa, mur, ns, ie, inj_node, sol, info, flags, per_pass, &next, &acc);
        for (auto& h : th) h.join();
        for (size_t k = 1; k < pl.size() && !err; ++k) err = errs[k];
        for (size_t k = 1; k < pl.size() && !err; ++k) {
            TAGS_CUDA_OK(cudaStreamWaitEvent(st, pl[k]->ev1, 0));
            acc.max_iterations = std::max(acc.max_iterations, accs[k].max_iterations);
            acc.max_backward_error = std::max(acc.max_backward_error, accs[k].max_backward_error);
            acc.fallbacks += accs[k].fallbacks;
        }
    } else {
        err = run_passes(p, s, kappa, mur, ns, ie, inj_node, sol, info, flags, per_pass, &next, &acc);
    }
    if (err) return err;
    TAGS_CUDA_OK(cudaEventRecord(p->ev1, st));
    int status[TAGS_MAX_PIPELINES] = {0};
    for (size_t k = 0; k < pl.size(); ++k)
        TAGS_CUDA_OK(cudaMemcpyAsync(&status[k], pl[k]->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (stats) {
        *stats = acc;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, p->ev0, p->ev1);
        stats->seconds = ms * 1e-3;
        stats->split = p->precision == TAGS_PLAIN_FP64 ? 0 : p->split_pieces;
    }
    int stt = 0;
    for (int k = 0; k < TAGS_MAX_PIPELINES; ++k) stt |= status[k];
    if (stt & TAGS_ST_DEGENERATE_PAIR)
        return tags_fail(TAGS_E_GEOMETRY, "coincident or overlapping segments: the pair integral diverges");
    if (stt & TAGS_ST_NONFINITE) return tags_fail(TAGS_E_NONFINITE, "non-finite value in the impedance fill");
    if (stt & TAGS_ST_BAD_ARG)
        return tags_fail(TAGS_E_ARG, "a sample's propagation constant is outside the supported range (|gamma| > 1e5 / m)");
    return 0;
}
