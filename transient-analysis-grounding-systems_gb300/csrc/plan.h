// Device context and batched-plan state shared by the C-ABI translation units.
#pragma once

#include <complex>
#include <mutex>
#include <vector>
#include <cuda_runtime.h>

#include "tags_internal.h"

struct DeviceCtx {
    bool ready = false;
    int device = -1;
    cudaStream_t stream = nullptr;
    int* status = nullptr;             // device status word(s)
    void* scratch_ptr[16] = {};
    size_t scratch_bytes[16] = {};
    void* scratch(int slot, size_t bytes);
};

DeviceCtx* tags_ctx();
std::mutex& tags_dropin_mutex();
int tags_fail(int code, const char* msg);
void tags_msg(const char* msg);
SampleCoef tags_sample_coef(std::complex<double> gamma, std::complex<double> s, double mur,
                            std::complex<double> kappa, std::complex<double> ref_l, std::complex<double> ref_t);

// Sparse incidence (from the exact node-matching codes): per node the
// incident segments (CSR by node) and per segment its nodes (CSR by segment),
// with the A value (+1/-1); B is 0.5 on the same pattern.
struct Incidence {
    int* node_ptr = nullptr;   // n + 1
    int* node_seg = nullptr;   // nnz
    signed char* node_a = nullptr;
    int* seg_ptr = nullptr;    // m + 1
    int* seg_node = nullptr;   // nnz
    signed char* seg_a = nullptr;
    int nnz = 0;
};

constexpr int TAGS_MAX_PIPELINES = 3;     // passes in flight per plan

struct tags_plan_s {
    int device = -1;
    int precision = 0;
    int m = 0, n = 0, N = 0;
    int has_images = 0;
    int batch = 0;               // samples per device pass
    cudaStream_t stream = nullptr;
    double* d_elec = nullptr;    // m x 11
    double* d_img = nullptr;     // m x 11
    signed char* d_cond = nullptr;  // n x m incidence codes
    Incidence inc;
    SampleCoef* d_coef = nullptr;   // batch
    int* d_status = nullptr;        // 4 words
    int* d_info = nullptr;          // batch
    int* d_ipiv = nullptr;          // batch x N
    double2* d_W = nullptr;         // plain: batch x N x N
    double2* d_x = nullptr;         // batch x N (solution, FP64)
    // mixed form
    float2* d_Z = nullptr;          // batch x 2 x m x m complex FP32 (ZL, ZT; full symmetric)
    float2* d_A = nullptr;          // batch x N x N FP32 working matrix (reordered, scaled)
    double* d_scale = nullptr;      // batch x N symmetric scaling (reordered index)
    double2* d_r = nullptr;         // batch x N residual (FP64)
    float2* d_rf = nullptr;         // batch x N correction right-hand side (FP32)
    double* d_norms = nullptr;      // batch x 4 reductions
    float2* d_yprev = nullptr;      // batch x N previous refinement correction (FP32, as d_rf)
    double* d_dots = nullptr;       // batch x 4 sums of the current against the previous correction
    void* d_fillws = nullptr;       // pair classes and geometry records of the mixed fill
    int n_touch = 0;                // pairs sharing an endpoint (FP64 Duffy rule)
    SpecialEntries spec;            // entries filled in FP64 per sample (touching pairs, diagonal)
    MomentFill mom;                 // moment expansion of the regular pairs (geometry moments, per-pass tables)
    float2* d_Zlo = nullptr;        // batch x 2 x m x m: low parts of ZL, ZT (Z holds the high parts)
    float* d_rowpart = nullptr;     // row statistics' partials of a pass (tags_launch_fill_mixed)
    void* d_ldlws = nullptr;        // tensor-core LDL^T workspace (split planes, block inverses)
    int* d_ldlerr = nullptr;        // error word of the tensor-core kernels
    int split_pieces = TAGS_SPLIT_F16;   // split form of the tensor-core products (2, 3 bf16 pieces; TAGS_SPLIT_F16)
    int fill_model = TAGS_INTG_DOUBLE;  // TAGS_INTG_DOUBLE (double line integrals) or TAGS_INTG_MHEM
    double2* d_pot = nullptr;       // mHEM: 4 x m x m static potentials (direct ZL, ZT; images ZL, ZT)
    SampleCoef* d_coef1 = nullptr;  // unit coefficients for the potentials
    int group_panels = 6;           // tensor-core LDL^T: panels per trailing update (1 .. 6; K = 128 x that)
    int max_steps = 40;             // refinement steps per pass before the FP64 fallback (1 .. 40)
    int tc_pairs = 0;               // trailing updates on two-SM clusters (tcgen05 cta_group::2)
    double ir_tol = 1e-9;           // refinement stopping tolerance (relative error left in x)
    int pass_batch = 0;             // samples per pass (<= batch; 0 = batch)
    int* d_iri = nullptr;           // refinement state: active, converged, iterations (batch each), step, continue,
                                    // step of the last extrapolation (batch)
    double* d_ird = nullptr;        // refinement state: previous correction, max row sum, backward error,
                                    // |lambda| of the last extrapolation (batch each)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // CUDA-graph passes: inputs staged in plan-owned buffers, one executable
    // graph per pass shape (samples, mu_r, injection form)
    int use_graphs = 1;
    double2* d_sin = nullptr;       // 2 x batch: s, kappa
    double2* d_iein = nullptr;      // batch x n injections (allocated on first use)
    struct GraphPass {
        int nb = 0, has_ie = 0, inj = 0;
        double mur = 0.0;
        cudaGraphExec_t exec = nullptr;
        long long launches_fixed = 0;   // kernels outside the refinement loop
        long long launches_step = 0;    // kernels of one refinement step
    };
    std::vector<GraphPass> graphs;
    // plan-owned scratch (so distinct plans run concurrently from several host
    // threads): host-input staging of kernel-by-kernel passes, FP64 fallback
    double2* d_stage = nullptr;
    size_t stage_bytes = 0;
    double2* d_fbW = nullptr;       // N x N (allocated on the first fallback)
    int* d_fbpiv = nullptr;         // N + 1
    // host copy of the geometry (11 doubles per segment; nodes 3 per node), so
    // a twin plan can be built from it
    std::vector<double> h_elec, h_img, h_nodes;
    // further pipelines (tags_plan_set_pipelines): a chain of plans of the
    // same geometry and settings, each on its own stream; a run's passes go to
    // whichever pipeline frees up first
    tags_plan_s* twin = nullptr;
    int pipelines = 1;                  // 1 .. TAGS_MAX_PIPELINES
};

int tags_plan_run_plain(tags_plan_s* p, const double2* d_s_unused, int nb, cudaStream_t st);
int tags_mixed_alloc(tags_plan_s* p);
int tags_mixed_free(tags_plan_s* p);
int tags_mixed_solve_batch(tags_plan_s* p, int nb, const double2* d_b, int* h_iters, double* h_berr,
                           int* h_conv, cudaStream_t st);
int tags_mixed_factor(tags_plan_s* p, int nb, cudaStream_t st);
// the impedance fill of a pass into W_G (plain) per the plan's fill model
int tags_plan_fill_fp64(tags_plan_s* p, const SampleCoef* d_coef, int nb, const FillOut& out, cudaStream_t st);
void tags_plan_drop_graphs(tags_plan_s* p);
int tags_mixed_ir_setup(tags_plan_s* p, int nb, cudaStream_t st);
int tags_mixed_ir_step(tags_plan_s* p, int nb, cudaStream_t st, cudaGraphConditionalHandle cond, int set_cond);
int tags_mixed_finish(tags_plan_s* p, int nb, cudaStream_t st, int* h_iters, double* h_berr, int* h_conv,
                      int* h_steps);
// Plain FP64 re-solve of one sample (inputs on the device) into x_out / info_out.
int tags_mixed_fallback_one(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur,
                            const double2* d_ie, int inj_node, double2* x_out, int* info_out, cudaStream_t st);
// While-node after the work captured so far on `st` (condition 1 at launch);
// its body graph is returned for a separate capture.
int tags_plan_add_while_node(cudaStream_t st, cudaGraphConditionalHandle* cond, cudaGraph_t* body);
