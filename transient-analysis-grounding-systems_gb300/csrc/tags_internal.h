// Internal interfaces between the CUDA translation units of the GB300 HEM
// library (not part of the public C-ABI in include/tags_gpu.h).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

// NVTX range over a host-side phase (fill, assemble, factor, refine, FP64
// re-solve, INLT, a pass or a grid batch): pushed on construction, popped on
// destruction. NVTX 3 is header-only; with no tool attached a push and a pop
// cost a few nanoseconds. In graph mode a pass is one range around its launch.
struct TagsRange {
    explicit TagsRange(const char* name) { nvtxRangePushA(name); }
    ~TagsRange() { nvtxRangePop(); }
    // ends this phase and opens the next one
    void next(const char* name) {
        nvtxRangePop();
        nvtxRangePushA(name);
    }
    TagsRange(const TagsRange&) = delete;
    TagsRange& operator=(const TagsRange&) = delete;
};

// Integration types, numbered as the reference's Integration_type
// (src/electrode.h:17-31).
enum { TAGS_INTG_NONE = 1, TAGS_INTG_DOUBLE = 2, TAGS_INTG_SINGLE = 3, TAGS_INTG_MHEM = 4 };

// Which couplings a fill launch computes.
enum { TAGS_FILL_DIRECT = 1, TAGS_FILL_IMAGE = 2, TAGS_FILL_BOTH = 3 };

// Per-sample coefficients, computed on the host from s, kappa, mur:
//   gamma = sqrt(s mur mu0 kappa), cL = s mur mu0 / 4pi, cT = 1 / (4 pi kappa),
//   cLi = ref_l cL, cTi = ref_t cT (examples/three_grids.c:326-333,
//   src/electrode.c:313-319, :391-399).
struct SampleCoef {
    double2 gamma;
    double2 cL, cT;
    double2 cLi, cTi;
};

// Where the lower triangle (row k >= col i) of ZL/ZT lands: element (k, i) of
// ZL goes to zl[(row0_l + k) + ld * (col0_l + i)] (+ batch_stride per sample),
// multiplied by `sign`; with `mirror` also to the transposed position.
struct FillOut {
    double2* zl;
    double2* zt;
    long long ld;
    long long batch_stride;
    int row0_l, col0_l, row0_t, col0_t;
    double sign;
    int mirror;
    int accumulate;
};

int tags_fill_tables_init();
// mHEM fill: static potentials once per geometry, then a rescale per sample
int tags_launch_mhem_potentials(const double* d_elec, const double* d_img, int m, int has_img, double2* d_pot,
                                SampleCoef* d_coef1, int* d_status, cudaStream_t st);
int tags_launch_mhem_fp64(const double* d_elec, const double* d_img, int m, int has_img, const double2* d_pot,
                          const SampleCoef* d_coef, int nsamp, const FillOut& out, int* d_status, cudaStream_t st);
int tags_launch_mhem_mixed(int m, int has_img, const double2* d_pot, void* ws, const SampleCoef* d_coef, int nsamp,
                           float2* d_zl, float2* d_zt, long long bstride, int* d_status, cudaStream_t st);
// mixed-form fill (FP32 regular pairs, FP64 log-singular pairs); the
// workspace holds the plan-time pair classes and geometry records
size_t tags_mixed_fill_workspace(int m);
int tags_launch_pair_plan(const double* d_elec, const double* d_img, int m, int has_img, void* ws, cudaStream_t st);
int tags_mixed_touch_count(void* ws, int m, cudaStream_t st, int* out);
// The entries of ZL/ZT the mixed fill computes in FP64 per sample: pairs with
// a kind (direct or image) that shares an endpoint (log-singular) and the
// diagonal (the self term), added to the regular kinds' value in FP64 and
// stored as a float pair (hi in Z, lo in Zlo).
struct SpecialEntries {
    int n = 0;                   // entries
    int2* ent = nullptr;         // (pair index p of (k, i), k >= i; kinds mask: bit 0 direct, 1 image, 2 self)
    double* tm = nullptr;        // FP64 Duffy moments of the touching kinds: [entry][kind][24]
    double tdmax = 0.0;          // bound of the Duffy distances (2 x the longest segment)
};
int tags_mixed_special_build(void* ws, int m, int batch, SpecialEntries* sp, cudaStream_t st);
// the Duffy moments of the special entries' touching kinds (once per plan)
int tags_mixed_special_moments(const double* d_elec, const double* d_img, int m, double lmax, SpecialEntries* sp,
                               cudaStream_t st);
void tags_mixed_special_free(SpecialEntries* sp);
// The moment expansion of the regular kinds (fill.cu): moments of every
// (pair, kind) once per plan; per pass the samples' constants and the table
// e^{-gamma b h} of the expansion centres.
struct MomentFill {
    float* mom = nullptr;        // (pair, kind) moments, 32 floats each
    void* rec = nullptr;         // (pair, kind) records
    void* coef = nullptr;        // per-sample constants, batch
    int* ok = nullptr;           // per sample: 1 where the series reaches FP64 accuracy (else the FP32 quadrature)
    float4* tab = nullptr;       // f e^{-gamma b h}, f = cT, cTi, cL: [3][bucket][sample], complex float pairs
    int nb = 0;                  // buckets
    double dmax = 0.0;           // bound of |r - R| over the pairs (m)
    int batch = 0;
};
int tags_moment_fill_build(const double* d_elec, const double* d_img, int m, int has_img, const double* h_elec,
                           const double* h_img, int batch, MomentFill* mf, cudaStream_t st);
void tags_moment_fill_free(MomentFill* mf);
// The mixed fill of a pass: ZL, ZT as float pairs (hi in d_zl / d_zt, lo in
// d_zlo / d_ztlo), full symmetric. rowpart (optional, 2 x 2 nsamp x ceil(m/32)
// x m floats): the row statistics' partials of the high parts, max then sum,
// [matrix][32-column block][row] (matrix = 2 sample + 0 for ZL, 1 for ZT).
int tags_launch_fill_mixed(const double* d_elec, const double* d_img, int m, void* ws, const SampleCoef* d_coef,
                           int nsamp, float2* d_zl, float2* d_zt, float2* d_zlo, float2* d_ztlo, long long bstride,
                           int has_img, const SpecialEntries& sp, const MomentFill& mf, int* d_status,
                           cudaStream_t st, float* rowpart = nullptr);
int tags_launch_fill_fp64(const double* d_elec, const double* d_img, int m, const SampleCoef* d_coef,
                          int nsamp, const FillOut& out, int mode, int itype, int tight, int* d_status,
                          cudaStream_t st);

// Double integrals of e^{-gamma r}/r over [0,1]^2 between each path (a
// segment record with radius 0) and each electrode, for every sample:
// jj[(s * npaths + l) * m + e], unscaled (FP64, the plain fill's rule).
int tags_launch_path_pairs(const double* d_elec, int m, const double* d_paths, int npaths, const SampleCoef* d_coef,
                           int nsamp, double2* d_jj, int* d_status, cudaStream_t st);
// Gauss-Legendre nodes (ascending) and weights on [0, 1] (host side).
void tags_gauss_legendre(int q, double* x, double* w);

// Bookkeeping of kernel launches (reported by tags_gpu_launch_count), also
// per host thread: a graph capture measures and removes its own launches by
// the calling thread's count, so passes captured on other threads at the
// same time (the pipelines' twins) do not disturb it.
void tags_note_launch(long long n = 1);
long long tags_thread_launch_count();
// Free device memory for sizing plans and grid batches (tags_gpu_set_memory_budget caps it).
cudaError_t tags_free_memory(size_t* freeb);
// Host arrays of n complex doubles (real, imaginary): all finite (null counts as finite).
bool tags_all_finite(const void* v, size_t n);

// assemble.cu
int tags_incidence_codes(const double* d_elec, int m, const double* d_nodes, int n, signed char* d_cond,
                         cudaStream_t st);
int tags_wg_incidence(double2* d_W, long long ld, long long stride, int batch, const signed char* d_cond, int n,
                      int m, cudaStream_t st);
int tags_wg_impedance(double2* d_W, long long ld, const double2* d_zl, const double2* d_zt, int m, int n,
                      cudaStream_t st);
int tags_symmetrize_lower(double2* d_W, int N, long long ld, long long stride, int batch, cudaStream_t st);

// lu.cu
int tags_lu_z(double2* A, int n, long long ld, long long stride, int batch, int pivot, int* ipiv, int* info,
              cudaStream_t st);
int tags_lu_c(float2* A, int n, long long ld, long long stride, int batch, int pivot, int* ipiv, int* info,
              cudaStream_t st);
int tags_lu_solve_z(const double2* A, int n, long long ld, long long stride, int batch, const int* ipiv, double2* X,
                    int nrhs, long long ldx, long long xstride, cudaStream_t st);
int tags_lu_solve_c(const float2* A, int n, long long ld, long long stride, int batch, const int* ipiv, float2* X,
                    int nrhs, long long ldx, long long xstride, cudaStream_t st);

// inlt.cu
int tags_twiddles(double2* d_tw, long long nt, cudaStream_t st);
int tags_launch_inlt(const double2* d_g, long long gstride, long long ns, const double2* d_s, const double2* d_tw,
                     long long nt, double tmax, int filter, double* d_f, long long fstride, int nseries,
                     cudaStream_t st);
int tags_launch_inlt_rows(const double2* d_g, long long ns, const double2* d_s, const double2* d_tw, long long nt,
                          double tmax, int filter, double* d_f, long long nser, cudaStream_t st);
int tags_launch_nlt(const double* d_f, long long fstride, long long nt, const double2* d_tw, double tmax,
                    double2* d_g, long long gstride, int nseries, cudaStream_t st);

// ldl_tc.cu: tensor-core LDL^T of complex FP32 symmetric matrices (no pivoting)
// Split forms of the tensor-core LDL^T (`pieces` argument of tags_ldl_tc):
// 2 or 3 bf16 pieces, or TAGS_SPLIT_F16 = two fp16 pieces of 2^8 x.
constexpr int TAGS_SPLIT_F16 = 16;
int tags_lu_prepare();
int tags_ldl_tc_prepare();
size_t tags_ldl_tc_workspace(int N, int batch);
// zl_m > 0: the matrix is ordered [ZL (zl_m), ZT (zl_m), rest] with a zero ZL/ZT
// coupling block, which the factorisation and the solves skip.
// pieces: bf16 pieces per real value in the split products (2: three
// products per real product, ~2^-16; 3: six products, ~2^-23).
// pairs: the mode-0 updates on two-SM clusters (tcgen05 cta_group::2) where available.
int tags_ldl_tc(float2* A, int N, long long ld, long long mstride, int nb, int batch_cap, void* ws, int* info,
                int* err, int zl_m, int pieces, int group_panels, cudaStream_t st, int pairs);
// active (optional, per sample): samples whose flag is 0 are skipped.
// lead_step (optional, device): while *lead_step is 0 the right-hand sides are
// zero in their first lead_zero rows, and the forward sweep starts at the
// first block that reaches past them.
// nact (optional, device, with active): the number of active samples; where
// the solves run one CTA per sample, a step with at most SMs / 4 of them
// active runs on clusters of four CTAs per active sample instead.
int tags_ldl_solve_c(const float2* A, int N, long long ld, long long mstride, int nb, int batch_cap, void* ws,
                     float2* x, long long xstride, int zl_m, cudaStream_t st, const int* active = nullptr,
                     const int* lead_step = nullptr, int lead_zero = 0, const int* nact = nullptr);

// profile.cu: optional CUDA-event timing of kernel families
enum {
    TAGS_PROF_FILL_FP64 = 0, TAGS_PROF_FILL_MIXED, TAGS_PROF_LDL_DIAG, TAGS_PROF_LDL_PANEL, TAGS_PROF_LDL_TRAIL,
    TAGS_PROF_LDL_SOLVE, TAGS_PROF_RESID, TAGS_PROF_BUILD, TAGS_PROF_LU64_GEMM, TAGS_PROF_LU64_OTHER,
    TAGS_PROF_FIELDS, TAGS_PROF_N
};
int tags_prof_begin(int fam, cudaStream_t st);
void tags_prof_end(int fam, int slot, cudaStream_t st, double flops, double bytes);
