/* GB300-native drop-in for the frequency-domain HEM hot path of
 * pedrohnv/transient-analysis-grounding-systems (TAGS).
 *
 * Part 1 -- drop-in entry points. Same names, argument meaning, return codes
 * and memory contract as the reference C library, so C callers relink against
 * libtags_gpu.so instead of libhphem.so (host buffers in, host buffers out;
 * each call copies to and from the GPU):
 *   calculate_impedances   replaces src/electrode.c:304-377 (decl src/electrode.h:276-281)
 *   impedances_images      replaces src/electrode.c:379-431 (decl src/electrode.h:310-317)
 *   fill_incidence_imm     replaces src/linalg.c:12-86      (decl src/linalg.h:38-41)
 *   fill_impedance_imm     replaces src/linalg.c:88-110     (decl src/linalg.h:56-59)
 *   solve_immittance       replaces src/linalg.c:112-139    (decl src/linalg.h:79-81)
 *   fill_incidence_adm     replaces src/linalg.c:142-204    (decl src/linalg.h:103-106)
 *   fill_impedance_adm     replaces src/linalg.c:206-259    (decl src/linalg.h:123-126)
 *   calculate_yla_ytb      replaces src/linalg.c:261-300    (decl src/linalg.h:145-149)
 *   fill_impedance_adm2    replaces src/linalg.c:302-325    (decl src/linalg.h:169-173)
 *   solve_admittance       replaces src/linalg.c:327-350    (decl src/linalg.h:192-193)
 *   electric_potential     replaces src/electrode.c:434-457 (decl src/electrode.h:333-337)
 *   magnetic_potential     replaces src/electrode.c:459-493 (decl src/electrode.h:355-360)
 *   electric_field         replaces src/electrode.c:522-560 (decl src/electrode.h:398-403)
 *   voltage                replaces src/electrode.c:637-668 (decl src/electrode.h:440-446)
 * and host-side helpers of the reference (no device work):
 *   electrodes_file        src/electrode.c:45-80    (decl src/electrode.h:127-128)
 *   nodes_file             src/electrode.c:82-101   (decl src/electrode.h:140-141)
 *   alipio_soil            src/auxiliary.c:60-70    (decl src/auxiliary.h:101-103)
 *   smith_longmire_soil    src/auxiliary.c:72-93    (decl src/auxiliary.h:119-121)
 *   heidler                src/auxiliary.c:331-336  (decl src/auxiliary.h:398)
 *   laplace_trans          replaces src/auxiliary.c:239-263 (decl src/auxiliary.h:320-321)
 *   inv_laplace_trans      replaces src/auxiliary.c:265-329 (decl src/auxiliary.h:366-368)
 *
 * Part 2 -- batched extension (no counterpart in the reference; it replaces the
 * per-sample OpenMP loop the reference's examples write around the calls
 * above, e.g. examples/three_grids.c:286-443): a plan keeps geometry,
 * incidence and workspaces on the device and solves many Laplace samples per
 * launch sequence, in plain FP64 or in the mixed-precision form.
 *
 * Complex numbers are C99 `double _Complex` (16 bytes, real part first).
 * Matrices are column-major, as in the reference.
 */
#ifndef TAGS_GPU_H_
#define TAGS_GPU_H_

#include <stddef.h>

#ifdef __cplusplus
/* Same size, alignment and calling convention as C99 double _Complex on the
 * x86-64 SysV and AArch64 ABIs (two doubles in floating-point registers). */
typedef struct { double re, im; } tags_cdouble;
extern "C" {
#else
#include <complex.h>
typedef double _Complex tags_cdouble;
#endif

/* The reference's segment record (src/electrode.h:33-45) and integration
 * types (src/electrode.h:17-31). Defined here only when the reference's
 * electrode.h was not included first. */
#ifndef ELECTRODE_H_
typedef struct {
    double start_point[3];
    double end_point[3];
    double middle_point[3];
    double length;
    double radius;
} Electrode;
enum Integration_type { INTG_NONE = 1, INTG_DOUBLE = 2, INTG_SINGLE = 3, INTG_MHEM = 4 };
#endif

/* ---- Part 1: drop-in entry points ----------------------------------------- */

/* Lower triangle (zl[i*m + k], k >= i) of ZL and ZT of the segments. The
 * cubature tolerances are accepted for source compatibility; the GPU uses a
 * fixed-order rule that meets ~1e-12 relative accuracy on every pair. zl == zt
 * is allowed and reproduces the reference's write order. Returns 0, or -10 for
 * an unknown integration_type, or a negative TAGS_E_* code. */
int calculate_impedances (tags_cdouble *zl, tags_cdouble *zt, const Electrode *electrodes,
                          size_t num_electrodes, tags_cdouble gamma, tags_cdouble s, double mur,
                          tags_cdouble kappa, size_t max_eval, double req_abs_error,
                          double req_rel_error, int integration_type);

/* Adds (+=) the couplings to the image segments (k >= i, diagonal included). */
int impedances_images (tags_cdouble *zl, tags_cdouble *zt, const Electrode *electrodes,
                       const Electrode *images, size_t num_electrodes, tags_cdouble gamma,
                       tags_cdouble s, double mur, tags_cdouble kappa, tags_cdouble ref_l,
                       tags_cdouble ref_t, size_t max_eval, double req_abs_error,
                       double req_rel_error, int integration_type);

/* Incidence blocks A, B (and transposes) of W_G, leading dimension n + 2m.
 * Returns 1 at the first node without incidence (nodes up to it are written),
 * -sum(A) or sum(B) - m on a bad checksum, 0 on success. */
int fill_incidence_imm (tags_cdouble *wg, const Electrode *electrodes, size_t num_electrodes,
                        const double *nodes, size_t num_nodes);

/* -ZL, -ZT (whole m x m blocks as stored), zero coupling blocks, zero Y_E. */
int fill_impedance_imm (tags_cdouble *wg, const tags_cdouble *zl, const tags_cdouble *zt,
                        size_t num_electrodes, size_t num_nodes);

/* Solves W_G x = ie (W_G symmetric, lower half read); ie <- [U; I_L; I_T].
 * Returns 0, or k > 0 when the k-th pivot of the factorisation is exactly
 * zero (singular system). wg is left unchanged (the reference leaves its
 * factorisation there; its content is not part of the contract). */
int solve_immittance (tags_cdouble *wg, tags_cdouble *ie, size_t num_electrodes, size_t num_nodes);

/* ---- geometry files and soil models (host only) ----------------------------- */

/* Reads num_electrodes lines "x0, y0, z0, x1, y1, z1, r". Returns 0, -10 if
 * the file cannot be opened, (values read - 7) at the first bad line, or
 * 1 / 2 for coincident end points / a radius <= 0. */
int electrodes_file (const char file_name[], Electrode *electrodes, size_t num_electrodes);

/* Reads num_nodes lines "x, y, z" into nodes (3 per node). Returns 0, -10 if
 * the file cannot be opened, or (values read - 3) at the first bad line. */
int nodes_file (const char file_name[], double *nodes, size_t num_nodes);

/* Alipio-Visacro soil: conductivity and relative permittivity at s. */
int alipio_soil (tags_cdouble *sigma, tags_cdouble *epsr, double sigma0, tags_cdouble s, double h, double g,
                 double eps_ratio);

/* Smith-Longmire soil: conductivity and relative permittivity at s. */
int smith_longmire_soil (tags_cdouble *sigma, tags_cdouble *epsr, double sigma0, tags_cdouble s, double erinf);

/* Heidler lightning-current waveform at time t (peak imax, front and tail
 * time constants tau1, tau2, steepness n). */
double heidler (double t, double imax, double tau1, double tau2, double n);

/* ---- nodal admittance formulation (the reference's mHEM examples) ---------- */

/* A (+1 start, -1 end) and B (0.5), num_electrodes x num_nodes column-major.
 * Written in the reference's order (b before a at a match: a == b leaves A);
 * returns 1 at the first node without incidence, -sum(A) or sum(B) - m on a
 * bad checksum (read back from the arrays), 0 on success. */
int fill_incidence_adm (tags_cdouble *a, tags_cdouble *b, const Electrode *electrodes, size_t num_electrodes,
                        const double *nodes, size_t num_nodes);

/* yn (n x n) = A^T ZL^{-1} A + B^T ZT^{-1} B from the lower triangles of
 * zl, zt (m x m), which are overwritten by the inverses' lower triangles as
 * the reference's zsytrf + zsytri leave them. Returns 0 or the order k > 0 of
 * an exactly zero pivot. */
int fill_impedance_adm (tags_cdouble *yn, tags_cdouble *zl, tags_cdouble *zt, tags_cdouble *a, tags_cdouble *b,
                        size_t num_electrodes, size_t num_nodes);

/* yla = ZL^{-1} A, ytb = ZT^{-1} B (m x n); zl, zt as in fill_impedance_adm. */
int calculate_yla_ytb (tags_cdouble *yla, tags_cdouble *ytb, tags_cdouble *zl, tags_cdouble *zt,
                       tags_cdouble *a, tags_cdouble *b, size_t num_electrodes, size_t num_nodes);

/* yn = A^T yla + B^T ytb (n x n). */
int fill_impedance_adm2 (tags_cdouble *yn, tags_cdouble *yla, tags_cdouble *ytb, tags_cdouble *a,
                         tags_cdouble *b, size_t num_electrodes, size_t num_nodes);

/* Solves YN u = ic (YN symmetric, lower half read); ic <- u. Returns 0 or
 * k > 0 for an exactly zero pivot. yn is left unchanged. */
int solve_admittance (tags_cdouble *yn, tags_cdouble *ic, size_t num_nodes);

/* Numerical Laplace transform and its inverse, with the reference's
 * conventions (s_k = c + j k 2pi/tmax, c = ln(nt^2)/tmax; window `filter` as
 * the reference's INLT_Filter: 0 none, 1 Blackman, 2 Hanning, 3 Lanczos,
 * 4 Riesz). */
int laplace_trans (double *f, tags_cdouble *g, tags_cdouble *s, double tmax, size_t nt);
int inv_laplace_trans (double *f, tags_cdouble *g, tags_cdouble *s, double tmax, size_t nt,
                       int filter);

/* No counterpart function in the reference: the inverse transform of many
 * series at once in the layout of the examples' fftw_plan_many_dft_c2r
 * (examples/three_grids.c:229-242): g[series + k * nseries] for the ns =
 * nt/2 + 1 samples (sample-major, e.g. node potentials of every sample), f
 * [series + j * nseries] for nt times, scaled by e^{c t_j} / (nt dt) as the
 * examples' output loop does (:447-465); filter as in inv_laplace_trans.
 * flags: TAGS_RUN_DEVICE_PTRS for device pointers (declared below). */
int tags_inv_laplace_batch (double *f, const tags_cdouble *g, const tags_cdouble *s, double tmax, size_t nt,
                            size_t nseries, int filter, int flags);
/* The same transform under the name of the batched extension. */
int tags_gpu_inlt (double *f, const tags_cdouble *g, const tags_cdouble *s, double tmax, size_t nt, size_t nseries,
                   int filter, int flags);

/* ---- post-processing: potentials, fields, path voltage --------------------- */
/* The tolerance arguments (max_eval, req_abs_error, req_rel_error) are
 * accepted and unused: the GPU rules integrate to ~1e-12 relative. A point on
 * an electrode (divergent integral) gives NaN. */

/* Scalar potential to remote earth at `point` from the transversal currents
 * it (num_electrodes): sum it[m] \int e^{-gamma r}/r dt / (4 pi kappa). */
tags_cdouble electric_potential (const double *point, const Electrode *electrodes, size_t num_electrodes,
                                 const tags_cdouble *it, tags_cdouble gamma, tags_cdouble kappa, size_t max_eval,
                                 double req_abs_error, double req_rel_error);

/* Magnetic vector potential (3 components, overwritten) from the
 * longitudinal currents il; electrodes with |il| < DBL_EPSILON are skipped. */
int magnetic_potential (const double *point, const Electrode *electrodes, size_t num_electrodes,
                        const tags_cdouble *il, tags_cdouble gamma, double mur, size_t max_eval,
                        double req_abs_error, double req_rel_error, tags_cdouble *va);

/* Electric field -grad u - s A. As in the reference, ve is overwritten by
 * -s A when |s| > DBL_EPSILON and the conservative part is then added; with
 * |s| <= DBL_EPSILON only the conservative part is added to ve. */
int electric_field (const double *point, const Electrode *electrodes, size_t num_electrodes,
                    const tags_cdouble *il, const tags_cdouble *it, tags_cdouble gamma, tags_cdouble s, double mur,
                    tags_cdouble kappa, size_t max_eval, double req_abs_error, double req_rel_error,
                    tags_cdouble *ve);

/* The reference's path voltage from point1 to point2: the integral over t in
 * [0, 1] of E . (point2 - point1) / |point2 - point1| (the voltage along the
 * straight path divided by its length). */
tags_cdouble voltage (const double *point1, const double *point2, const Electrode *electrodes,
                      size_t num_electrodes, const tags_cdouble *il, const tags_cdouble *it, tags_cdouble gamma,
                      tags_cdouble s, double mur, tags_cdouble kappa, size_t max_eval, double req_abs_error,
                      double req_rel_error);

/* Batched post-processing (no counterpart function in the reference; it
 * replaces the per-point, per-sample loops of examples/visacro57emc01.c:
 * 406-460). Currents il/it are [sample][injection][electrode] (each sample's
 * ne x nrhs column-major block, samples one after another); gamma and kappa
 * per sample.
 *   pot     [sample][point][injection]      electric_potential
 *   vecpot  [sample][point][injection][3]   magnetic_potential
 *   efield  [sample][point][injection][3]   conservative field -grad u (the
 *           full field is efield - s vecpot), as electric_field with s = 0
 * Any output may be NULL. Returns 0, TAGS_E_GEOMETRY when a point lies on an
 * electrode (its outputs are NaN), or another TAGS_E_* code. */
int tags_fields_batch (const double *points, size_t num_points, const Electrode *electrodes, size_t num_electrodes,
                       const tags_cdouble *il, const tags_cdouble *it, size_t nrhs, size_t nsamples,
                       const tags_cdouble *gamma, const tags_cdouble *kappa, double mur, tags_cdouble *pot,
                       tags_cdouble *vecpot, tags_cdouble *efield);

/* Ground potential by the examples' closed-form mHEM expression
 * (examples/visacro57emc01.c:406-430): gpd[sample][point][injection] = sum_m
 * it[m] e^{-gamma rbar} log((r1 + r2 + L) / (r1 + r2 - L)) / (L 4 pi kappa),
 * rbar, r1, r2 the distances from the point to the midpoint and the ends of
 * electrode m. it as above, already multiplied by (1 + ref_t) where the
 * caller wants the images' effect at ground level (as the example does). */
int tags_gpd_mhem_batch (const double *points, size_t num_points, const Electrode *electrodes,
                         size_t num_electrodes, const tags_cdouble *it, size_t nrhs, size_t nsamples,
                         const tags_cdouble *gamma, const tags_cdouble *kappa, tags_cdouble *gpd);

/* Path voltages (the reference's voltage) for paths[6 * l] = (x1, y1, z1, x2,
 * y2, z2): v[sample][path][injection]; s per sample. NaN for a path whose
 * squared length is below DBL_EPSILON. */
int tags_voltage_batch (const double *paths, size_t num_paths, const Electrode *electrodes, size_t num_electrodes,
                        const tags_cdouble *il, const tags_cdouble *it, size_t nrhs, size_t nsamples,
                        const tags_cdouble *gamma, const tags_cdouble *s, const tags_cdouble *kappa, double mur,
                        tags_cdouble *v);

/* Node evaluations (rule node x sample) made by the field kernels on the
 * current device since the last reset: the unit of work of the post-processing
 * rules, for throughput reports. reset != 0 zeroes the counter after reading. */
int tags_fields_evaluations (unsigned long long *count, int reset);

/* ---- Part 2: batched extension -------------------------------------------- */

enum {
    TAGS_PLAIN_FP64 = 0,  /* FP64 fill, FP64 LU with partial pivoting */
    TAGS_MIXED = 1        /* FP32/FP64 fill, low-precision LU + FP64 refinement */
};

/* Error codes (negative) of the extension and of argument checks. */
enum {
    TAGS_E_ARG = -101,          /* invalid argument or size */
    TAGS_E_CUDA = -102,         /* CUDA runtime failure (see tags_gpu_last_error) */
    TAGS_E_NOMEM = -103,        /* device allocation failed */
    TAGS_E_GEOMETRY = -104,     /* coincident/overlapping segments (divergent integral) */
    TAGS_E_NONFINITE = -105     /* NaN or Inf in a result */
};

/* Run flags. */
enum {
    TAGS_RUN_DEVICE_PTRS = 1,   /* s, kappa, ie and the outputs are device pointers */
    TAGS_TUNE_REFRESH = 256     /* tags_plan_tune only: time the candidates even where the tune cache holds the shape */
};

typedef struct tags_plan_s *tags_plan;

/* Per-run statistics (optional). */
typedef struct {
    int max_iterations;        /* largest refinement iteration count (mixed) */
    int fallbacks;             /* samples re-solved in plain FP64 (mixed) */
    double max_backward_error; /* largest normwise backward error |b - W x| / (|W| |x|) of the last
                                  iterate whose residual the refinement formed: the one before
                                  the final correction (which shrinks the error further) */
    double seconds;            /* device time of the run */
    int split;                 /* split form used by the last pass (mixed; see tags_plan_set_split) */
} tags_run_stats;

/* Geometry and incidence are uploaded once. images may be NULL (no images).
 * max_batch = samples resident at once (0 = sized from free device memory). */
int tags_plan_create (tags_plan *plan, const Electrode *electrodes, const Electrode *images,
                      size_t num_electrodes, const double *nodes, size_t num_nodes,
                      int precision, size_t max_batch);

/* Solve ns samples: s[k], kappa[k] (soil complex conductivity sigma + s eps),
 * ie: ns x n injected node currents (sample-major; NULL = unit current at
 * inj_node). Outputs (any may be NULL): sol ns x (n + 2m) = [U; I_L; I_T],
 * info ns ints (0 ok, >0 singular pivot, <0 error). */
int tags_plan_run (tags_plan plan, const tags_cdouble *s, const tags_cdouble *kappa, double mur,
                   size_t ns, const tags_cdouble *ie, size_t inj_node, tags_cdouble *sol,
                   int *info, int flags, tags_run_stats *stats);

int tags_plan_destroy (tags_plan plan);

/* One grid of a many-grid run (tags_gpu_solve_batch): geometry, its samples
 * and injections as for tags_plan_create / tags_plan_run, and where its
 * solutions go (sol ns x (n + 2m) and info ns, either may be NULL). */
typedef struct {
    const Electrode *electrodes;
    const Electrode *images;           /* NULL: no images */
    size_t num_electrodes;
    const double *nodes;
    size_t num_nodes;
    const tags_cdouble *s;
    const tags_cdouble *kappa;
    size_t ns;
    const tags_cdouble *ie;            /* ns x n injected currents, or NULL: unit current at inj_node */
    size_t inj_node;
    tags_cdouble *sol;
    int *info;
} tags_grid_job;

/* No counterpart function in the reference: many grids x many Laplace samples
 * in one call (host buffers), on the calling thread's device: a grid batch
 * (tags_batch_create, one tags_batch_run, tags_batch_destroy). If the grids
 * do not fit in device memory together, a plan per grid runs from `workers`
 * host threads (0 = 4) instead. max_batch = samples resident per grid (0 =
 * min(ns, 256), reduced by the memory admission). Returns 0 or the first
 * error code of any grid. */
int tags_gpu_solve_batch (const tags_grid_job *jobs, size_t njobs, int precision, double mur, size_t max_batch,
                          int workers);

/* No counterpart in the reference (it loops over grids and samples with
 * OpenMP, examples/three_grids.c:286-443). A grid batch holds, for many grids
 * of uneven size, a plan per grid, device arrays for every grid's samples,
 * injections and solutions, and ONE executable CUDA graph in which each grid
 * is an independent branch: its passes in sequence (fill, assembly,
 * factorisation and, for TAGS_MIXED, the refinement loop as a conditional
 * while-node), so grids of different sizes run side by side. The samples
 * resident per grid (at most max_batch, 0 = 256) are admitted against 60 %
 * of the free device memory. Built once; every run reuses it. */
typedef struct tags_batch_s *tags_batch;
int tags_batch_create (tags_batch *batch, const tags_grid_job *jobs, size_t njobs, int precision, double mur,
                       size_t max_batch);
/* Solves every sample of every grid: copies the jobs' s, kappa (and ie) to
 * the device, launches the graph once, re-solves in plain FP64 the samples
 * whose refinement did not converge, and copies sol / info back. The jobs
 * must have the shapes (ns, m, n, injection form) the batch was built with.
 * stats: largest refinement count, fallbacks, largest backward error, and the
 * device time of the graph launch. */
int tags_batch_run (tags_batch batch, const tags_grid_job *jobs, size_t njobs, tags_run_stats *stats);
int tags_batch_destroy (tags_batch batch);

/* Passes in flight (1 = default, 2 or 3): with k > 1 the plan builds k - 1
 * twins of the same geometry and settings (k times the device memory), and a
 * run of several passes hands each pass to whichever pipeline frees up first,
 * each twin on its own stream from its own host thread, so that one pass's
 * latency-bound phases (diagonal blocks, triangular sweeps, refinement steps)
 * overlap another's dense work. The run's statistics cover all of them; its
 * device time spans all streams. Fewer pipelines later keep the twins' memory
 * until the plan is destroyed. */
int tags_plan_set_pipelines (tags_plan plan, int pipelines);

/* Passes as CUDA graphs (default on): each pass shape (samples in the pass,
 * mur, injection form) is captured once into an executable graph holding
 * the fill, the factorisation and, for TAGS_MIXED, a conditional while-node
 * that repeats the refinement step until the device-side stopping test
 * clears it; later passes of that shape are one graph launch. 0 = launch
 * the same kernels one by one (the host reads the stopping flag per step). */
int tags_plan_set_graphs (tags_plan plan, int enable);

/* Split form of the TAGS_MIXED tensor-core products: 3 = three bf16 pieces
 * per FP32 value (6 products per real product, FP32-level), 2 = two bf16
 * pieces (3 products, ~16 bits), 16 = two fp16 pieces of 2^8 x (3 products,
 * 22 bits; a value outside fp16's range makes the plan fall back to 3 and
 * solve that pass again). Default 16. */
int tags_plan_set_split (tags_plan plan, int pieces);

/* Panels of 128 columns per trailing update of the TAGS_MIXED factorisation
 * (1 .. 6; 0 = the default, 6): each group of that many panels updates its
 * own block columns left-looking (K = 128 .. 128 (panels - 1)) and then the
 * trailing matrix once with K = 128 x panels. tags_plan_tune picks among
 * 1, 2, 4 and 6. */
int tags_plan_set_panels (tags_plan plan, int panels);

/* Impedance model of the plan's passes: 2 (the reference's INTG_DOUBLE,
 * default) fills ZL/ZT with the double line integrals of e^{-gamma r}/r;
 * 4 (INTG_MHEM) uses the reference's mHEM examples' model: static potentials
 * (INTG_MHEM integrals, computed once here) times e^{-gamma rbar} of the
 * segments' midpoint distance, images with ref_l = 1 and ref_t
 * (examples/three_grids.c:335-350). The node potentials then equal those of
 * the examples' nodal admittance solve (Y_N is W_G's node Schur complement). */
int tags_plan_set_fill (tags_plan plan, int integration_type);

/* Result of tags_plan_tune: the configuration kept and its measured rate. */
typedef struct {
    int samples_per_pass;      /* samples factorised together (<= the plan's capacity) */
    int panels_per_update;     /* 128-column panels per trailing update (1, 2, 4 or 6; K = 128 x that) */
    int split;                 /* split form kept (TAGS_MIXED; 0 for TAGS_PLAIN_FP64) */
    double solves_per_second;  /* device rate of the kept configuration on the given samples */
    int candidates;            /* configurations timed */
} tags_tune_result;

/* Autotuner: times one pass for each candidate configuration (samples per
 * pass in powers of two up to the plan's capacity; for TAGS_MIXED also 1, 2,
 * 4 or 6 panels per trailing update and the fp16 or three-piece bf16 split) on
 * the first samples of s / kappa (ns >= 1; unit current at inj_node; flags as
 * in tags_plan_run) and keeps the fastest in the plan. Quadrature orders are
 * not tuned: they follow the fill's error model, so accuracy does not depend
 * on the tuner. out may be NULL. */
int tags_plan_tune (tags_plan plan, const tags_cdouble *s, const tags_cdouble *kappa, double mur, size_t ns,
                    size_t inj_node, int flags, tags_tune_result *out);

/* Autotuner cache file (process-wide; NULL or "" switches it off, the
 * default). With a cache set, tags_plan_tune first looks for the plan's key:
 * system size N, segments m, precision, impedance model, the samples it may
 * put in one pass (min(capacity, ns)), pipelines, pair setting, and the GPU
 * (name, SM count, compute capability). On a hit it applies the stored
 * configuration without timing anything (candidates = 0, solves_per_second
 * as stored); otherwise, or with TAGS_TUNE_REFRESH in flags, it times the
 * candidates and appends a line. The file is plain text, one line per timed
 * tune; the last line of a key wins. Returns TAGS_E_ARG if the file cannot be
 * opened for appending. */
int tags_gpu_set_tune_cache (const char *path);

/* ---- Part 3: solve without device allocation -------------------------------- */

/* No counterpart in the reference. For callers that may not allocate device
 * memory, e.g. code inside a larger GPU application that owns a fixed memory
 * pool, or code that must not allocate after start-up: the same solve as
 * solve_immittance on device buffers the caller owns. d_wg (N x N,
 * column-major, lower half read) is factorised in place and d_ie (N values) is
 * overwritten with [U; I_L; I_T]; N = n + 2m must not exceed
 * TAGS_NOALLOC_MAX_N. The solver's scratch is a fixed device array inside the
 * library (no cudaMalloc or cudaFree on any call); every GPU that loads the
 * library holds it until exit. The first call on a device looks the array up:
 * make that call before any stream capture. That address is kept for the
 * life of the process: after cudaDeviceReset on a device, this entry point
 * must not be called on that device again. All calls share the array, so
 * calls that overlap on the GPU race. stream may be NULL (default stream).
 * Returns 0, k > 0 when the k-th pivot is exactly zero (ie unchanged), or a
 * negative TAGS_E_* code (TAGS_E_ARG for a system above the limit). */
#define TAGS_NOALLOC_MAX_N 32768
int tags_solve_immittance_noalloc (tags_cdouble *d_wg, tags_cdouble *d_ie, size_t num_electrodes,
                                   size_t num_nodes, void *stream);

/* ---- Part 4: diagnostics -------------------------------------------------------- */

/* No counterpart in the reference. Stopping tolerance of the mixed form's
 * refinement: a sample stops once the error its corrections predict (four
 * times the last correction times their measured contraction) is below
 * tol |x|, or once a correction is below tol / 10 |x| (0 restores the default
 * 1e-9; at most 1e-3). The residual sees the impedance entries to ~1e-13, so
 * tol bounds the error against the FP64 solution; smaller values cost
 * refinement steps. */
int tags_plan_set_refine_tol (tags_plan plan, double tol);

/* No counterpart in the reference. How the mixed form's trailing updates use
 * the tensor cores. 0 (default): one SM per 128 x 128 tile (complex products
 * as 4 real ones). 1: clusters of two SMs (tcgen05.mma.cta_group::2, 256 x 128
 * products, each SM staging its own 128 rows of A and half of B). 2: clusters
 * of two SMs with the complex update as one real product of N = 256
 * ([Re | Im] = [Ar Ai] [[Br, -Bi], [Bi, Br]]^T, each SM staging its own 128
 * rows of A and its 128 B rows; the panel GEMM also writes the negated
 * imaginary planes); with three bf16 pieces this falls back to 1. Where the
 * device cannot host such clusters the single-SM kernel runs. */
int tags_plan_set_tc_pairs (tags_plan plan, int on);

/* No counterpart in the reference. The same switch for the diagnostic entry
 * points tags_debug_ldl and tags_debug_ldl_solve (process-wide). */
int tags_debug_tc_pairs (int on);

/* No counterpart in the reference. The tile list of a trailing update of M
 * rows (lower triangle of 128 x 128 tiles) whose rows and columns zlo .. zhi
 * are structurally zero: the tiles that do work, row by row, plus (planes)
 * the first-column tiles that only write the next panel's split planes, in
 * the band's rows too when planes_band; when no tile lies wholly in the band,
 * the full triangle, which the kernel walks then. Writes (I, J, planes only)
 * triples into out (up to cap) and returns the count. Host code, no device
 * work. */
int tags_debug_tri_tiles (int M, int zlo, int zhi, int planes, int planes_band, int *out, int cap);

/* No counterpart in the reference. Test hook (process-wide, for passes and
 * graphs built afterwards): how the mixed form's triangular solves run.
 * 0: block by block (two kernels per 128-row block and sweep); 1: one CTA per
 * sample with x in shared memory; 2, 4, 8: a cluster of that many CTAs per
 * sample, x spread over their shared memory; -1 (default): the larger of
 * the cluster sizes 4 and 2 with G x samples per pass <= SMs, else one CTA
 * per sample. Paths 1..8
 * need x in shared memory (N up to about 25000) and otherwise run block by
 * block. All form every sum in the same order and give identical results. */
int tags_debug_solve_path (int path);

/* No counterpart in the reference. Caps the refinement steps of the mixed
 * form's passes (1 .. 40; 0 restores the default 40). A sample that has not
 * met its stopping rule after that many steps is re-solved by the plain FP64
 * path (partial pivoting), as one whose refinement stops converging; the
 * run's stats count it in `fallbacks`. A cap of 1 sends every sample there
 * (the first correction is the whole solution), which tests that path. */
int tags_plan_set_max_steps (tags_plan plan, int steps);

/* No counterpart in the reference. The mixed form's impedance fill of ns
 * samples (1 <= ns <= the plan's batch; INTG_DOUBLE fill) on a mixed plan:
 * zl, zt (ns x m x m each, sample-major, column-major, both triangles)
 * receive the values the refinement's residual uses: the FP32 entries of
 * the regular pairs and, for pairs sharing an endpoint and the diagonal,
 * their FP64 value (FP32 part + stored rounding residue). */
int tags_debug_mixed_fill (tags_plan plan, const tags_cdouble *s, const tags_cdouble *kappa, double mur,
                           size_t ns, tags_cdouble *zl, tags_cdouble *zt);

/* No counterpart in the reference. Test hook: the wall-clock limit, in
 * nanoseconds, of each wait in the main loops of the tensor-core
 * factorisation kernels on the current device (ns <= 0 restores the default
 * 50 ms). When a wait runs out the kernel raises its error word, lets the
 * copies and products it issued finish (those waits keep the 50 ms limit),
 * frees its tensor memory and returns; the pass is then re-solved by the
 * plain FP64 path and tags_run_stats counts the fallbacks. Waits a few
 * microseconds long run out within a pass, which exercises that path.
 * Synchronises the device first. */
int tags_debug_tc_wait_limit (long long ns);

/* No counterpart in the reference. Factorises nb complex symmetric N x N
 * matrices (host, column-major, sample-major; lower half read) with the mixed
 * form's tensor-core LDL^T (FP32 storage, no pivoting; the products use
 * pieces = 2 or 3 bf16 pieces per real value, or pieces = 16: two fp16
 * pieces of 2^8 x) and returns L (strictly lower, unit diagonal implied) and
 * D (diagonal) in place, rounded from FP32. Returns 0, k > 0 for a zero
 * pivot, or a TAGS_E_* code (TAGS_E_NONFINITE: a value left the fp16 range). */
int tags_debug_ldl (tags_cdouble *a, int N, int nb, int pieces);

/* No counterpart in the reference. As tags_debug_ldl, then one solve
 * L D L^T x = b per matrix with the factors (no refinement); b (N x nb,
 * sample-major) is replaced by x, rounded from FP32. zl_m > 0 declares rows
 * and columns zl_m .. 2 zl_m - 1 structurally zero against columns 0 ..
 * zl_m - 1 (the ZL/ZT coupling of the immittance system), which the
 * factorisation and the solves skip. group: 128-column panels per trailing
 * update (1 .. 6). */
int tags_debug_ldl_solve (tags_cdouble *a, tags_cdouble *b, int N, int nb, int pieces, int zl_m, int group);

/* No counterpart in the reference. FP64 throughput of the current device, in
 * TFLOP/s: dfma from eight independent FMA chains per thread on the CUDA
 * cores, dmma from mma.sync m8n8k4 f64 on the FP64 tensor path (best of three
 * timed launches each). The plain form's roofline is reported against these. */
int tags_probe_fp64 (double *dfma_tflops, double *dmma_tflops);

/* Per-family kernel timing with CUDA events on the launching stream (0 = off,
 * the default). Enabling resets the counters. Families, in this order:
 * fill_fp64, fill_mixed, ldl_diag, ldl_panel_gemm, ldl_trailing_gemm,
 * ldl_solve, residual_fp64, build_fp32, lu_fp64_gemm, lu_fp64_other, fields. */
int tags_gpu_profile (int enable);
/* launches, device milliseconds, algorithmic flops and bytes of one family. */
int tags_gpu_profile_read (int family, long long *launches, double *ms, double *flops, double *bytes,
                           char *name, int name_len);

/* Number of CUDA kernel launches issued by this library since load. */
long long tags_gpu_launch_count (void);

/* Last error message of the calling thread ("" if none). */
const char *tags_gpu_last_error (void);

/* 0/1: suppress the reference-style messages printed on errors. */
void tags_gpu_set_quiet (int quiet);

/* No counterpart in the reference. Caps, process-wide, the free device memory
 * that plans and grid batches size themselves against (bytes; 0 = no cap).
 * Plans created afterwards take fewer samples per pass, or fail with
 * TAGS_E_NOMEM when not even one sample fits. */
int tags_gpu_set_memory_budget (unsigned long long bytes);

#ifdef __cplusplus
}
#endif

#endif /* TAGS_GPU_H_ */
