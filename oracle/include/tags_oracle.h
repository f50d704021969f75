/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * Restatement, in plain C, of the reference's per-Laplace-sample path
 * (pedrohnv/transient-analysis-grounding-systems): thin-wire impedance fill
 * with adaptive cubature, immittance assembly, Bunch-Kaufman solve (LAPACK
 * zsysv through oracle/lapack_shim.c), and the numerical Laplace transform
 * pair. Every function cites the reference file:line it follows. Only the
 * tests, the smoke check and the bench's CPU-baseline leg link this library;
 * the GPU product never does.
 */
#ifndef TAGS_ORACLE_H_
#define TAGS_ORACLE_H_

#include <complex.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same 88-byte layout as the reference's Electrode (src/electrode.h:33-45). */
typedef struct {
    double start_point[3];
    double end_point[3];
    double middle_point[3];
    double length;
    double radius;
} OracleElectrode;

/* Same field order as the reference's Grid (src/grid.h:35-52). */
typedef struct {
    unsigned int vertices_x, vertices_y;
    double length_x, length_y;
    unsigned int edge_segments_x, edge_segments_y;
    double radius, depth;
} OracleGrid;

enum { ORACLE_INTG_NONE = 1, ORACLE_INTG_DOUBLE = 2, ORACLE_INTG_SINGLE = 3, ORACLE_INTG_MHEM = 4 };
enum { ORACLE_FILTER_NONE = 0, ORACLE_FILTER_BLACKMAN, ORACLE_FILTER_HANNING,
       ORACLE_FILTER_LANCZOS, ORACLE_FILTER_RIESZ };

extern const double ORACLE_PI, ORACLE_TWO_PI, ORACLE_FOUR_PI, ORACLE_MU0, ORACLE_EPS0;

/* geometry (src/electrode.c:12-32, :103-127; src/auxiliary.c:24-50; src/grid.c:9-92) */
int oracle_populate_electrode (OracleElectrode *e, const double *a, const double *b, double radius);
int oracle_segment_electrode (OracleElectrode *e, double *nodes, size_t nseg,
                              const double *a, const double *b, double radius);
int oracle_linspace (double a, double b, size_t n, double *u);
int oracle_logspace (double a, double b, size_t n, double *u);
int oracle_number_segments (OracleGrid g);
int oracle_number_nodes (OracleGrid g);
int oracle_electrode_grid (OracleGrid g, OracleElectrode *e, double *nodes);
double oracle_vector_length (const double *a, const double *b);

/* soil (src/auxiliary.c:60-70) */
int oracle_alipio_soil (double _Complex *sigma, double _Complex *epsr, double sigma0,
                        double _Complex s, double h, double g, double eps_ratio);

/* impedance fill (src/electrode.c:176-431) */
double oracle_self_integral (const OracleElectrode *e);
int oracle_integral (const OracleElectrode *sender, const OracleElectrode *receiver,
                     double _Complex gamma, size_t max_eval, double req_abs, double req_rel,
                     int type, double result[2], double error[2]);
int oracle_calculate_impedances (double _Complex *zl, double _Complex *zt,
                                 const OracleElectrode *e, size_t m, double _Complex gamma,
                                 double _Complex s, double mur, double _Complex kappa,
                                 size_t max_eval, double req_abs, double req_rel, int type);
int oracle_impedances_images (double _Complex *zl, double _Complex *zt,
                              const OracleElectrode *e, const OracleElectrode *img, size_t m,
                              double _Complex gamma, double _Complex s, double mur,
                              double _Complex kappa, double _Complex ref_l, double _Complex ref_t,
                              size_t max_eval, double req_abs, double req_rel, int type);

/* immittance system (src/linalg.c:12-139) */
int oracle_fill_incidence_imm (double _Complex *wg, const OracleElectrode *e, size_t m,
                               const double *nodes, size_t n);
int oracle_fill_impedance_imm (double _Complex *wg, const double _Complex *zl,
                               const double _Complex *zt, size_t m, size_t n);
int oracle_solve_immittance (double _Complex *wg, double _Complex *ie, size_t m, size_t n);
int oracle_fill_incidence_adm (double _Complex *a, double _Complex *b, const OracleElectrode *e, size_t m,
                               const double *nodes, size_t n);
int oracle_calculate_yla_ytb (double _Complex *yla, double _Complex *ytb, double _Complex *zl,
                              double _Complex *zt, double _Complex *a, double _Complex *b, size_t m, size_t n);
int oracle_fill_impedance_adm2 (double _Complex *yn, double _Complex *yla, double _Complex *ytb,
                                double _Complex *a, double _Complex *b, size_t m, size_t n);
int oracle_fill_impedance_adm (double _Complex *yn, double _Complex *zl, double _Complex *zt,
                               double _Complex *a, double _Complex *b, size_t m, size_t n);
int oracle_solve_admittance (double _Complex *yn, double _Complex *ic, size_t n);
int oracle_mhem_impedances (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                            const double _Complex *potzl, const double _Complex *potzt,
                            const double _Complex *potzli, const double _Complex *potzti,
                            double _Complex s, double _Complex kappa, double mur,
                            double _Complex *zl, double _Complex *zt);
int oracle_mhem_sweep (const OracleElectrode *e, const OracleElectrode *img, size_t m, const double *nodes,
                       size_t n, const double _Complex *s, const double _Complex *kappa, size_t ns, double mur,
                       size_t inj_node, const double _Complex *inj, size_t max_eval, double req_abs,
                       double req_rel, int threads, double _Complex *sol, int *info);

/* numerical Laplace transform pair (src/auxiliary.c:239-336) */
int oracle_laplace_trans (const double *f, double _Complex *g, double _Complex *s,
                          double tmax, size_t nt);
int oracle_inv_laplace_trans (double *f, const double _Complex *g, const double _Complex *s,
                              double tmax, size_t nt, int filter);
double oracle_heidler (double t, double imax, double tau1, double tau2, double n);

/* Per-sample driver of the traditional-HEM immittance path, call stack as
 * the reference documents it (src/linalg.h:61-78 with the sample loop of
 * examples/three_grids.c:286-333): for every sample k,
 *   gamma = sqrt(s mu0 mur kappa), ref_t = (kappa - s eps0)/(kappa + s eps0),
 *   ref_l = 1; calculate_impedances + impedances_images (INTG_DOUBLE);
 *   fill_impedance_imm on a copy of the incidence-filled W_G; ie = [I_E;0;0]
 *   with I_E[inj_node] = inj[k]; solve_immittance.
 * Samples run in parallel over `threads` OpenMP threads (0 = all).
 * sol: ns x (n + 2m) complex, sample-major. info: ns ints. Returns 0, or the
 * incidence/integration error code of the set-up. */
int oracle_hem_sweep (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                      const double *nodes, size_t n, const double _Complex *s,
                      const double _Complex *kappa, size_t ns, double mur,
                      size_t inj_node, const double _Complex *inj,
                      size_t max_eval, double req_abs, double req_rel, int threads,
                      double _Complex *sol, int *info);

/* ZL/ZT (direct + images, lower triangles) for one sample. */
int oracle_hem_impedances (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                           double _Complex s, double _Complex kappa, double mur,
                           size_t max_eval, double req_abs, double req_rel, int type,
                           double _Complex *zl, double _Complex *zt);

/* Post-processing: potentials, fields and path voltage (src/electrode.c:434-668)
 * and the closed-form mHEM ground potential (examples/visacro57emc01.c:406-430). */
double _Complex oracle_electric_potential (const double *point, const OracleElectrode *e, size_t m,
                                           const double _Complex *it, double _Complex gamma,
                                           double _Complex kappa, size_t max_eval, double req_abs,
                                           double req_rel, int *failure);
int oracle_magnetic_potential (const double *point, const OracleElectrode *e, size_t m,
                               const double _Complex *il, double _Complex gamma, double mur,
                               size_t max_eval, double req_abs, double req_rel, double _Complex *va);
int oracle_electric_field (const double *point, const OracleElectrode *e, size_t m,
                           const double _Complex *il, const double _Complex *it,
                           double _Complex gamma, double _Complex s, double mur,
                           double _Complex kappa, size_t max_eval, double req_abs, double req_rel,
                           double _Complex *ve);
double _Complex oracle_voltage (const double *point1, const double *point2, const OracleElectrode *e,
                                size_t m, const double _Complex *il, const double _Complex *it,
                                double _Complex gamma, double _Complex s, double mur,
                                double _Complex kappa, size_t max_eval, double req_abs, double req_rel,
                                int *failure);
int oracle_gpd_mhem (const double *points, size_t np, const OracleElectrode *e, size_t m,
                     const double _Complex *it, size_t nrhs, double _Complex gamma,
                     double _Complex kappa, double _Complex *gpd);

/* LAPACK binding (oracle/lapack_shim.c) */
int tags_lapack_bind (const char *name, void *fn);
int tags_lapack_ready (void);

#ifdef __cplusplus
}
#endif

#endif /* TAGS_ORACLE_H_ */
