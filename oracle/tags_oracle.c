/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * Plain-C restatement of the reference's per-Laplace-sample path
 * (pedrohnv/transient-analysis-grounding-systems). Each function names the
 * reference file:line whose behaviour it follows, including the modelling
 * quirks the GPU path must reproduce:
 *   - the diagonal of ZL/ZT is the static closed form (no e^{-gamma r});
 *   - |cos(theta)| is used, so segment direction is ignored;
 *   - ZL = 0 for perpendicular pairs;
 *   - r < DBL_EPSILON in the double integrand is replaced by the radius;
 *   - images include k = i and are accumulated (+=) into the outputs;
 *   - solve_immittance caps the zsysv workspace at 100 entries.
 * The arithmetic follows the same expression order as the reference so that
 * both agree to rounding. Used only by tests, the smoke check and the bench's
 * CPU baseline; the GPU library never links it.
 */
#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "cubature.h"
#include "tags_dft.h"
#include "tags_oracle.h"

/* constants: src/auxiliary.c:17-21 */
const double ORACLE_PI = 3.1415926535897932384626433832795029;
const double ORACLE_TWO_PI = 6.283185307179586476925286766559;
const double ORACLE_FOUR_PI = 12.5663706143591729538505735331;
const double ORACLE_MU0 = 1.256637061435917e-6;
const double ORACLE_EPS0 = 8.854187817620e-12;

void tags_zsysv_ (char *uplo, int *n, int *nrhs, double _Complex *a, int *lda, int *ipiv,
                  double _Complex *b, int *ldb, double _Complex *work, int *lwork, int *info);

/* ---- points and geometry ------------------------------------------------ */

/* src/auxiliary.c:101-108 */
static bool equal_points_tol (const double *p1, const double *p2, double tol)
{
    for (int i = 0; i < 3; i++)
        if (fabs(p1[i] - p2[i]) > tol) return false;
    return true;
}

/* src/auxiliary.c:110-125 (sum of squared differences, then sqrt) */
double oracle_vector_length (const double *a, const double *b)
{
    double r = 0.0;
    for (int i = 0; i < 3; i++) r += pow(a[i] - b[i], 2.0);
    return sqrt(r);
}

/* src/electrode.c:12-32 */
int oracle_populate_electrode (OracleElectrode *e, const double *a, const double *b, double radius)
{
    if (equal_points_tol(a, b, DBL_EPSILON)) return 1;
    if (radius <= 0) return 2;
    e->radius = radius;
    e->length = oracle_vector_length(a, b);
    for (int i = 0; i < 3; i++) {
        e->start_point[i] = a[i];
        e->end_point[i] = b[i];
        e->middle_point[i] = (a[i] + b[i]) / 2.0;
    }
    return 0;
}

/* src/auxiliary.c:24-36: n points, last one pinned to b */
int oracle_linspace (double a, double b, size_t n, double *u)
{
    if (n < 2 || !u) return 1;
    double c = (b - a) / (n - 1);
    for (size_t i = 0; i < n - 1; ++i) u[i] = a + i * c;
    u[n - 1] = b;
    return 0;
}

/* src/auxiliary.c:38-50 */
int oracle_logspace (double a, double b, size_t n, double *u)
{
    if (n < 2 || !u) return 1;
    double c = (b - a) / (n - 1);
    for (size_t i = 0; i < n - 1; ++i) u[i] = pow(10.0, a + i * c);
    u[n - 1] = pow(10.0, b);
    return 0;
}

/* src/electrode.c:103-127 */
int oracle_segment_electrode (OracleElectrode *e, double *nodes, size_t nseg,
                              const double *a, const double *b, double radius)
{
    if (nseg < 1) return 1;
    size_t nn = nseg + 1;
    double *xyz = malloc(3 * nn * sizeof(double));
    if (!xyz) return 1;
    for (int d = 0; d < 3; d++) oracle_linspace(a[d], b[d], nn, xyz + d * nn);
    for (size_t i = 0; i < nn; i++)
        for (int d = 0; d < 3; d++) nodes[3 * i + d] = xyz[d * nn + i];
    free(xyz);
    for (size_t i = 0; i < nseg; i++)
        oracle_populate_electrode(&e[i], nodes + 3 * i, nodes + 3 * i + 3, radius);
    return 0;
}

/* src/grid.c:9-17 */
int oracle_number_segments (OracleGrid g)
{
    return (int) (g.edge_segments_x * g.vertices_y * (g.vertices_x - 1)
                  + g.edge_segments_y * g.vertices_x * (g.vertices_y - 1));
}

/* src/grid.c:19-27 */
int oracle_number_nodes (OracleGrid g)
{
    return (int) (g.vertices_x * g.vertices_y
                  + g.vertices_x * (g.vertices_y - 1) * (g.edge_segments_y - 1)
                  + g.vertices_y * (g.vertices_x - 1) * (g.edge_segments_x - 1));
}

/* src/grid.c:29-92: x-directed conductors row by row first (nodes: the row's
 * first vertex, then every segment end), then y-directed conductors column by
 * column (nodes: interior segment ends only). */
int oracle_electrode_grid (OracleGrid g, OracleElectrode *e, double *nodes)
{
    const size_t nx = g.edge_segments_x, vx = g.vertices_x;
    const size_t ny = g.edge_segments_y, vy = g.vertices_y;
    const double lx = g.length_x / (nx * (vx - 1));
    const double ly = g.length_y / (ny * (vy - 1));
    double a[3] = {0.0, 0.0, g.depth}, b[3] = {0.0, 0.0, g.depth};
    size_t ed = 0, nd = 0;
    for (size_t row = 0; row < vy; row++) {
        for (size_t span = 0; span + 1 < vx; span++) {
            for (size_t k = 0; k < nx; k++) {
                a[0] = lx * (span * nx + k);
                a[1] = ly * ny * row;
                b[0] = a[0] + lx;
                b[1] = a[1];
                oracle_populate_electrode(&e[ed++], a, b, g.radius);
                if (span == 0 && k == 0) {
                    memcpy(nodes + 3 * nd, a, 3 * sizeof(double));
                    nd++;
                }
                memcpy(nodes + 3 * nd, b, 3 * sizeof(double));
                nd++;
            }
        }
    }
    for (size_t col = 0; col < vx; col++) {
        for (size_t span = 0; span + 1 < vy; span++) {
            for (size_t k = 0; k < ny; k++) {
                a[0] = lx * nx * col;
                a[1] = ly * (span * ny + k);
                b[0] = a[0];
                b[1] = a[1] + ly;
                oracle_populate_electrode(&e[ed++], a, b, g.radius);
                if (k + 1 < ny) {
                    memcpy(nodes + 3 * nd, b, 3 * sizeof(double));
                    nd++;
                }
            }
        }
    }
    return 0;
}

/* ---- soil ---------------------------------------------------------------- */

/* src/auxiliary.c:60-70 (Alipio-Visacro frequency-dependent soil) */
int oracle_alipio_soil (double _Complex *sigma, double _Complex *epsr, double sigma0,
                        double _Complex s, double h, double g, double eps_ratio)
{
    double _Complex f = s / (ORACLE_TWO_PI * I);
    *sigma = (sigma0 + sigma0 * h * cpow(f / 1e6, g));
    double t = tan(ORACLE_PI * g / 2) / (ORACLE_TWO_PI * ORACLE_EPS0 * pow(1e6, g));
    *epsr = eps_ratio + t * sigma0 * h * cpow(f, g - 1.0);
    return 0;
}

/* ---- integrands and quadrature driver ------------------------------------ */

typedef struct {
    const OracleElectrode *sender, *receiver;
    double _Complex gamma;
} pair_data;

/* src/electrode.c:176-197: e^{-gamma r}/r, t[0] on the receiver, t[1] on the
 * sender; r below DBL_EPSILON is replaced by the receiver radius. */
static int integrand_double (unsigned ndim, const double *t, void *aux, unsigned fdim, double *fval)
{
    (void) ndim; (void) fdim;
    const pair_data *p = aux;
    double pr[3], ps[3];
    for (int i = 0; i < 3; i++) {
        pr[i] = t[0] * (p->receiver->end_point[i] - p->receiver->start_point[i])
              + p->receiver->start_point[i];
        ps[i] = t[1] * (p->sender->end_point[i] - p->sender->start_point[i])
              + p->sender->start_point[i];
    }
    double r = oracle_vector_length(ps, pr);
    if (r < DBL_EPSILON) r = p->receiver->radius;
    double _Complex eg = cexp(-p->gamma * r);
    fval[0] = creal(eg) / r;
    fval[1] = cimag(eg) / r;
    return 0;
}

/* src/electrode.c:199-218: receiver point fixed at its middle; r clamped to
 * DBL_EPSILON. */
static int integrand_single (unsigned ndim, const double *t, void *aux, unsigned fdim, double *fval)
{
    (void) ndim; (void) fdim;
    const pair_data *p = aux;
    double ps[3];
    for (int i = 0; i < 3; i++)
        ps[i] = t[0] * (p->sender->end_point[i] - p->sender->start_point[i])
              + p->sender->start_point[i];
    double r = oracle_vector_length(ps, p->receiver->middle_point);
    if (r < DBL_EPSILON) r = DBL_EPSILON;
    double _Complex eg = cexp(-p->gamma * r);
    fval[0] = creal(eg) / r;
    fval[1] = cimag(eg) / r;
    return 0;
}

/* src/electrode.c:220-236: closed-form integral of 1/r over the sender seen
 * from a point of the receiver, log((r1 + r2 + Ls) / (r1 + r2 - Ls)). */
static int integrand_logn (unsigned ndim, const double *t, void *aux, unsigned fdim, double *fval)
{
    (void) ndim; (void) fdim;
    const pair_data *p = aux;
    double pr[3];
    for (int i = 0; i < 3; i++)
        pr[i] = t[0] * (p->receiver->end_point[i] - p->receiver->start_point[i])
              + p->receiver->start_point[i];
    double r1 = oracle_vector_length(pr, p->sender->start_point);
    double r2 = oracle_vector_length(pr, p->sender->end_point);
    double nf = (r1 + r2 + p->sender->length) / (r1 + r2 - p->sender->length);
    fval[0] = log(nf);
    return 0;
}

/* src/electrode.c:238-245 */
double oracle_self_integral (const OracleElectrode *e)
{
    double ls = e->length;
    double k1 = e->radius / ls;
    double k2 = sqrt(1.0 + k1 * k1);
    return (2.0 * ls * (log((k2 + 1.0) / k1) - k2 + k1));
}

/* src/electrode.c:247-302: integral over [0,1]^d scaled by the lengths. */
int oracle_integral (const OracleElectrode *sender, const OracleElectrode *receiver,
                     double _Complex gamma, size_t max_eval, double req_abs, double req_rel,
                     int type, double result[2], double error[2])
{
    pair_data aux = {sender, receiver, gamma};
    const double tmin[2] = {0.0, 0.0}, tmax[2] = {1.0, 1.0};
    int failure = -1;
    result[0] = result[1] = 0.0;
    error[0] = error[1] = 0.0;
    switch (type) {
    case ORACLE_INTG_NONE:
        result[0] = oracle_vector_length(sender->middle_point, receiver->middle_point);
        failure = 0;
        break;
    case ORACLE_INTG_DOUBLE:
        failure = hcubature(2, integrand_double, &aux, 2, tmin, tmax, max_eval,
                            req_abs, req_rel, ERROR_PAIRED, result, error);
        result[0] *= receiver->length * sender->length;
        result[1] *= receiver->length * sender->length;
        break;
    case ORACLE_INTG_SINGLE:
        failure = hcubature(2, integrand_single, &aux, 1, tmin, tmax, max_eval,
                            req_abs, req_rel, ERROR_PAIRED, result, error);
        result[0] *= sender->length;
        result[1] *= sender->length;
        break;
    case ORACLE_INTG_MHEM:
        failure = hcubature(1, integrand_logn, &aux, 1, tmin, tmax, max_eval,
                            req_abs, req_rel, ERROR_INDIVIDUAL, result, error);
        result[0] *= receiver->length;
        break;
    default:
        failure = -10;
        break;
    }
    return failure;
}

/* src/electrode.c:304-377: lower triangle (zl[i*m + k], k >= i). */
int oracle_calculate_impedances (double _Complex *zl, double _Complex *zt,
                                 const OracleElectrode *e, size_t m, double _Complex gamma,
                                 double _Complex s, double mur, double _Complex kappa,
                                 size_t max_eval, double req_abs, double req_rel, int type)
{
    double result[2], error[2];
    double _Complex iwu_4pi, one_4pik;
    if (type == ORACLE_INTG_MHEM || type == ORACLE_INTG_NONE) {
        iwu_4pi = 1.0;
        one_4pik = 1.0;
    } else {
        iwu_4pi = s * mur * ORACLE_MU0 / (ORACLE_FOUR_PI);
        one_4pik = 1.0 / (ORACLE_FOUR_PI * kappa);
    }
    for (size_t i = 0; i < m; i++) {
        double ls = e[i].length, d1[3];
        double _Complex intg = oracle_self_integral(&e[i]);
        zl[i * m + i] = iwu_4pi * intg;
        zt[i * m + i] = one_4pik / (ls * ls) * intg;
        for (int c = 0; c < 3; c++) d1[c] = e[i].end_point[c] - e[i].start_point[c];
        for (size_t k = i + 1; k < m; k++) {
            double lr = e[k].length, cost = 0.0;
            for (int c = 0; c < 3; c++) cost += d1[c] * (e[k].end_point[c] - e[k].start_point[c]);
            cost = fabs(cost);
            int failure = oracle_integral(&e[i], &e[k], gamma, max_eval, req_abs, req_rel,
                                          type, result, error);
            if (failure != 0) return failure;
            intg = result[0] + I * result[1];
            zt[i * m + k] = one_4pik / (ls * lr) * intg;
            if (cost < DBL_EPSILON) {
                zl[i * m + k] = 0.0;
            } else {
                cost = cost / (ls * lr);
                zl[i * m + k] = iwu_4pi * intg * cost;
            }
        }
    }
    return 0;
}

/* src/electrode.c:379-431: adds image couplings (k >= i, diagonal included). */
int oracle_impedances_images (double _Complex *zl, double _Complex *zt,
                              const OracleElectrode *e, const OracleElectrode *img, size_t m,
                              double _Complex gamma, double _Complex s, double mur,
                              double _Complex kappa, double _Complex ref_l, double _Complex ref_t,
                              size_t max_eval, double req_abs, double req_rel, int type)
{
    double result[2], error[2];
    double _Complex iwu_4pi, one_4pik;
    if (type == ORACLE_INTG_MHEM || type == ORACLE_INTG_NONE) {
        iwu_4pi = 1.0;
        one_4pik = 1.0;
    } else {
        iwu_4pi = ref_l * s * mur * ORACLE_MU0 / (ORACLE_FOUR_PI);
        one_4pik = ref_t / (ORACLE_FOUR_PI * kappa);
    }
    for (size_t i = 0; i < m; i++) {
        double ls = e[i].length, d1[3];
        for (int c = 0; c < 3; c++) d1[c] = e[i].end_point[c] - e[i].start_point[c];
        for (size_t k = i; k < m; k++) {
            double lr = img[k].length, cost = 0.0;
            for (int c = 0; c < 3; c++) cost += d1[c] * (img[k].end_point[c] - img[k].start_point[c]);
            cost = fabs(cost);
            int failure = oracle_integral(&e[i], &img[k], gamma, max_eval, req_abs, req_rel,
                                          type, result, error);
            if (failure != 0) return failure;
            double _Complex intg = result[0] + I * result[1];
            zt[i * m + k] += one_4pik / (ls * lr) * intg;
            if (cost > DBL_EPSILON) {
                cost = cost / (ls * lr);
                zl[i * m + k] += iwu_4pi * intg * cost;
            }
        }
    }
    return 0;
}

/* ---- immittance system --------------------------------------------------- */

/* src/linalg.c:12-86: A (+1 start, -1 end), B (0.5) and their transposes in
 * W_G (leading dimension n + 2m); node matching with tolerance 1e-5; returns 1
 * at the first node without incidence, -sum(A) or sum(B) - m on a bad
 * checksum. */
int oracle_fill_incidence_imm (double _Complex *wg, const OracleElectrode *e, size_t m,
                               const double *nodes, size_t n)
{
    const size_t ld = 2 * m + n;
    const double tol = 1e-5;
    long int suma = 0;
    double sumb = 0.0;
    for (size_t nd = 0; nd < n; nd++) {
        bool none = true;
        for (size_t k = 0; k < m; k++) {
            int cond = 0;
            if (equal_points_tol(e[k].start_point, nodes + nd * 3, tol)) cond = 1;
            else if (equal_points_tol(e[k].end_point, nodes + nd * 3, tol)) cond = 2;
            size_t a = (k + n) + ld * nd;
            size_t b = (k + n + m) + ld * nd;
            size_t c = nd + ld * (k + n);
            size_t d = nd + ld * (k + n + m);
            double av = (cond == 1) ? 1.0 : (cond == 2) ? -1.0 : 0.0;
            double bv = cond ? 0.5 : 0.0;
            wg[a] = av;
            wg[b] = bv;
            wg[c] = av;
            wg[d] = bv;
            suma += (long int) creal(wg[a]);
            sumb += creal(wg[b]);
            if (cond) none = false;
        }
        if (none) return 1;
    }
    if (suma != 0) return (int) -suma;
    if (sumb != (double) m) return (int) (sumb - (double) m);
    return 0;
}

/* src/linalg.c:88-110: -ZL and -ZT (whole m x m blocks as stored), zero
 * off-diagonal blocks and a zero Y_E. */
int oracle_fill_impedance_imm (double _Complex *wg, const double _Complex *zl,
                               const double _Complex *zt, size_t m, size_t n)
{
    const size_t ld = n + 2 * m;
    for (size_t k = 0; k < m; k++) {
        for (size_t i = 0; i < m; i++) {
            wg[(i + n) + ld * (k + n)] = -zl[i + m * k];
            wg[(i + n) + ld * (k + n + m)] = 0.0;
            wg[(i + n + m) + ld * (k + n)] = 0.0;
            wg[(i + n + m) + ld * (k + n + m)] = -zt[i + m * k];
        }
    }
    for (size_t k = 0; k < n; k++)
        for (size_t i = 0; i < n; i++) wg[i + ld * k] = 0.0;
    return 0;
}

/* src/linalg.c:112-139: zsysv('L') with the workspace capped at 100 entries
 * (which makes LAPACK fall back to its unblocked factorisation for large n). */
int oracle_solve_immittance (double _Complex *wg, double _Complex *ie, size_t m, size_t n)
{
    int nn = (int) (m * 2 + n);
    int *ipiv = malloc((nn > 0 ? nn : 1) * sizeof(int));
    double _Complex *work = malloc(100 * sizeof(double _Complex));
    if (!ipiv || !work) { free(ipiv); free(work); return -1000; }
    int info = 0, nrhs = 1, lwmax = 100, lwork = -1;
    char uplo = 'L';
    tags_zsysv_(&uplo, &nn, &nrhs, wg, &nn, ipiv, ie, &nn, work, &lwork, &info);
    lwork = (int) creal(work[0]);
    if (lwork > lwmax) lwork = lwmax;
    if (lwork < 1) lwork = 1;
    tags_zsysv_(&uplo, &nn, &nrhs, wg, &nn, ipiv, ie, &nn, work, &lwork, &info);
    free(work);
    free(ipiv);
    return info;
}

/* ---- nodal admittance formulation (mHEM examples) -------------------------- */

void tags_zsytrf_ (char *uplo, int *n, double _Complex *a, int *lda, int *ipiv, double _Complex *work,
                   int *lwork, int *info);
void tags_zsytri_ (char *uplo, int *n, double _Complex *a, int *lda, int *ipiv, double _Complex *work,
                   int *info);
void tags_zsymm_ (char *side, char *uplo, int *m, int *n, double _Complex *alpha, double _Complex *a, int *lda,
                  double _Complex *b, int *ldb, double _Complex *beta, double _Complex *c, int *ldc);
void tags_zgemm_ (char *ta, char *tb, int *m, int *n, int *k, double _Complex *alpha, double _Complex *a,
                  int *lda, double _Complex *b, int *ldb, double _Complex *beta, double _Complex *c, int *ldc);

/* src/linalg.c:142-204: A (+1 start, -1 end) and B (0.5) as dense m x n
 * column-major arrays (element (k, node) at k + m * node), the same node
 * matching and checksums as the immittance version. */
int oracle_fill_incidence_adm (double _Complex *a, double _Complex *b, const OracleElectrode *e, size_t m,
                               const double *nodes, size_t n)
{
    const double tol = 1e-5;
    long int suma = 0;
    double sumb = 0.0;
    for (size_t nd = 0; nd < n; nd++) {
        bool none = true;
        for (size_t k = 0; k < m; k++) {
            int cond = 0;
            if (equal_points_tol(e[k].start_point, nodes + nd * 3, tol)) cond = 1;
            else if (equal_points_tol(e[k].end_point, nodes + nd * 3, tol)) cond = 2;
            size_t pos = m * nd + k;
            /* the reference's write order: b before a at a match, so that
             * a == b (documented in src/linalg.h:90) leaves A */
            if (cond == 1) { b[pos] = 0.5; a[pos] = 1.0; }
            else if (cond == 2) { b[pos] = 0.5; a[pos] = -1.0; }
            else { a[pos] = 0.0; b[pos] = 0.0; }
            if (cond) none = false;
            suma += (long int) creal(a[pos]);
            sumb += creal(b[pos]);
        }
        if (none) return 1;
    }
    if (suma != 0) return (int) -suma;
    if (sumb != (double) m) return (int) (sumb - (double) m);
    return 0;
}

/* inv(Z) in place (lower triangle) by zsytrf + zsytri with the queried
 * workspace, as src/linalg.c:226-237 and :278-289. */
static int sym_inverse (double _Complex *z, int ne, int *ipiv)
{
    char uplo = 'L';
    int lwork = -1, info = 0;
    double _Complex q;
    tags_zsytrf_(&uplo, &ne, z, &ne, ipiv, &q, &lwork, &info);
    if (info != 0) return info;
    lwork = (int) creal(q);
    if (lwork < 1) lwork = 1;
    double _Complex *work = malloc(lwork * sizeof(double _Complex));
    if (!work) return -1000;
    tags_zsytrf_(&uplo, &ne, z, &ne, ipiv, work, &lwork, &info);
    if (info == 0) tags_zsytri_(&uplo, &ne, z, &ne, ipiv, work, &info);
    free(work);
    return info;
}

/* src/linalg.c:261-300: yla = inv(ZL) A, ytb = inv(ZT) B (zsymm on the lower
 * triangles); ZL and ZT are overwritten by their inverses. */
int oracle_calculate_yla_ytb (double _Complex *yla, double _Complex *ytb, double _Complex *zl,
                              double _Complex *zt, double _Complex *a, double _Complex *b, size_t m, size_t n)
{
    int ne = (int) m, nn = (int) n;
    int *ipiv = malloc((m > 0 ? m : 1) * sizeof(int));
    if (!ipiv) return -1000;
    int info = sym_inverse(zl, ne, ipiv);
    if (info == 0) info = sym_inverse(zt, ne, ipiv);
    if (info == 0) {
        char side = 'L', uplo = 'L';
        double _Complex one = 1.0, zero = 0.0;
        tags_zsymm_(&side, &uplo, &ne, &nn, &one, zl, &ne, a, &ne, &zero, yla, &ne);
        tags_zsymm_(&side, &uplo, &ne, &nn, &one, zt, &ne, b, &ne, &zero, ytb, &ne);
    }
    free(ipiv);
    return info;
}

/* src/linalg.c:302-325: yn = A^T yla + B^T ytb (n x n). */
int oracle_fill_impedance_adm2 (double _Complex *yn, double _Complex *yla, double _Complex *ytb,
                                double _Complex *a, double _Complex *b, size_t m, size_t n)
{
    int ne = (int) m, nn = (int) n;
    char notrans = 'N', trans = 'T';
    double _Complex one = 1.0, zero = 0.0;
    tags_zgemm_(&trans, &notrans, &nn, &nn, &ne, &one, a, &ne, yla, &ne, &zero, yn, &nn);
    tags_zgemm_(&trans, &notrans, &nn, &nn, &ne, &one, b, &ne, ytb, &ne, &one, yn, &nn);
    return 0;
}

/* src/linalg.c:206-259: yn = A^T inv(ZL) A + B^T inv(ZT) B in one call. */
int oracle_fill_impedance_adm (double _Complex *yn, double _Complex *zl, double _Complex *zt,
                               double _Complex *a, double _Complex *b, size_t m, size_t n)
{
    double _Complex *c1 = malloc((m * n > 0 ? m * n : 1) * sizeof(double _Complex));
    double _Complex *c2 = malloc((m * n > 0 ? m * n : 1) * sizeof(double _Complex));
    if (!c1 || !c2) { free(c1); free(c2); return -1000; }
    int info = oracle_calculate_yla_ytb(c1, c2, zl, zt, a, b, m, n);
    if (info == 0) oracle_fill_impedance_adm2(yn, c1, c2, a, b, m, n);
    free(c1);
    free(c2);
    return info;
}

/* src/linalg.c:327-350: zsysv('L') on YN with the queried workspace. */
int oracle_solve_admittance (double _Complex *yn, double _Complex *ic, size_t n)
{
    int nn = (int) n, nrhs = 1, info = 0, lwork = -1;
    char uplo = 'L';
    int *ipiv = malloc((n > 0 ? n : 1) * sizeof(int));
    double _Complex q;
    if (!ipiv) return -1000;
    tags_zsysv_(&uplo, &nn, &nrhs, yn, &nn, ipiv, ic, &nn, &q, &lwork, &info);
    lwork = (int) creal(q);
    if (lwork < 1) lwork = 1;
    double _Complex *work = malloc(lwork * sizeof(double _Complex));
    if (!work) { free(ipiv); return -1000; }
    tags_zsysv_(&uplo, &nn, &nrhs, yn, &nn, ipiv, ic, &nn, work, &lwork, &info);
    free(work);
    free(ipiv);
    return info;
}

/* ---- numerical Laplace transform ----------------------------------------- */

/* src/auxiliary.c:239-263: s_k = c + j k dw with c = ln(nt^2)/tmax,
 * g = r2c(f(t_k) dt e^{-c t_k}). */
int oracle_laplace_trans (const double *f, double _Complex *g, double _Complex *s,
                          double tmax, size_t nt)
{
    size_t ns = nt / 2 + 1;
    double *in = malloc(nt * sizeof(double));
    if (!in) return 1;
    double c = log(pow(nt, 2.0)) / tmax;
    double dt = tmax / (nt - 1);
    double dw = ORACLE_TWO_PI / tmax;
    for (size_t k = 0; k < ns; k++) s[k] = c + I * dw * k;
    for (size_t k = 0; k < nt; k++) in[k] = f[k] * dt * exp(-c * k * dt);
    int err = tags_dft_r2c((long) nt, in, 1, g, 1);
    free(in);
    return err;
}

/* src/auxiliary.c:265-329: windowed c2r, then f(t_k) = y_k e^{c t_k}/(nt dt). */
int oracle_inv_laplace_trans (double *f, const double _Complex *g, const double _Complex *s,
                              double tmax, size_t nt, int filter)
{
    size_t ns = nt / 2 + 1;
    double _Complex *in = malloc(ns * sizeof(double _Complex));
    double *out = malloc(nt * sizeof(double));
    if (!in || !out) { free(in); free(out); return 1; }
    double dt = tmax / (nt - 1);
    double omega = cimag(s[ns - 1]);
    for (size_t k = 0; k < ns; k++) {
        double w = cimag(s[k]), sigma = 1.0, alpha;
        switch (filter) {
        case ORACLE_FILTER_BLACKMAN:
            alpha = ORACLE_PI * w / omega;
            sigma = 0.42 + 0.5 * cos(alpha) + 0.08 * cos(2 * alpha);
            break;
        case ORACLE_FILTER_HANNING:
            sigma = (1 + cos(ORACLE_PI * w / omega)) / 2;
            break;
        case ORACLE_FILTER_LANCZOS:
            alpha = ORACLE_PI * w / omega;
            sigma = sin(alpha) / alpha;
            break;
        case ORACLE_FILTER_RIESZ:
            sigma = 1.0 - pow(fabs(w / omega), 2.0);
            break;
        default:
            break;
        }
        in[k] = (filter >= ORACLE_FILTER_BLACKMAN && filter <= ORACLE_FILTER_RIESZ)
              ? sigma * g[k] : g[k];
    }
    int err = tags_dft_c2r((long) nt, in, 1, out, 1);
    double c = creal(s[0]);
    for (size_t k = 0; k < nt; k++) f[k] = out[k] * exp(c * k * dt) / (nt * dt);
    free(in);
    free(out);
    return err;
}

/* src/auxiliary.c:331-336 */
double oracle_heidler (double t, double imax, double tau1, double tau2, double n)
{
    double xi = exp(-(tau1 / tau2) * pow((n * tau2 / tau1), (1.0 / n)));
    double tt1n = pow(t / tau1, n);
    return imax / xi * tt1n / (1 + tt1n) * exp(-t / tau2);
}

/* ---- per-sample drivers -------------------------------------------------- */

/* Per-sample medium terms, examples/three_grids.c:326-333. */
static void medium (double _Complex s, double _Complex kappa, double mur,
                    double _Complex *gamma, double _Complex *ref_t)
{
    *gamma = csqrt(s * mur * ORACLE_MU0 * kappa);
    *ref_t = (kappa - s * ORACLE_EPS0) / (kappa + s * ORACLE_EPS0);
}

int oracle_hem_impedances (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                           double _Complex s, double _Complex kappa, double mur,
                           size_t max_eval, double req_abs, double req_rel, int type,
                           double _Complex *zl, double _Complex *zt)
{
    double _Complex gamma, ref_t;
    medium(s, kappa, mur, &gamma, &ref_t);
    int err = oracle_calculate_impedances(zl, zt, e, m, gamma, s, mur, kappa,
                                          max_eval, req_abs, req_rel, type);
    if (err) return err;
    if (img)
        err = oracle_impedances_images(zl, zt, e, img, m, gamma, s, mur, kappa, 1.0, ref_t,
                                       max_eval, req_abs, req_rel, type);
    return err;
}

/* mHEM per-sample impedances, examples/three_grids.c:335-350: the static
 * potentials (INTG_MHEM integrals, computed once) times e^{-gamma rbar} of
 * the segments' midpoint distance, images with ref_l = 1 and ref_t, scaled by
 * s mur MU0 / (4 pi) and 1 / (4 pi kappa); lower triangle (k >= i) written. */
int oracle_mhem_impedances (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                            const double _Complex *potzl, const double _Complex *potzt,
                            const double _Complex *potzli, const double _Complex *potzti,
                            double _Complex s, double _Complex kappa, double mur,
                            double _Complex *zl, double _Complex *zt)
{
    double _Complex gamma, ref_t;
    medium(s, kappa, mur, &gamma, &ref_t);
    const double _Complex ref_l = 1.0;
    const double _Complex iwu_4pi = s * mur * ORACLE_MU0 / ORACLE_FOUR_PI;
    const double _Complex one_4pik = 1.0 / (ORACLE_FOUR_PI * kappa);
    for (size_t i = 0; i < m; i++) {
        for (size_t k = i; k < m; k++) {
            double rbar = oracle_vector_length(e[k].middle_point, e[i].middle_point);
            double _Complex exp_gr = cexp(-gamma * rbar);
            zl[i * m + k] = exp_gr * potzl[i * m + k];
            zt[i * m + k] = exp_gr * potzt[i * m + k];
            rbar = oracle_vector_length(e[k].middle_point, img[i].middle_point);
            exp_gr = cexp(-gamma * rbar);
            zl[i * m + k] += ref_l * exp_gr * potzli[i * m + k];
            zt[i * m + k] += ref_t * exp_gr * potzti[i * m + k];
            zl[i * m + k] *= iwu_4pi;
            zt[i * m + k] *= one_4pik;
        }
    }
    return 0;
}

/* The mHEM + nodal-admittance sample loop of examples/three_grids.c:270-392:
 * incidence and static potentials once, then per sample the mHEM rescale,
 * yla/ytb, YN and zsysv; sol (ns x n) receives the node potentials for the
 * injection inj[k] at inj_node. */
int oracle_mhem_sweep (const OracleElectrode *e, const OracleElectrode *img, size_t m, const double *nodes,
                       size_t n, const double _Complex *s, const double _Complex *kappa, size_t ns, double mur,
                       size_t inj_node, const double _Complex *inj, size_t max_eval, double req_abs,
                       double req_rel, int threads, double _Complex *sol, int *info)
{
    double _Complex *a = calloc(m * n, sizeof(double _Complex));
    double _Complex *b = calloc(m * n, sizeof(double _Complex));
    double _Complex *pl = calloc(m * m, sizeof(double _Complex));
    double _Complex *pt = calloc(m * m, sizeof(double _Complex));
    double _Complex *pli = calloc(m * m, sizeof(double _Complex));
    double _Complex *pti = calloc(m * m, sizeof(double _Complex));
    int err = (!a || !b || !pl || !pt || !pli || !pti) ? -1000 : 0;
    if (!err) err = oracle_fill_incidence_adm(a, b, e, m, nodes, n);
    if (!err) err = oracle_calculate_impedances(pl, pt, e, m, 0.0, 0.0, 0.0, 0.0, max_eval, req_abs, req_rel,
                                                ORACLE_INTG_MHEM);
    if (!err) err = oracle_impedances_images(pli, pti, e, img, m, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, max_eval,
                                             req_abs, req_rel, ORACLE_INTG_MHEM);
    int setup_err = err;
    if (!err) {
#ifdef _OPENMP
        int nthr = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr)
#else
        (void) threads;
#endif
        {
            double _Complex *zl = calloc(m * m, sizeof(double _Complex));
            double _Complex *zt = calloc(m * m, sizeof(double _Complex));
            double _Complex *yla = malloc(m * n * sizeof(double _Complex));
            double _Complex *ytb = malloc(m * n * sizeof(double _Complex));
            double _Complex *yn = malloc(n * n * sizeof(double _Complex));
            bool ok = zl && zt && yla && ytb && yn;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (size_t k = 0; k < ns; k++) {
                if (!ok) { info[k] = -1000; continue; }
                oracle_mhem_impedances(e, img, m, pl, pt, pli, pti, s[k], kappa[k], mur, zl, zt);
                int ierr = oracle_calculate_yla_ytb(yla, ytb, zl, zt, a, b, m, n);
                if (ierr) { info[k] = ierr; continue; }
                oracle_fill_impedance_adm2(yn, yla, ytb, a, b, m, n);
                double _Complex *x = sol + k * n;
                for (size_t q = 0; q < n; q++) x[q] = 0.0;
                x[inj_node] = inj[k];
                info[k] = oracle_solve_admittance(yn, x, n);
            }
            free(zl);
            free(zt);
            free(yla);
            free(ytb);
            free(yn);
        }
    }
    free(a);
    free(b);
    free(pl);
    free(pt);
    free(pli);
    free(pti);
    return setup_err;
}

int oracle_hem_sweep (const OracleElectrode *e, const OracleElectrode *img, size_t m,
                      const double *nodes, size_t n, const double _Complex *s,
                      const double _Complex *kappa, size_t ns, double mur,
                      size_t inj_node, const double _Complex *inj,
                      size_t max_eval, double req_abs, double req_rel, int threads,
                      double _Complex *sol, int *info)
{
    const size_t N = n + 2 * m;
    double _Complex *wg0 = calloc(N * N, sizeof(double _Complex));
    if (!wg0) return -1000;
    int err = oracle_fill_incidence_imm(wg0, e, m, nodes, n);
    if (err) { free(wg0); return err; }
    int setup_err = 0;
#ifdef _OPENMP
    int nthr = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr)
#else
    (void) threads;
#endif
    {
        double _Complex *zl = calloc(m * m, sizeof(double _Complex));
        double _Complex *zt = calloc(m * m, sizeof(double _Complex));
        double _Complex *wg = malloc(N * N * sizeof(double _Complex));
        if (!zl || !zt || !wg) {
#ifdef _OPENMP
#pragma omp atomic write
#endif
            setup_err = -1000;
        }
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
        for (size_t k = 0; k < ns; k++) {
            if (!zl || !zt || !wg) { info[k] = -1000; continue; }
            int ierr = oracle_hem_impedances(e, img, m, s[k], kappa[k], mur, max_eval,
                                             req_abs, req_rel, ORACLE_INTG_DOUBLE, zl, zt);
            if (ierr) { info[k] = -2000 + ierr; continue; }
            memcpy(wg, wg0, N * N * sizeof(double _Complex));
            oracle_fill_impedance_imm(wg, zl, zt, m, n);
            double _Complex *x = sol + k * N;
            for (size_t q = 0; q < N; q++) x[q] = 0.0;
            x[inj_node] = inj[k];
            info[k] = oracle_solve_immittance(wg, x, m, n);
        }
        free(zl);
        free(zt);
        free(wg);
    }
    free(wg0);
    return setup_err;
}

/* ---- post-processing: potentials, fields, voltage ------------------------ */

/* src/electrode.c:434-457: the scalar potential at a point, one INTG_SINGLE
 * integral per electrode towards the point (as a receiver's middle point),
 * times it[m] / L_m, over 4 pi kappa. No skipping of small currents. */
double _Complex oracle_electric_potential (const double *point, const OracleElectrode *e, size_t m,
                                           const double _Complex *it, double _Complex gamma,
                                           double _Complex kappa, size_t max_eval, double req_abs,
                                           double req_rel, int *failure)
{
    OracleElectrode pe;
    memset(&pe, 0, sizeof(pe));
    for (int i = 0; i < 3; i++) pe.middle_point[i] = point[i];
    double result[2], error[2];
    double _Complex pot = 0.0;
    *failure = 0;
    for (size_t k = 0; k < m; k++) {
        int f = oracle_integral(&e[k], &pe, gamma, max_eval, req_abs, req_rel, ORACLE_INTG_SINGLE,
                                result, error);
        if (f) { *failure = f; return f; }
        pot += (result[0] + I * result[1]) * it[k] / e[k].length;
    }
    return pot / (ORACLE_FOUR_PI * kappa);
}

/* src/electrode.c:459-493: vector potential; electrodes with |il| below
 * DBL_EPSILON are skipped; va is overwritten. */
int oracle_magnetic_potential (const double *point, const OracleElectrode *e, size_t m,
                               const double _Complex *il, double _Complex gamma, double mur,
                               size_t max_eval, double req_abs, double req_rel, double _Complex *va)
{
    OracleElectrode pe;
    memset(&pe, 0, sizeof(pe));
    double result[2], error[2];
    for (int i = 0; i < 3; i++) {
        pe.middle_point[i] = point[i];
        va[i] = 0.0;
    }
    for (size_t k = 0; k < m; k++) {
        if (cabs(il[k]) < DBL_EPSILON) continue;
        double dx = e[k].end_point[0] - e[k].start_point[0];
        double dy = e[k].end_point[1] - e[k].start_point[1];
        double dz = e[k].end_point[2] - e[k].start_point[2];
        int f = oracle_integral(&e[k], &pe, gamma, max_eval, req_abs, req_rel, ORACLE_INTG_SINGLE,
                                result, error);
        if (f) return f;
        double _Complex pot = (result[0] + I * result[1]) * il[k] / e[k].length;
        va[0] += pot * dx;
        va[1] += pot * dy;
        va[2] += pot * dz;
    }
    double _Complex u_4pi = mur * ORACLE_MU0 / ORACLE_FOUR_PI;
    for (int i = 0; i < 3; i++) va[i] *= u_4pi;
    return 0;
}

typedef struct {
    const double *point1, *point2;
    const OracleElectrode *e;
    size_t m;
    const double _Complex *il, *it;
    double _Complex gamma, s, kappa;
    double mur;
    size_t max_eval;
    double req_abs, req_rel;
} field_data;

/* src/electrode.c:495-520: (1 + gamma r) e^{-gamma r} / r^2 along (p - x)/r;
 * r is taken before r^2 is clamped to DBL_EPSILON. */
static int integrand_efield (unsigned ndim, const double *t, void *aux, unsigned fdim, double *fval)
{
    (void) ndim; (void) fdim;
    const field_data *p = aux;
    const OracleElectrode *el = p->e;
    double dx[3], r2 = 0.0;
    for (int i = 0; i < 3; i++) {
        double x = t[0] * (el->end_point[i] - el->start_point[i]) + el->start_point[i];
        dx[i] = p->point1[i] - x;
        r2 += pow(dx[i], 2.0);
    }
    double r1 = sqrt(r2);
    if (r2 < DBL_EPSILON) r2 = DBL_EPSILON;
    double _Complex ef = (1 + p->gamma * r1) * cexp(-p->gamma * r1) / r2;
    for (int i = 0; i < 3; i++) {
        double _Complex ex = ef * dx[i] / r1;
        fval[2 * i] = creal(ex);
        fval[2 * i + 1] = cimag(ex);
    }
    return 0;
}

/* src/electrode.c:522-560: E = -s A (only when |s| > DBL_EPSILON, which
 * overwrites ve) plus the conservative part accumulated into ve, one 1-D
 * cubature (6 outputs, ERROR_PAIRED) per electrode with |it| >= DBL_EPSILON. */
int oracle_electric_field (const double *point, const OracleElectrode *e, size_t m,
                           const double _Complex *il, const double _Complex *it,
                           double _Complex gamma, double _Complex s, double mur,
                           double _Complex kappa, size_t max_eval, double req_abs, double req_rel,
                           double _Complex *ve)
{
    if (cabs(s) > DBL_EPSILON) {
        oracle_magnetic_potential(point, e, m, il, gamma, mur, max_eval, req_abs, req_rel, ve);
        for (int i = 0; i < 3; i++) ve[i] *= -s;
    }
    field_data aux;
    memset(&aux, 0, sizeof(aux));
    aux.point1 = point;
    aux.gamma = gamma;
    const double tmin[1] = {0.0}, tmax[1] = {1.0};
    double result[6], error[6];
    int failure = 0;
    for (size_t k = 0; k < m; k++) {
        if (cabs(it[k]) < DBL_EPSILON) continue;
        aux.e = e + k;
        failure = hcubature(6, integrand_efield, &aux, 1, tmin, tmax, max_eval, req_abs, req_rel,
                            ERROR_PAIRED, result, error);
        double _Complex it_4pik = it[k] / (ORACLE_FOUR_PI * kappa);
        for (int i = 0; i < 3; i++) ve[i] += (result[2 * i] + I * result[2 * i + 1]) * it_4pik;
    }
    return failure;
}

/* src/electrode.c:599-635: E at p1 + t (p2 - p1) projected on the unit
 * direction of the path; 1 (failure) for a path shorter than DBL_EPSILON.
 * The field starts from zero (the reference passes an uninitialised array,
 * which electric_field overwrites whenever |s| > DBL_EPSILON). */
static int integrand_voltage (unsigned ndim, const double *t, void *aux, unsigned fdim, double *fval)
{
    (void) ndim; (void) fdim;
    const field_data *p = aux;
    double point[3], dx[3], length = 0.0;
    for (int i = 0; i < 3; i++) {
        dx[i] = p->point2[i] - p->point1[i];
        point[i] = t[0] * dx[i] + p->point1[i];
        length += pow(dx[i], 2.0);
    }
    if (length < DBL_EPSILON) return 1;
    length = sqrt(length);
    double _Complex ve[3] = {0.0, 0.0, 0.0};
    oracle_electric_field(point, p->e, p->m, p->il, p->it, p->gamma, p->s, p->mur, p->kappa,
                          p->max_eval, p->req_abs, p->req_rel, ve);
    double _Complex vc = 0.0;
    for (int i = 0; i < 3; i++) vc += ve[i] * dx[i];
    vc /= length;
    fval[0] = creal(vc);
    fval[1] = cimag(vc);
    return 0;
}

/* src/electrode.c:637-668: the integral over t in [0, 1] of E . (p2 - p1) /
 * |p2 - p1| (nested cubature; the result is the path voltage divided by the
 * path length, as the reference returns it). */
double _Complex oracle_voltage (const double *point1, const double *point2, const OracleElectrode *e,
                                size_t m, const double _Complex *il, const double _Complex *it,
                                double _Complex gamma, double _Complex s, double mur,
                                double _Complex kappa, size_t max_eval, double req_abs, double req_rel,
                                int *failure)
{
    field_data aux;
    memset(&aux, 0, sizeof(aux));
    aux.point1 = point1;
    aux.point2 = point2;
    aux.e = e;
    aux.m = m;
    aux.il = il;
    aux.it = it;
    aux.gamma = gamma;
    aux.s = s;
    aux.mur = mur;
    aux.kappa = kappa;
    aux.max_eval = max_eval;
    aux.req_abs = req_abs;
    aux.req_rel = req_rel;
    const double tmin[1] = {0.0}, tmax[1] = {1.0};
    double result[2] = {0.0, 0.0}, error[2];
    *failure = hcubature(2, integrand_voltage, &aux, 1, tmin, tmax, max_eval, req_abs, req_rel,
                         ERROR_PAIRED, result, error);
    return result[0] + I * result[1];
}

/* Ground potential by the closed-form mHEM loop of
 * examples/visacro57emc01.c:406-430: for each point p and electrode m,
 * e^{-gamma rbar} log((r1 + r2 + L) / (r1 + r2 - L)) / L with rbar, r1, r2 the
 * distances from p to the midpoint and the ends, times it[m] / (4 pi kappa).
 * it holds the transversal currents already multiplied by (1 + ref_t) and is
 * laid out (ne x nrhs) column-major; gpd[p * nrhs + k]. */
int oracle_gpd_mhem (const double *points, size_t np, const OracleElectrode *e, size_t m,
                     const double _Complex *it, size_t nrhs, double _Complex gamma,
                     double _Complex kappa, double _Complex *gpd)
{
    const double _Complex one_4pik = 1.0 / (ORACLE_FOUR_PI * kappa);
    for (size_t p = 0; p < np; p++) {
        for (size_t k = 0; k < nrhs; k++) gpd[p * nrhs + k] = 0.0;
        for (size_t q = 0; q < m; q++) {
            double rbar = oracle_vector_length(points + p * 3, e[q].middle_point);
            double r1 = oracle_vector_length(points + p * 3, e[q].start_point);
            double r2 = oracle_vector_length(points + p * 3, e[q].end_point);
            double r0 = (r1 + r2 + e[q].length) / (r1 + r2 - e[q].length);
            double _Complex exp_gr = cexp(-gamma * rbar) * log(r0) / e[q].length;
            for (size_t k = 0; k < nrhs; k++) gpd[p * nrhs + k] += one_4pik * it[q + m * k] * exp_gr;
        }
    }
    return 0;
}
