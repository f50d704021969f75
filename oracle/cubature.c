/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * Project-written h-adaptive cubature with the signature of `hcubature`
 * (stevengj/cubature, the git submodule the reference declares in
 * .gitmodules:1-3; it is not vendored and no commit is pinned, so its source
 * is not available here). This file restates the published method that
 * library documents:
 *   - dim == 1: 15-point Gauss-Kronrod rule with the embedded 7-point Gauss
 *     rule; error = |K15 - G7|; a region is split by bisection.
 *   - dim >= 2: Genz-Malik degree-7 rule with the embedded degree-5 rule
 *     (A. C. Genz, A. A. Malik, J. Comput. Appl. Math. 6 (1980) 295-302);
 *     error = |I7 - I5|; a region is bisected along the axis with the largest
 *     fourth divided difference.
 *   - global adaptivity: the region with the largest error is split until the
 *     summed error meets the requested tolerance (per error norm) or the
 *     evaluation budget is spent.
 * The reference calls it at src/electrode.c:273-291 (DOUBLE: fdim 2, dim 2,
 * ERROR_PAIRED; SINGLE: fdim 2, dim 1; MHEM: fdim 1, dim 1, ERROR_INDIVIDUAL).
 * Only tests, the smoke check and the CPU baseline of the bench use it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "cubature.h"

/* Gauss-Kronrod 7-15 abscissae on [-1, 1] (descending, last = 0) and weights
 * (published QUADPACK qk15 table). */
static const double gk_x[8] = {
    0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
    0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
    0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
    0.207784955007898467600689403773245, 0.000000000000000000000000000000000};
static const double gk_wk[8] = {
    0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
    0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
    0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
    0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
/* Gauss 7-point weights for abscissae gk_x[1], gk_x[3], gk_x[5], gk_x[7]. */
static const double gk_wg[4] = {
    0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
    0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

#define MAX_REGIONS (1u << 22)

typedef struct {
    unsigned dim, fdim;
    size_t cap, count;      /* heap capacity / size (regions) */
    double *geom;           /* per region: center[dim], half[dim] */
    double *est;            /* per region: val[fdim], err[fdim] */
    unsigned *split;        /* split axis chosen when the region was evaluated */
    double *key;            /* heap key: largest component error */
    size_t *slot;           /* heap of storage slots */
} region_heap;

typedef struct {
    unsigned dim, fdim;
    integrand f;
    void *fdata;
    double *x;              /* one point */
    double *fv;             /* all point values of one rule application */
    size_t neval;
} rule_ctx;

static int eval_point (rule_ctx *r, const double *x, double *out)
{
    r->neval++;
    return r->f(r->dim, x, r->fdata, r->fdim, out);
}

/* 1-D Gauss-Kronrod rule on [c-h, c+h]. */
static int rule_gk15 (rule_ctx *r, const double *c, const double *h,
                      double *val, double *err, unsigned *split)
{
    const unsigned fd = r->fdim;
    double *fc = r->fv;                 /* centre value */
    double *f1 = r->fv + fd;            /* f(c - h x) */
    double *f2 = r->fv + 2 * fd;        /* f(c + h x) */
    double *gsum = r->fv + 3 * fd;
    if (eval_point(r, c, fc)) return 1;
    for (unsigned j = 0; j < fd; j++) {
        val[j] = gk_wk[7] * fc[j];
        gsum[j] = gk_wg[3] * fc[j];
    }
    for (int i = 0; i < 7; i++) {
        r->x[0] = c[0] - h[0] * gk_x[i];
        if (eval_point(r, r->x, f1)) return 1;
        r->x[0] = c[0] + h[0] * gk_x[i];
        if (eval_point(r, r->x, f2)) return 1;
        for (unsigned j = 0; j < fd; j++) {
            double s = f1[j] + f2[j];
            val[j] += gk_wk[i] * s;
            if (i & 1) gsum[j] += gk_wg[i >> 1] * s;
        }
    }
    for (unsigned j = 0; j < fd; j++) {
        val[j] *= h[0];
        err[j] = fabs(val[j] - gsum[j] * h[0]);
    }
    *split = 0;
    return 0;
}

/* Genz-Malik degree 7/5 rule on the box c +- h (dim >= 2). */
static int rule_gm (rule_ctx *r, const double *c, const double *h,
                    double *val, double *err, unsigned *split)
{
    const unsigned n = r->dim, fd = r->fdim;
    const double l2 = sqrt(9.0 / 70.0), l3 = sqrt(9.0 / 10.0);
    const double l4 = sqrt(9.0 / 10.0), l5 = sqrt(9.0 / 19.0);
    const double dn = (double) n;
    const double w1 = (12824.0 - 9120.0 * dn + 400.0 * dn * dn) / 19683.0;
    const double w2 = 980.0 / 6561.0;
    const double w3 = (1820.0 - 400.0 * dn) / 19683.0;
    const double w4 = 200.0 / 19683.0;
    const double w5 = 6859.0 / 19683.0 / ldexp(1.0, (int) n);
    const double v1 = (729.0 - 950.0 * dn + 50.0 * dn * dn) / 729.0;
    const double v2 = 245.0 / 486.0;
    const double v3 = (265.0 - 100.0 * dn) / 1458.0;
    const double v4 = 25.0 / 729.0;
    const double ratio = (l2 * l2) / (l3 * l3);
    double *f0 = r->fv, *fa = f0 + fd, *fb = fa + fd;
    double *s2 = fb + fd, *s3 = s2 + fd, *s4 = s3 + fd, *s5 = s4 + fd;
    double vol = 1.0;
    for (unsigned i = 0; i < n; i++) vol *= 2.0 * h[i];
    if (eval_point(r, c, f0)) return 1;
    for (unsigned j = 0; j < fd; j++) { s2[j] = s3[j] = s4[j] = s5[j] = 0.0; }
    double best = -1.0;
    unsigned best_axis = 0;
    memcpy(r->x, c, n * sizeof(double));
    for (unsigned i = 0; i < n; i++) {
        double d2 = 0.0;
        double t2[64], t3[64];
        /* +-lambda2 and +-lambda3 along axis i */
        r->x[i] = c[i] - l2 * h[i];
        if (eval_point(r, r->x, fa)) return 1;
        r->x[i] = c[i] + l2 * h[i];
        if (eval_point(r, r->x, fb)) return 1;
        for (unsigned j = 0; j < fd; j++) {
            double s = fa[j] + fb[j];
            s2[j] += s;
            if (j < 64) t2[j] = s;
        }
        r->x[i] = c[i] - l3 * h[i];
        if (eval_point(r, r->x, fa)) return 1;
        r->x[i] = c[i] + l3 * h[i];
        if (eval_point(r, r->x, fb)) return 1;
        for (unsigned j = 0; j < fd; j++) {
            double s = fa[j] + fb[j];
            s3[j] += s;
            if (j < 64) t3[j] = s;
        }
        r->x[i] = c[i];
        for (unsigned j = 0; j < fd && j < 64; j++)
            d2 += fabs(t2[j] - 2.0 * f0[j] - ratio * (t3[j] - 2.0 * f0[j]));
        if (d2 > best) { best = d2; best_axis = i; }
    }
    /* +-lambda4 on every pair of axes */
    for (unsigned i = 0; i < n; i++) {
        for (unsigned k = i + 1; k < n; k++) {
            for (int sg = 0; sg < 4; sg++) {
                r->x[i] = c[i] + ((sg & 1) ? l4 : -l4) * h[i];
                r->x[k] = c[k] + ((sg & 2) ? l4 : -l4) * h[k];
                if (eval_point(r, r->x, fa)) return 1;
                for (unsigned j = 0; j < fd; j++) s4[j] += fa[j];
            }
            r->x[i] = c[i];
            r->x[k] = c[k];
        }
    }
    /* +-lambda5 on all 2^n corners */
    for (unsigned long corner = 0; corner < (1ul << n); corner++) {
        for (unsigned i = 0; i < n; i++)
            r->x[i] = c[i] + (((corner >> i) & 1ul) ? l5 : -l5) * h[i];
        if (eval_point(r, r->x, fa)) return 1;
        for (unsigned j = 0; j < fd; j++) s5[j] += fa[j];
    }
    for (unsigned j = 0; j < fd; j++) {
        double i7 = vol * (w1 * f0[j] + w2 * s2[j] + w3 * s3[j] + w4 * s4[j] + w5 * s5[j]);
        double i5 = vol * (v1 * f0[j] + v2 * s2[j] + v3 * s3[j] + v4 * s4[j]);
        val[j] = i7;
        err[j] = fabs(i7 - i5);
    }
    *split = best_axis;
    return 0;
}

static int heap_grow (region_heap *hp)
{
    size_t cap = hp->cap ? hp->cap * 2 : 64;
    if (cap > MAX_REGIONS) cap = MAX_REGIONS;
    if (cap <= hp->cap) return 1;
    double *g = realloc(hp->geom, cap * 2 * hp->dim * sizeof(double));
    if (!g) return 1;
    hp->geom = g;
    double *e = realloc(hp->est, cap * 2 * hp->fdim * sizeof(double));
    if (!e) return 1;
    hp->est = e;
    unsigned *s = realloc(hp->split, cap * sizeof(unsigned));
    if (!s) return 1;
    hp->split = s;
    double *k = realloc(hp->key, cap * sizeof(double));
    if (!k) return 1;
    hp->key = k;
    size_t *sl = realloc(hp->slot, cap * sizeof(size_t));
    if (!sl) return 1;
    hp->slot = sl;
    hp->cap = cap;
    return 0;
}

static void heap_push (region_heap *hp, size_t s)
{
    size_t i = hp->count++;
    hp->slot[i] = s;
    while (i > 0) {
        size_t p = (i - 1) / 2;
        if (hp->key[hp->slot[p]] >= hp->key[hp->slot[i]]) break;
        size_t t = hp->slot[p]; hp->slot[p] = hp->slot[i]; hp->slot[i] = t;
        i = p;
    }
}

static size_t heap_pop (region_heap *hp)
{
    size_t top = hp->slot[0];
    hp->slot[0] = hp->slot[--hp->count];
    size_t i = 0;
    for (;;) {
        size_t l = 2 * i + 1, r = l + 1, m = i;
        if (l < hp->count && hp->key[hp->slot[l]] > hp->key[hp->slot[m]]) m = l;
        if (r < hp->count && hp->key[hp->slot[r]] > hp->key[hp->slot[m]]) m = r;
        if (m == i) break;
        size_t t = hp->slot[m]; hp->slot[m] = hp->slot[i]; hp->slot[i] = t;
        i = m;
    }
    return top;
}

static int is_converged (unsigned fdim, const double *val, const double *err,
                         double abs_tol, double rel_tol, error_norm norm)
{
    switch (norm) {
    case ERROR_PAIRED: {
        unsigned j = 0;
        for (; j + 1 < fdim; j += 2) {
            double e = hypot(err[j], err[j + 1]);
            double v = hypot(val[j], val[j + 1]);
            if (e > abs_tol && e > rel_tol * v) return 0;
        }
        if (j < fdim && err[j] > abs_tol && err[j] > rel_tol * fabs(val[j])) return 0;
        return 1;
    }
    case ERROR_L2: case ERROR_L1: case ERROR_LINF: {
        double e = 0.0, v = 0.0;
        for (unsigned j = 0; j < fdim; j++) {
            if (norm == ERROR_L2) { e += err[j] * err[j]; v += val[j] * val[j]; }
            else if (norm == ERROR_L1) { e += fabs(err[j]); v += fabs(val[j]); }
            else { e = fmax(e, fabs(err[j])); v = fmax(v, fabs(val[j])); }
        }
        if (norm == ERROR_L2) { e = sqrt(e); v = sqrt(v); }
        return !(e > abs_tol && e > rel_tol * v);
    }
    default:
        for (unsigned j = 0; j < fdim; j++)
            if (err[j] > abs_tol && err[j] > rel_tol * fabs(val[j])) return 0;
        return 1;
    }
}

int hcubature (unsigned fdim, integrand f, void *fdata, unsigned dim,
               const double *xmin, const double *xmax, size_t maxEval,
               double reqAbsError, double reqRelError, error_norm norm,
               double *val, double *err)
{
    if (fdim == 0) return 0;
    for (unsigned j = 0; j < fdim; j++) { val[j] = 0.0; err[j] = 0.0; }
    if (dim == 0) return f(0, xmin, fdata, fdim, val);
    if (dim > 20 || fdim > 64) return 1;
    int status = 0;
    region_heap hp = {dim, fdim, 0, 0, NULL, NULL, NULL, NULL, NULL};
    rule_ctx rc = {dim, fdim, f, fdata, NULL, NULL, 0};
    rc.x = malloc(dim * sizeof(double));
    rc.fv = malloc(8 * fdim * sizeof(double));
    double *tv = calloc(2 * fdim, sizeof(double)); /* running totals: val, err */
    size_t used = 0;                               /* storage slots handed out */
    if (!rc.x || !rc.fv || !tv || heap_grow(&hp)) { status = 1; goto done; }
    int (*rule)(rule_ctx *, const double *, const double *, double *, double *, unsigned *)
        = (dim == 1) ? rule_gk15 : rule_gm;
    /* root region */
    {
        size_t s = used++;
        double *g = hp.geom + s * 2 * dim, *e = hp.est + s * 2 * fdim;
        for (unsigned i = 0; i < dim; i++) {
            g[i] = 0.5 * (xmin[i] + xmax[i]);
            g[dim + i] = 0.5 * (xmax[i] - xmin[i]);
        }
        if (rule(&rc, g, g + dim, e, e + fdim, &hp.split[s])) { status = 1; goto done; }
        double k = 0.0;
        for (unsigned j = 0; j < fdim; j++) {
            tv[j] += e[j]; tv[fdim + j] += e[fdim + j];
            if (e[fdim + j] > k) k = e[fdim + j];
        }
        hp.key[s] = k;
        heap_push(&hp, s);
    }
    for (;;) {
        if (is_converged(fdim, tv, tv + fdim, reqAbsError, reqRelError, norm)) break;
        if (maxEval && rc.neval >= maxEval) break;
        if (used + 1 > hp.cap) {
            if (hp.cap >= MAX_REGIONS || heap_grow(&hp)) { status = 1; break; }
        }
        size_t p = heap_pop(&hp);
        double *pg = hp.geom + p * 2 * dim, *pe = hp.est + p * 2 * fdim;
        unsigned ax = hp.split[p];
        /* child 0 overwrites the parent's slot, child 1 takes a fresh one */
        size_t kids[2] = {p, used++};
        double pc[20], ph[20], pv[64], perr[64];
        memcpy(pc, pg, dim * sizeof(double));
        memcpy(ph, pg + dim, dim * sizeof(double));
        for (unsigned j = 0; j < fdim; j++) { pv[j] = pe[j]; perr[j] = pe[fdim + j]; }
        ph[ax] *= 0.5;
        for (int q = 0; q < 2; q++) {
            size_t s = kids[q];
            double *g = hp.geom + s * 2 * dim, *e = hp.est + s * 2 * fdim;
            memcpy(g, pc, dim * sizeof(double));
            memcpy(g + dim, ph, dim * sizeof(double));
            g[ax] = pc[ax] + (q ? ph[ax] : -ph[ax]);
            if (rule(&rc, g, g + dim, e, e + fdim, &hp.split[s])) { status = 1; goto done; }
            double k = 0.0;
            for (unsigned j = 0; j < fdim; j++) {
                tv[j] += e[j]; tv[fdim + j] += e[fdim + j];
                if (e[fdim + j] > k) k = e[fdim + j];
            }
            hp.key[s] = k;
        }
        for (unsigned j = 0; j < fdim; j++) { tv[j] -= pv[j]; tv[fdim + j] -= perr[j]; }
        heap_push(&hp, kids[0]);
        heap_push(&hp, kids[1]);
    }
    /* final value: exact sum over the live regions */
    for (unsigned j = 0; j < fdim; j++) { val[j] = 0.0; err[j] = 0.0; }
    for (size_t i = 0; i < hp.count; i++) {
        const double *e = hp.est + hp.slot[i] * 2 * fdim;
        for (unsigned j = 0; j < fdim; j++) { val[j] += e[j]; err[j] += e[fdim + j]; }
    }
done:
    free(rc.x); free(rc.fv); free(tv);
    free(hp.geom); free(hp.est); free(hp.split); free(hp.key); free(hp.slot);
    return status;
}
