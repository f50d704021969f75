/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * FFTW-compatible real DFTs for the numerical Laplace transform and its
 * inverse (src/auxiliary.c:239-329). Written from FFTW's documented transform
 * definitions, not from FFTW source:
 *   r2c: Y[k] = sum_{j<n} x[j] e^{-2 pi i jk/n},             k = 0..n/2
 *   c2r: y[j] = sum_{k<n} X[k] e^{+2 pi i jk/n}, X[n-k] = conj(X[k]),
 *        unnormalised; Im X[0] (and Im X[n/2] for even n) are ignored.
 * A direct O(n^2) sum with exact integer reduction of the twiddle index,
 * accurate to ~n*eps; the oracle's transforms are a few thousand points.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fftw3.h"
#include "tags_dft.h"

static const double DFT_TWO_PI = 6.283185307179586476925286766559;

static void twiddles (long n, double *cs, double *sn)
{
    for (long q = 0; q < n; q++) {
        double a = DFT_TWO_PI * (double) q / (double) n;
        cs[q] = cos(a);
        sn[q] = sin(a);
    }
}

int tags_dft_r2c (long n, const double *x, long xs, double _Complex *y, long ys)
{
    if (n < 1) return 1;
    double *cs = malloc(2 * n * sizeof(double));
    if (!cs) return 1;
    double *sn = cs + n;
    twiddles(n, cs, sn);
    for (long k = 0; k <= n / 2; k++) {
        double re = 0.0, im = 0.0;
        for (long j = 0; j < n; j++) {
            long q = (long) (((unsigned long long) j * (unsigned long long) k) % (unsigned long long) n);
            re += x[j * xs] * cs[q];
            im -= x[j * xs] * sn[q];
        }
        y[k * ys] = re + I * im;
    }
    free(cs);
    return 0;
}

int tags_dft_c2r (long n, const double _Complex *x, long xs, double *y, long ys)
{
    if (n < 1) return 1;
    double *cs = malloc(2 * n * sizeof(double));
    if (!cs) return 1;
    double *sn = cs + n;
    twiddles(n, cs, sn);
    long half = n / 2;
    for (long j = 0; j < n; j++) {
        double acc = creal(x[0]);
        long kmax = (n % 2 == 0) ? half - 1 : half;
        for (long k = 1; k <= kmax; k++) {
            long q = (long) (((unsigned long long) j * (unsigned long long) k) % (unsigned long long) n);
            acc += 2.0 * (creal(x[k * xs]) * cs[q] - cimag(x[k * xs]) * sn[q]);
        }
        if (n % 2 == 0 && n > 1) acc += (j % 2 ? -1.0 : 1.0) * creal(x[half * xs]);
        y[j * ys] = acc;
    }
    free(cs);
    return 0;
}

/* ---- FFTW entry points used by the reference ---------------------------- */

struct tags_fftw_plan_s {
    int kind;           /* 0 = r2c, 1 = c2r */
    long n;
    int howmany;
    void *in, *out;
    long istride, idist, ostride, odist;
};

void *fftw_malloc (size_t n) { return malloc(n ? n : 1); }
void fftw_free (void *p) { free(p); }

static fftw_plan make_plan (int kind, long n, int howmany, void *in, long is, long id,
                            void *out, long os, long od)
{
    fftw_plan p = malloc(sizeof(*p));
    if (!p) return NULL;
    p->kind = kind; p->n = n; p->howmany = howmany; p->in = in; p->out = out;
    p->istride = is; p->idist = id; p->ostride = os; p->odist = od;
    return p;
}

fftw_plan fftw_plan_dft_r2c_1d (int n, double *in, fftw_complex *out, unsigned flags)
{
    (void) flags;
    return make_plan(0, n, 1, in, 1, n, out, 1, n / 2 + 1);
}

fftw_plan fftw_plan_dft_c2r_1d (int n, fftw_complex *in, double *out, unsigned flags)
{
    (void) flags;
    return make_plan(1, n, 1, in, 1, n / 2 + 1, out, 1, n);
}

fftw_plan fftw_plan_many_dft_r2c (int rank, const int *n, int howmany,
                                  double *in, const int *inembed, int istride, int idist,
                                  fftw_complex *out, const int *onembed, int ostride, int odist,
                                  unsigned flags)
{
    (void) inembed; (void) onembed; (void) flags;
    if (rank != 1) return NULL;
    return make_plan(0, n[0], howmany, in, istride, idist, out, ostride, odist);
}

fftw_plan fftw_plan_many_dft_c2r (int rank, const int *n, int howmany,
                                  fftw_complex *in, const int *inembed, int istride, int idist,
                                  double *out, const int *onembed, int ostride, int odist,
                                  unsigned flags)
{
    (void) inembed; (void) onembed; (void) flags;
    if (rank != 1) return NULL;
    return make_plan(1, n[0], howmany, in, istride, idist, out, ostride, odist);
}

void fftw_execute (const fftw_plan p)
{
    if (!p) return;
    for (int h = 0; h < p->howmany; h++) {
        if (p->kind == 0) {
            const double *x = (const double *) p->in + (long) h * p->idist;
            double _Complex *y = (double _Complex *) p->out + (long) h * p->odist;
            tags_dft_r2c(p->n, x, p->istride, y, p->ostride);
        } else {
            /* FFTW's c2r may overwrite its input; this one does not. */
            const double _Complex *x = (const double _Complex *) p->in + (long) h * p->idist;
            double *y = (double *) p->out + (long) h * p->odist;
            tags_dft_c2r(p->n, x, p->istride, y, p->ostride);
        }
    }
}

void fftw_destroy_plan (fftw_plan p) { free(p); }
