/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * Interface subset of FFTW3 that the reference uses (src/auxiliary.c:239-329,
 * examples/three_grids.c:49-87): plans for 1-D real-to-complex and
 * complex-to-real transforms and their "many" forms. FFTW is not installed
 * here; oracle/dft.c implements these entry points from FFTW's documented
 * transform definitions (unnormalised DFT, e^{-2 pi i jk/n} forward,
 * e^{+2 pi i jk/n} backward, Hermitian half-spectrum of n/2+1 values).
 */
#ifndef TAGS_ORACLE_FFTW3_H_
#define TAGS_ORACLE_FFTW3_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* As in FFTW: when <complex.h> was included first, fftw_complex is the C99
 * complex type, otherwise a pair of doubles (same memory layout). */
#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif

typedef struct tags_fftw_plan_s *fftw_plan;

#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

void *fftw_malloc (size_t n);
void fftw_free (void *p);
fftw_plan fftw_plan_dft_r2c_1d (int n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d (int n, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_many_dft_r2c (int rank, const int *n, int howmany,
                                  double *in, const int *inembed, int istride, int idist,
                                  fftw_complex *out, const int *onembed, int ostride, int odist,
                                  unsigned flags);
fftw_plan fftw_plan_many_dft_c2r (int rank, const int *n, int howmany,
                                  fftw_complex *in, const int *inembed, int istride, int idist,
                                  double *out, const int *onembed, int ostride, int odist,
                                  unsigned flags);
void fftw_execute (const fftw_plan p);
void fftw_destroy_plan (fftw_plan p);

#ifdef __cplusplus
}
#endif

#endif /* TAGS_ORACLE_FFTW3_H_ */
