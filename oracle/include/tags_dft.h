/* Test infrastructure only: CPU oracle for the HEM hot path.
 * Direct real DFTs with FFTW's conventions (see oracle/dft.c). */
#ifndef TAGS_ORACLE_DFT_H_
#define TAGS_ORACLE_DFT_H_
#include <complex.h>
#ifdef __cplusplus
extern "C" {
#endif
int tags_dft_r2c (long n, const double *x, long xs, double _Complex *y, long ys);
int tags_dft_c2r (long n, const double _Complex *x, long xs, double *y, long ys);
#ifdef __cplusplus
}
#endif
#endif
