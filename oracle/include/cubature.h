/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * Interface of the h-adaptive cubature routine `hcubature` that the reference
 * calls (src/electrode.c:273-291). The reference takes it from the git
 * submodule stevengj/cubature, which is not vendored and not pinned; this
 * header declares the published call signature so that the reference sources
 * (and the oracle's own restatement) compile against the project-written
 * implementation in oracle/cubature.c. Nothing in the shipped GPU library
 * includes this file.
 */
#ifndef TAGS_ORACLE_CUBATURE_H_
#define TAGS_ORACLE_CUBATURE_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* How the per-component error estimates are combined in the convergence test.
 * ERROR_INDIVIDUAL: every component must converge on its own.
 * ERROR_PAIRED: components (2j, 2j+1) are the real and imaginary parts of one
 * complex value; the test uses the Euclidean norm of the pair. */
typedef enum {
    ERROR_INDIVIDUAL = 0,
    ERROR_PAIRED,
    ERROR_L2,
    ERROR_L1,
    ERROR_LINF
} error_norm;

/* Integrand: fill fval[0..fdim) at the point x[0..ndim). Nonzero return aborts. */
typedef int (*integrand) (unsigned ndim, const double *x, void *fdata,
                          unsigned fdim, double *fval);

/* Integrate f over the box [xmin, xmax]^dim. Stops when the summed error
 * estimate meets reqAbsError or reqRelError*|value| (per `norm`), or when
 * maxEval evaluations were spent (0 = no limit). Returns 0 on success. */
int hcubature (unsigned fdim, integrand f, void *fdata, unsigned dim,
               const double *xmin, const double *xmax, size_t maxEval,
               double reqAbsError, double reqRelError, error_norm norm,
               double *val, double *err);

#ifdef __cplusplus
}
#endif

#endif /* TAGS_ORACLE_CUBATURE_H_ */
