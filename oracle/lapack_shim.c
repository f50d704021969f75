/* Test infrastructure only: CPU oracle for the HEM hot path.
 *
 * LAPACK/BLAS routines the reference calls (src/lapack.h, src/blas.h:
 * zsysv_, zsytrf_, zsytri_, zsymm_, zgemm_, zgesv_) resolved at run time.
 * The system has no LAPACK; the Python side of the oracle loads the OpenBLAS
 * that ships inside scipy and hands its function pointers to
 * tags_lapack_bind(). The reference sources are compiled with
 * -Dzsysv_=tags_zsysv_ (and so on) so that they call these forwarders.
 */
#include <complex.h>
#include <stdio.h>
#include <string.h>

typedef double _Complex zc;
typedef void (*zsysv_t)(char *, int *, int *, zc *, int *, int *, zc *, int *, zc *, int *, int *);
typedef void (*zsytrf_t)(char *, int *, zc *, int *, int *, zc *, int *, int *);
typedef void (*zsytri_t)(char *, int *, zc *, int *, int *, zc *, int *);
typedef void (*zsymm_t)(char *, char *, int *, int *, zc *, zc *, int *, zc *, int *, zc *, zc *, int *);
typedef void (*zgemm_t)(char *, char *, int *, int *, int *, zc *, zc *, int *, zc *, int *, zc *, zc *, int *);
typedef void (*zgesv_t)(int *, int *, zc *, int *, int *, zc *, int *, int *);

static zsysv_t p_zsysv;
static zsytrf_t p_zsytrf;
static zsytri_t p_zsytri;
static zsymm_t p_zsymm;
static zgemm_t p_zgemm;
static zgesv_t p_zgesv;

/* Bind one routine by its LAPACK name ("zsysv", ...). Returns 0 on success. */
int tags_lapack_bind (const char *name, void *fn)
{
    if (!strcmp(name, "zsysv")) p_zsysv = (zsysv_t) fn;
    else if (!strcmp(name, "zsytrf")) p_zsytrf = (zsytrf_t) fn;
    else if (!strcmp(name, "zsytri")) p_zsytri = (zsytri_t) fn;
    else if (!strcmp(name, "zsymm")) p_zsymm = (zsymm_t) fn;
    else if (!strcmp(name, "zgemm")) p_zgemm = (zgemm_t) fn;
    else if (!strcmp(name, "zgesv")) p_zgesv = (zgesv_t) fn;
    else return 1;
    return 0;
}

int tags_lapack_ready (void) { return p_zsysv != NULL; }

static void missing (const char *name, int *info)
{
    fprintf(stderr, "oracle: LAPACK routine %s was not bound\n", name);
    if (info) *info = -1000;
}

void tags_zsysv_ (char *uplo, int *n, int *nrhs, zc *a, int *lda, int *ipiv,
                  zc *b, int *ldb, zc *work, int *lwork, int *info)
{
    if (!p_zsysv) { missing("zsysv", info); return; }
    p_zsysv(uplo, n, nrhs, a, lda, ipiv, b, ldb, work, lwork, info);
}

void tags_zsytrf_ (char *uplo, int *n, zc *a, int *lda, int *ipiv, zc *work,
                   int *lwork, int *info)
{
    if (!p_zsytrf) { missing("zsytrf", info); return; }
    p_zsytrf(uplo, n, a, lda, ipiv, work, lwork, info);
}

void tags_zsytri_ (char *uplo, int *n, zc *a, int *lda, int *ipiv, zc *work, int *info)
{
    if (!p_zsytri) { missing("zsytri", info); return; }
    p_zsytri(uplo, n, a, lda, ipiv, work, info);
}

void tags_zsymm_ (char *side, char *uplo, int *m, int *n, zc *alpha, zc *a, int *lda,
                  zc *b, int *ldb, zc *beta, zc *c, int *ldc)
{
    if (!p_zsymm) { missing("zsymm", NULL); return; }
    p_zsymm(side, uplo, m, n, alpha, a, lda, b, ldb, beta, c, ldc);
}

void tags_zgemm_ (char *ta, char *tb, int *m, int *n, int *k, zc *alpha, zc *a, int *lda,
                  zc *b, int *ldb, zc *beta, zc *c, int *ldc)
{
    if (!p_zgemm) { missing("zgemm", NULL); return; }
    p_zgemm(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void tags_zgesv_ (int *n, int *nrhs, zc *a, int *lda, int *ipiv, zc *b, int *ldb, int *info)
{
    if (!p_zgesv) { missing("zgesv", info); return; }
    p_zgesv(n, nrhs, a, lda, ipiv, b, ldb, info);
}
