/* A reference-style C caller of the drop-in entry points, compiled against
 * include/tags_gpu.h and linked with libtags_gpu.so by tests/test_c_caller.py.
 *
 * It follows the per-sample sequence of the reference's harmonic-impedance
 * example (examples/harmonic_impedance.c): segment a 3 m rod into 10
 * segments, then per frequency calculate_impedances + impedances_images,
 * fill_incidence_imm + fill_impedance_imm and solve_immittance with 1 A
 * injected at the top node; prints "f re im" of Z(f) = U[0] per line.
 *
 *   rod_caller host    only host-side calls (no GPU): alipio_soil
 *   rod_caller gpu F.. the rod solve at the frequencies F (Hz)
 */
#include <complex.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tags_gpu.h"

#define NSEG 10
#define PI_ 3.1415926535897932384626433832795029
#define NNODE 11

static void rod(Electrode* e, double* nodes) {
    const double len = 3.0, a = 7e-3;
    for (int k = 0; k < NNODE; ++k) {
        nodes[3 * k + 0] = 0.0;
        nodes[3 * k + 1] = 0.0;
        nodes[3 * k + 2] = -len * k / NSEG;
    }
    for (int k = 0; k < NSEG; ++k) {
        for (int i = 0; i < 3; ++i) {
            e[k].start_point[i] = nodes[3 * k + i];
            e[k].end_point[i] = nodes[3 * (k + 1) + i];
            e[k].middle_point[i] = 0.5 * (nodes[3 * k + i] + nodes[3 * (k + 1) + i]);
        }
        e[k].length = len / NSEG;
        e[k].radius = a;
    }
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    if (strcmp(argv[1], "host") == 0) {
        tags_cdouble sigma, epsr;
        const tags_cdouble s = 2.0 * I * PI_ * 1e5;
        int rc = alipio_soil(&sigma, &epsr, 1e-3, s, 1.26, 0.54, 12.0);
        printf("%d %.17g %.17g %.17g %.17g\n", rc, creal(sigma), cimag(sigma), creal(epsr), cimag(epsr));
        return rc;
    }
    const double mu0 = 1.256637061435917e-6, eps0 = 8.854187817620e-12;
    Electrode e[NSEG], img[NSEG];
    double nodes[3 * NNODE];
    rod(e, nodes);
    memcpy(img, e, sizeof e);
    for (int k = 0; k < NSEG; ++k) {
        img[k].start_point[2] = -e[k].start_point[2];
        img[k].end_point[2] = -e[k].end_point[2];
        img[k].middle_point[2] = -e[k].middle_point[2];
    }
    const size_t m = NSEG, n = NNODE, N = n + 2 * m;
    tags_cdouble* zl = calloc(m * m, sizeof(tags_cdouble));
    tags_cdouble* zt = calloc(m * m, sizeof(tags_cdouble));
    tags_cdouble* wg = calloc(N * N, sizeof(tags_cdouble));
    tags_cdouble* ie = calloc(N, sizeof(tags_cdouble));
    for (int a = 2; a < argc; ++a) {
        const double f = atof(argv[a]);
        const tags_cdouble s = 2.0 * I * PI_ * f;
        const tags_cdouble kappa = 1.0 / 100.0 + s * 10.0 * eps0;
        const tags_cdouble gamma = csqrt(s * mu0 * kappa);
        const tags_cdouble ref_t = (kappa - s * eps0) / (kappa + s * eps0);
        int rc = calculate_impedances(zl, zt, e, m, gamma, s, 1.0, kappa, 0, 1e-6, 1e-6, INTG_DOUBLE);
        if (!rc) rc = impedances_images(zl, zt, e, img, m, gamma, s, 1.0, kappa, 1.0, ref_t, 0, 1e-6, 1e-6,
                                        INTG_DOUBLE);
        memset(wg, 0, N * N * sizeof(tags_cdouble));
        if (!rc) rc = fill_incidence_imm(wg, e, m, nodes, n);
        if (!rc) rc = fill_impedance_imm(wg, zl, zt, m, n);
        memset(ie, 0, N * sizeof(tags_cdouble));
        ie[0] = 1.0;
        if (!rc) rc = solve_immittance(wg, ie, m, n);
        if (rc) {
            fprintf(stderr, "call failed: %d\n", rc);
            return 1;
        }
        printf("%.17g %.17g %.17g\n", f, creal(ie[0]), cimag(ie[0]));
    }
    free(zl);
    free(zt);
    free(wg);
    free(ie);
    return 0;
}
