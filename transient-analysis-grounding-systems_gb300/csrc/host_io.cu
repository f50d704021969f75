// Host-side helpers of the reference kept as C-ABI exports with its names,
// so callers that relink find them here too (no device code):
//   electrodes_file      src/electrode.c:45-80  (CSV "x0, y0, z0, x1, y1, z1, r" per line)
//   nodes_file           src/electrode.c:82-101 (CSV "x, y, z" per line)
//   alipio_soil          src/auxiliary.c:60-70
//   smith_longmire_soil  src/auxiliary.c:72-93
//   heidler              src/auxiliary.c:331-336
// Return codes follow the reference: -10 when the file cannot be opened, the
// fscanf shortfall (count read - count expected) of the first bad line, or
// populate_electrode's error for a degenerate segment.
#include <cmath>
#include <complex>
#include <cstdio>

#include "tags_common.cuh"
#include "../../include/tags_gpu.h"
#include "plan.h"

using zd = std::complex<double>;

namespace {

// src/electrode.c:12-32 (populate_electrode): 1 for coincident end points
// (within DBL_EPSILON per coordinate), 2 for a radius <= 0, else the
// segment's geometry with its length as the root of the summed squares
// (src/auxiliary.c:110-125).
int populate(Electrode* e, const double* a, const double* b, double r) {
    bool same = true;
    for (int d = 0; d < 3; ++d)
        if (std::fabs(a[d] - b[d]) > TAGS_DBL_EPSILON) same = false;
    if (same) {
        tags_msg("Error: start_point and end_point are equal.\n");
        return 1;
    }
    if (r <= 0) {
        tags_msg("Error: radius < 0.\n");
        return 2;
    }
    double len2 = 0.0;
    for (int d = 0; d < 3; ++d) len2 += (a[d] - b[d]) * (a[d] - b[d]);
    e->radius = r;
    e->length = std::sqrt(len2);
    for (int d = 0; d < 3; ++d) {
        e->start_point[d] = a[d];
        e->end_point[d] = b[d];
        e->middle_point[d] = (a[d] + b[d]) / 2.0;
    }
    return 0;
}

}  // namespace

extern "C" int electrodes_file(const char file_name[], Electrode* electrodes, size_t num_electrodes) {
    FILE* f = std::fopen(file_name, "r");
    if (!f) {
        char msg[320];
        std::snprintf(msg, sizeof(msg), "Cannot open file %s\n", file_name);
        tags_msg(msg);
        return -10;
    }
    const int want = 7;
    int got = want, bad = 0;
    for (size_t i = 0; i < num_electrodes; ++i) {
        double a[3], b[3], r;
        got = std::fscanf(f, "%lf, %lf, %lf, %lf, %lf, %lf, %lf", &a[0], &a[1], &a[2], &b[0], &b[1], &b[2], &r);
        if (got != want) {
            char msg[320];
            std::snprintf(msg, sizeof(msg), "error reading line %i of file %s\n", (int)(i + 1), file_name);
            tags_msg(msg);
            break;
        }
        bad = populate(&electrodes[i], a, b, r);
        if (bad) {
            char msg[320];
            std::snprintf(msg, sizeof(msg), "Bad input: could not create electrode %i from file %s\n", (int)(i + 1),
                          file_name);
            tags_msg(msg);
            break;
        }
    }
    std::fclose(f);
    return bad ? bad : got - want;
}

extern "C" int nodes_file(const char file_name[], double* nodes, size_t num_nodes) {
    FILE* f = std::fopen(file_name, "r");
    if (!f) {
        char msg[320];
        std::snprintf(msg, sizeof(msg), "Cannot open file %s\n", file_name);
        tags_msg(msg);
        return -10;
    }
    int got = 3;
    for (size_t i = 0; i < num_nodes; ++i) {
        got = std::fscanf(f, "%lf, %lf, %lf", &nodes[3 * i], &nodes[3 * i + 1], &nodes[3 * i + 2]);
        if (got != 3) {
            char msg[320];
            std::snprintf(msg, sizeof(msg), "error reading line %i of file %s\n", (int)(i + 1), file_name);
            tags_msg(msg);
            break;
        }
    }
    std::fclose(f);
    return got - 3;
}

// Alipio-Visacro frequency-dependent soil: sigma = sigma0 (1 + h (f / 1 MHz)^g),
// eps_r = eps_ratio + tan(pi g / 2) sigma0 h f^(g - 1) / (2 pi eps0 (1 MHz)^g),
// f = s / (2 pi j).
extern "C" int alipio_soil(tags_cdouble* sigma, tags_cdouble* epsr, double sigma0, tags_cdouble s, double h,
                           double g, double eps_ratio) {
    if (!sigma || !epsr) return tags_fail(TAGS_E_ARG, "null pointer argument");
    const zd f = zd(s.re, s.im) / (TAGS_TWO_PI * zd(0.0, 1.0));
    const zd sg = sigma0 + sigma0 * h * std::pow(f / 1e6, g);
    const double t = std::tan(TAGS_PI * g / 2) / (TAGS_TWO_PI * TAGS_EPS0 * std::pow(1e6, g));
    const zd er = eps_ratio + t * sigma0 * h * std::pow(f, g - 1.0);
    *sigma = {sg.real(), sg.imag()};
    *epsr = {er.real(), er.imag()};
    return 0;
}

// Smith-Longmire soil model: 13 Debye-like terms with relaxation frequencies
// F_i = (125 sigma0)^0.8312 10^i and the published weights a_i.
extern "C" int smith_longmire_soil(tags_cdouble* sigma, tags_cdouble* epsr, double sigma0, tags_cdouble s,
                                   double erinf) {
    if (!sigma || !epsr) return tags_fail(TAGS_E_ARG, "null pointer argument");
    static const double a[13] = {3.4e6, 2.74e5, 2.58e4, 3.38e3, 5.26e2, 1.33e2, 2.72e1,
                                 1.25e1, 4.8e0, 2.17e0, 9.8e-1, 3.92e-1, 1.73e-1};
    const zd sv(s.re, s.im);
    const zd fdc = std::pow(zd(125.0 * sigma0, 0.0), zd(0.8312, 0.0));
    zd se = 0.0, ss = 0.0;
    for (int i = 0; i < 13; ++i) {
        const zd F = fdc * std::pow(zd(10.0, 0.0), zd((double)i, 0.0));
        const zd r = sv / (zd(0.0, 1.0) * TAGS_TWO_PI * F);
        const zd r2 = r * r;
        const zd den = 1.0 + r2;
        se += a[i] / den;
        ss += a[i] * F * (r2 / den);
    }
    const zd er = erinf + se, sg = sigma0 + TAGS_TWO_PI * TAGS_EPS0 * ss;
    *sigma = {sg.real(), sg.imag()};
    *epsr = {er.real(), er.imag()};
    return 0;
}

// Heidler lightning current: imax / xi (t/tau1)^n / (1 + (t/tau1)^n) e^{-t/tau2},
// xi = e^{-(tau1/tau2) (n tau2/tau1)^(1/n)} the peak correction factor.
extern "C" double heidler(double t, double imax, double tau1, double tau2, double n) {
    const double xi = std::exp(-(tau1 / tau2) * std::pow(n * tau2 / tau1, 1.0 / n));
    const double u = std::pow(t / tau1, n);
    return imax / xi * u / (1.0 + u) * std::exp(-t / tau2);
}
