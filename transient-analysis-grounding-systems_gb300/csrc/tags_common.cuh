// Shared device helpers for the GB300 HEM path: complex arithmetic on
// double2/float2, the segment record, launch checks and status words.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define TAGS_HD __host__ __device__ __forceinline__
#define TAGS_D __device__ __forceinline__

// Same field order and size (11 doubles, 88 bytes) as the reference's
// Electrode (src/electrode.h:33-45); arrays of it cross the C-ABI unchanged.
struct Seg {
    double a[3];   // start point
    double b[3];   // end point
    double mid[3]; // middle point
    double len;
    double radius;
};
static_assert(sizeof(Seg) == 88, "Seg must match the reference Electrode layout");

// Status bits a kernel may raise in its status word (never traps).
enum : int {
    TAGS_ST_OK = 0,
    TAGS_ST_DEGENERATE_PAIR = 1,   // overlapping/coincident segments: integral diverges
    TAGS_ST_ZERO_PIVOT = 2,        // exact zero pivot in a factorisation
    TAGS_ST_NONFINITE = 4,         // NaN/Inf met in a result
    TAGS_ST_NO_CONVERGENCE = 8,    // iterative refinement did not reach its tolerance
    TAGS_ST_BAD_ARG = 16,
};

// Physical constants of the reference (src/auxiliary.c:17-21).
#define TAGS_PI 3.1415926535897932384626433832795029
#define TAGS_TWO_PI 6.283185307179586476925286766559
#define TAGS_FOUR_PI 12.5663706143591729538505735331
#define TAGS_MU0 1.256637061435917e-6
#define TAGS_EPS0 8.854187817620e-12
#define TAGS_DBL_EPSILON 2.2204460492503131e-16

// ---- complex helpers ------------------------------------------------------
TAGS_HD double2 cz(double re, double im) { return make_double2(re, im); }
TAGS_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
TAGS_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
TAGS_HD double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
TAGS_HD double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
TAGS_HD double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// c + a*b with four fused multiply-adds
TAGS_HD double2 cfma(double2 a, double2 b, double2 c) {
    c.x = fma(a.x, b.x, c.x);
    c.x = fma(-a.y, b.y, c.x);
    c.y = fma(a.x, b.y, c.y);
    c.y = fma(a.y, b.x, c.y);
    return c;
}
TAGS_HD double2 cdiv(double2 a, double2 b) {
    // Smith's algorithm: avoids overflow of |b|^2
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    } else {
        double r = b.x / b.y, d = b.x * r + b.y;
        return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
    }
}
TAGS_HD double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
TAGS_HD double cabs1(double2 a) { return fabs(a.x) + fabs(a.y); }

TAGS_HD float2 fz(float re, float im) { return make_float2(re, im); }
TAGS_HD float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
TAGS_HD float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
TAGS_HD float2 fmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
TAGS_HD float2 ffmac(float2 a, float2 b, float2 c) {
    c.x = fmaf(a.x, b.x, c.x);
    c.x = fmaf(-a.y, b.y, c.x);
    c.y = fmaf(a.x, b.y, c.y);
    c.y = fmaf(a.y, b.x, c.y);
    return c;
}

// e^{z} for complex z in FP64 (CUDA's exp and sincos).
TAGS_D double2 cexp_d(double2 z) {
    double e = exp(z.x), s, c;
    sincos(z.y, &s, &c);
    return make_double2(e * c, e * s);
}

TAGS_D void raise_status(int* status, int bits) {
    if (status) atomicOr(status, bits);
}

// Host-side launch check used by the C-ABI layer.
#define TAGS_CUDA_OK(expr)                                  \
    do {                                                    \
        cudaError_t _e = (expr);                            \
        if (_e != cudaSuccess) return tags_fail_cuda(_e, #expr, __FILE__, __LINE__); \
    } while (0)

int tags_fail_cuda(cudaError_t e, const char* what, const char* file, int line);
