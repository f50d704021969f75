// Thin-wire impedance fill (ZL, ZT) for the HEM hot path on GB300.
//
// Replaces the reference's calculate_impedances / impedances_images
// (src/electrode.c:304-431), which call an adaptive cubature per segment pair
// (src/electrode.c:247-302). Here every pair integral
//     J = \int_0^1 \int_0^1 e^{-gamma r(t0,t1)} / r  dt0 dt1
// (t0 on the receiver, t1 on the sender; INTG_DOUBLE, src/electrode.c:176-197)
// is evaluated by a geometry-driven fixed-order rule:
//   * pairs sharing an endpoint: a Duffy split at the shared corner reduces J
//     exactly to two 1-D integrals of phi(gamma rho(w)) / rho(w),
//     phi(x) = (1 - e^{-x}) / x, which are smooth -> Gauss-Legendre;
//   * other pairs: tensor Gauss-Legendre whose order follows the ratio
//     (minimum distance / longer length) and |gamma| * length; pairs closer
//     than two lengths are split into panels so every panel pair is >= 2
//     panel lengths apart;
//   * the diagonal keeps the reference's static closed form
//     (self_integral, src/electrode.c:238-245, used at :346-348).
// INTG_MHEM is the static kernel 1/r (the reference's logNf, :220-236, is its
// exact inner integral), INTG_SINGLE the 1-D integral to the receiver's
// midpoint (:199-218), INTG_NONE the midpoint distance (:267-270).
// The scaling and the quirks follow the reference: |cos theta| of the
// direction vectors, ZL = 0 when cos < DBL_EPSILON (direct) and image ZL only
// when cos > DBL_EPSILON, images include k = i and accumulate.
// The mixed form's fill (entries as float pairs hi + lo, ~1e-14 of the FP64
// fill): regular pairs by a moment expansion about the nearest multiple of
// 1/8 m (FP64 moments once per plan, k_moments; a per-sample series in float
// pairs times a per-sample FP64 table, k_fill_moment), pairs sharing an
// endpoint by the FP64 series of their Duffy moments (k_touch_moments once,
// k_fill_special64 per sample), the self term in closed form; the upper
// triangle and the row statistics' partials by k_zmirror. k_fill_mixed (FP32
// quadrature) covers the samples whose series would need more than MOM_N
// terms.
#include <map>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"

namespace {

constexpr int QMAX = 40;                      // largest Gauss-Legendre order tabulated
constexpr int GL_TOTAL = QMAX * (QMAX + 1) / 2;

__device__ double g_glx[GL_TOTAL];            // nodes on [0,1], order q at q(q-1)/2
__device__ double g_glw[GL_TOTAL];            // weights on [0,1]
constexpr int MOM_N = 24;                     // terms of the moment expansion stored (mixed fill)
constexpr double MOM_H = 0.125;               // spacing of its expansion centres (m)
constexpr int QMIX = 24;                      // largest order of the FP32 fill
constexpr int GL_MIX = QMIX * (QMIX + 1) / 2;
__device__ float g_glxm[GL_MIX];              // FP32 fill: nodes shifted to [-1/2, 1/2], orders 1..QMIX
__device__ float g_glwm[GL_MIX];

TAGS_D int gl_off(int q) { return q * (q - 1) / 2; }

struct GLTab {
    const double* x;
    const double* w;
};

// ---- geometry ---------------------------------------------------------------

TAGS_D void ld_seg(const double* __restrict__ p, Seg& s) {
#pragma unroll
    for (int c = 0; c < 11; ++c) (&s.a[0])[c] = __ldg(p + c);
}

TAGS_D double dot3(const double* u, const double* v) { return u[0] * v[0] + u[1] * v[1] + u[2] * v[2]; }

// Minimum distance between segments [p0,p1] and [q0,q1] (closest points of
// two segments, clamped parameters).
TAGS_D double seg_seg_dist(const double* p0, const double* p1, const double* q0, const double* q1) {
    double d1[3], d2[3], r[3];
    for (int c = 0; c < 3; ++c) { d1[c] = p1[c] - p0[c]; d2[c] = q1[c] - q0[c]; r[c] = p0[c] - q0[c]; }
    double a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
    double s, t;
    double c_ = dot3(d1, r), b = dot3(d1, d2);
    double den = a * e - b * b;
    if (den > 1e-14 * a * e) s = fmin(fmax((b * f - c_ * e) / den, 0.0), 1.0);
    else s = 0.0;
    t = (b * s + f) / e;
    if (t < 0.0) { t = 0.0; s = fmin(fmax(-c_ / a, 0.0), 1.0); }
    else if (t > 1.0) { t = 1.0; s = fmin(fmax((b - c_) / a, 0.0), 1.0); }
    double dd = 0.0;
    for (int c = 0; c < 3; ++c) {
        double v = r[c] + s * d1[c] - t * d2[c];
        dd += v * v;
    }
    return sqrt(dd);
}

// Shared endpoint of receiver R and sender S: ia/ib = 0 (start) or 1 (end).
TAGS_D bool touching(const Seg& R, const Seg& S, double tol, int& ia, int& ib) {
    const double* ra[2] = {R.a, R.b};
    const double* sb[2] = {S.a, S.b};
    for (int x = 0; x < 2; ++x)
        for (int y = 0; y < 2; ++y) {
            double d = fmax(fabs(ra[x][0] - sb[y][0]), fmax(fabs(ra[x][1] - sb[y][1]), fabs(ra[x][2] - sb[y][2])));
            if (d <= tol) { ia = x; ib = y; return true; }
        }
    return false;
}

// (1 - e^{-x}) / x for complex x.
TAGS_D double2 phi_c(double2 x) {
    double ax = fabs(x.x) + fabs(x.y);
    if (ax < 0.1) {
        // Taylor series: sum_k (-x)^k / (k+1)!, error < 0.1^10/10! ~ 3e-17
        double2 term = cz(1.0, 0.0), acc = cz(1.0, 0.0);
        for (int k = 1; k <= 9; ++k) {
            term = cscale(cmul(term, x), -1.0 / (double)(k + 1));
            acc = cadd(acc, term);
        }
        return acc;
    }
    double2 e = cexp_d(cneg(x));
    return cdiv(cz(1.0 - e.x, -e.y), x);
}

// ---- quadrature pieces ---------------------------------------------------------

// sum over a (P x P)-panel tensor Gauss-Legendre rule of order q of
// f(r) = e^{-gamma r}/r (or 1/r when stat) over [0,1]^2 with
// r = |R(t0) - S(t1)|.
TAGS_D double2 j_tensor(const Seg& R, const Seg& S, double2 gamma, bool stat, int q, int P,
                        const GLTab& gl) {
    const double* x = gl.x + gl_off(q);
    const double* w = gl.w + gl_off(q);
    double dr[3], ds[3];
    for (int c = 0; c < 3; ++c) { dr[c] = R.b[c] - R.a[c]; ds[c] = S.b[c] - S.a[c]; }
    const double h = 1.0 / (double)P;
    double2 acc = cz(0.0, 0.0);
    for (int pi = 0; pi < P; ++pi) {
        for (int qi = 0; qi < q; ++qi) {
            double t0 = (pi + x[qi]) * h;
            double pr[3] = {R.a[0] + t0 * dr[0], R.a[1] + t0 * dr[1], R.a[2] + t0 * dr[2]};
            double w0 = w[qi] * h;
            for (int pj = 0; pj < P; ++pj) {
                double2 row = cz(0.0, 0.0);
                for (int qj = 0; qj < q; ++qj) {
                    double t1 = (pj + x[qj]) * h;
                    double dx = pr[0] - (S.a[0] + t1 * ds[0]);
                    double dy = pr[1] - (S.a[1] + t1 * ds[1]);
                    double dz = pr[2] - (S.a[2] + t1 * ds[2]);
                    double r = sqrt(dx * dx + dy * dy + dz * dz);
                    if (r < TAGS_DBL_EPSILON) r = R.radius;   // src/electrode.c:192
                    double ir = w[qj] / r;
                    if (stat) {
                        row.x += ir;
                    } else {
                        double2 e = cexp_d(cz(-gamma.x * r, -gamma.y * r));
                        row.x = fma(e.x, ir, row.x);
                        row.y = fma(e.y, ir, row.y);
                    }
                }
                acc.x = fma(row.x, w0 * h, acc.x);
                acc.y = fma(row.y, w0 * h, acc.y);
            }
        }
    }
    return acc;
}

// Pair sharing a corner: R from the corner along a, S along b (full lengths).
TAGS_D double2 j_touch(const Seg& R, const Seg& S, int ia, int ib, double2 gamma, bool stat, int q,
                       const GLTab& gl) {
    double a[3], b[3];
    for (int c = 0; c < 3; ++c) {
        a[c] = ia == 0 ? R.b[c] - R.a[c] : R.a[c] - R.b[c];
        b[c] = ib == 0 ? S.b[c] - S.a[c] : S.a[c] - S.b[c];
    }
    const double* x = gl.x + gl_off(q);
    const double* w = gl.w + gl_off(q);
    double2 acc = cz(0.0, 0.0);
    for (int qi = 0; qi < q; ++qi) {
        double t = x[qi];
        double u1[3] = {a[0] - t * b[0], a[1] - t * b[1], a[2] - t * b[2]};
        double u2[3] = {t * a[0] - b[0], t * a[1] - b[1], t * a[2] - b[2]};
        double rho1 = sqrt(dot3(u1, u1)), rho2 = sqrt(dot3(u2, u2));
        if (stat) {
            acc.x += w[qi] * (1.0 / rho1 + 1.0 / rho2);
        } else {
            double2 p1 = phi_c(cz(gamma.x * rho1, gamma.y * rho1));
            double2 p2 = phi_c(cz(gamma.x * rho2, gamma.y * rho2));
            acc = cadd(acc, cscale(p1, w[qi] / rho1));
            acc = cadd(acc, cscale(p2, w[qi] / rho2));
        }
    }
    return acc;
}

// 1-D rule for INTG_SINGLE: \int_0^1 e^{-gamma r}/r dt1, r = |S(t1) - mid(R)|,
// r clamped to DBL_EPSILON (src/electrode.c:212-213).
TAGS_D double2 j_single(const Seg& R, const Seg& S, double2 gamma, int q, int P, const GLTab& gl) {
    const double* x = gl.x + gl_off(q);
    const double* w = gl.w + gl_off(q);
    const double h = 1.0 / (double)P;
    double2 acc = cz(0.0, 0.0);
    for (int pj = 0; pj < P; ++pj)
        for (int qj = 0; qj < q; ++qj) {
            double t1 = (pj + x[qj]) * h;
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = S.a[c] + t1 * (S.b[c] - S.a[c]) - R.mid[c];
            double r = sqrt(dot3(d, d));
            if (r < TAGS_DBL_EPSILON) r = TAGS_DBL_EPSILON;
            double2 e = cexp_d(cz(-gamma.x * r, -gamma.y * r));
            acc = cadd(acc, cscale(e, w[qj] * h / r));
        }
    return acc;
}

// Order of the tensor rule for a pair at distance ratio `ratio` >= 2 and
// |gamma| * length `gl`; `tight` selects the ~1e-12 table (FP64 plain form),
// otherwise the ~3e-8 table.
TAGS_D int order_for(double ratio, double gl, bool tight) {
    int base;
    if (tight) base = ratio >= 16.0 ? 4 : ratio >= 8.0 ? 5 : ratio >= 4.0 ? 6 : 8;
    else base = ratio >= 8.0 ? 3 : ratio >= 4.0 ? 4 : 5;
    // clamped before the conversion: a huge (or NaN) |gamma| L gives QMAX, never an overflow
    const int extra = (int)ceil(fmin((tight ? 1.5 : 1.0) * gl, (double)QMAX));
    const int q = base + extra;
    return q > QMAX ? QMAX : q;
}

// Reference-scaled pair integral `intg` of src/electrode.c:247-302 (result
// already multiplied by the lengths), for integration type `itype`.
TAGS_D double2 pair_integral(const Seg& S, const Seg& R, double2 gamma, int itype, bool tight,
                             const GLTab& gl, int* status) {
    if (itype == TAGS_INTG_NONE) {
        double d[3] = {S.mid[0] - R.mid[0], S.mid[1] - R.mid[1], S.mid[2] - R.mid[2]};
        return cz(sqrt(dot3(d, d)), 0.0);
    }
    const bool stat = (itype == TAGS_INTG_MHEM);
    const double lmax = fmax(S.len, R.len);
    const double gabs = stat ? 0.0 : sqrt(cabs2(gamma));
    if (itype == TAGS_INTG_SINGLE) {
        // distance from the receiver midpoint to the sender segment
        double dist = seg_seg_dist(R.mid, R.mid, S.a, S.b);
        double ratio = dist / S.len;
        int P = ratio >= 2.0 ? 1 : (int)fmin(32.0, ceil(2.0 / fmax(ratio, 1e-3)));
        int q = order_for(fmax(ratio * P, 2.0), gabs * S.len / P, tight);
        double2 j = j_single(R, S, gamma, q, P, gl);
        return cscale(j, S.len);
    }
    int ia, ib;
    double2 J;
    if (touching(R, S, 1e-9 * lmax, ia, ib)) {
        // both ends shared: coincident segments, the integral diverges
        const double* ro = ia == 0 ? R.b : R.a;
        const double* so = ib == 0 ? S.b : S.a;
        double od = fmax(fabs(ro[0] - so[0]), fmax(fabs(ro[1] - so[1]), fabs(ro[2] - so[2])));
        if (od <= 1e-9 * lmax) {
            raise_status(status, TAGS_ST_DEGENERATE_PAIR);
            return cz(nan(""), nan(""));
        }
        const int glen = (int)ceil(fmin(gabs * lmax, (double)QMAX));    // clamped before the conversion
        int q = 16 + 2 * glen;
        if (!tight) q = 10 + glen;
        if (q > QMAX) q = QMAX;
        J = j_touch(R, S, ia, ib, gamma, stat, q, gl);
    } else {
        double dmin = seg_seg_dist(R.a, R.b, S.a, S.b);
        double ratio = dmin / lmax;
        if (dmin <= 1e-12 * lmax) {
            raise_status(status, TAGS_ST_DEGENERATE_PAIR);
            return cz(nan(""), nan(""));
        }
        int P = 1;
        if (ratio < 2.0) P = (int)fmin(32.0, ceil(2.0 / ratio));
        int q = order_for(ratio * P, gabs * lmax / P, tight);
        J = j_tensor(R, S, gamma, stat, q, P, gl);
    }
    return cscale(J, R.len * S.len);
}

// self_integral (src/electrode.c:238-245)
TAGS_D double self_integral_d(const Seg& s) {
    double ls = s.len;
    double k1 = s.radius / ls;
    double k2 = sqrt(1.0 + k1 * k1);
    return 2.0 * ls * (log((k2 + 1.0) / k1) - k2 + k1);
}

TAGS_D void pair_index(long long p, int m, int& i, int& k) {
    // p enumerates (i, k), k >= i, column by column: start(i) = i(2m - i + 1)/2.
    // FP32 estimate (the FP64 pipe is ~1/58 of FP32 here), made exact by the
    // integer corrections below.
    const float b = 2.f * m + 1.f;
    int ii = (int)floorf((b - sqrtf(fmaxf(b * b - 8.f * (float)p, 0.f))) * 0.5f);
    if (ii < 0) ii = 0;
    if (ii > m - 1) ii = m - 1;
    while (ii > 0 && (long long)ii * (2LL * m - ii + 1) / 2 > p) --ii;
    while (ii < m - 1 && (long long)(ii + 1) * (2LL * m - ii) / 2 <= p) ++ii;
    i = ii;
    k = ii + (int)(p - (long long)ii * (2LL * m - ii + 1) / 2);
}

TAGS_D void store(double2* base, long long idx, double2 v, bool acc) {
    if (acc) {
        double2 o = base[idx];
        base[idx] = cadd(o, v);
    } else {
        base[idx] = v;
    }
}

// One thread per (pair, sample). Writes the lower triangle (row k >= col i).
__global__ void __launch_bounds__(128) k_fill_fp64(const double* __restrict__ elec,
                                                   const double* __restrict__ img, int m,
                                                   const SampleCoef* __restrict__ coef, int nsamp,
                                                   FillOut out, int mode, int itype, int tight,
                                                   int* status) {
    __shared__ double sx[GL_TOTAL], sw[GL_TOTAL];
    for (int t = threadIdx.x; t < GL_TOTAL; t += blockDim.x) { sx[t] = g_glx[t]; sw[t] = g_glw[t]; }
    __syncthreads();
    GLTab gl{sx, sw};
    const long long npairs = (long long)m * (m + 1) / 2;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int smp = blockIdx.y;
    if (p >= npairs || smp >= nsamp) return;
    int i, k;
    pair_index(p, m, i, k);
    const SampleCoef c = coef[smp];
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    double2 zl = cz(0.0, 0.0), zt = cz(0.0, 0.0);
    const bool scaled = (itype == TAGS_INTG_DOUBLE || itype == TAGS_INTG_SINGLE);
    const double2 cL = scaled ? c.cL : cz(1.0, 0.0);
    const double2 cT = scaled ? c.cT : cz(1.0, 0.0);
    const double ds[3] = {S.b[0] - S.a[0], S.b[1] - S.a[1], S.b[2] - S.a[2]};
    if (mode & TAGS_FILL_DIRECT) {
        if (i == k) {
            double intg = self_integral_d(S);
            zl = cscale(cL, intg);
            zt = cscale(cT, intg / (S.len * S.len));
        } else {
            ld_seg(elec + 11LL * k, R);
            double2 intg = pair_integral(S, R, c.gamma, itype, tight, gl, status);
            double cost = 0.0;
            for (int d = 0; d < 3; ++d) cost += ds[d] * (R.b[d] - R.a[d]);
            cost = fabs(cost);
            zt = cmul(cscale(cT, 1.0 / (S.len * R.len)), intg);
            if (cost < TAGS_DBL_EPSILON) zl = cz(0.0, 0.0);
            else zl = cscale(cmul(cL, intg), cost / (S.len * R.len));
        }
    }
    if (mode & TAGS_FILL_IMAGE) {
        ld_seg(img + 11LL * k, R);
        const double2 cLi = scaled ? c.cLi : cz(1.0, 0.0);
        const double2 cTi = scaled ? c.cTi : cz(1.0, 0.0);
        double2 intg = pair_integral(S, R, c.gamma, itype, tight, gl, status);
        double cost = 0.0;
        for (int d = 0; d < 3; ++d) cost += ds[d] * (R.b[d] - R.a[d]);
        cost = fabs(cost);
        zt = cadd(zt, cmul(cscale(cTi, 1.0 / (S.len * R.len)), intg));
        if (cost > TAGS_DBL_EPSILON) zl = cadd(zl, cscale(cmul(cLi, intg), cost / (S.len * R.len)));
    }
    if (!isfinite(zl.x + zl.y + zt.x + zt.y)) raise_status(status, TAGS_ST_NONFINITE);
    const bool acc = out.accumulate != 0;
    const double sg = out.sign;
    zl = cscale(zl, sg);
    zt = cscale(zt, sg);
    const long long bs = out.batch_stride * smp;
    if (out.zl) {
        store(out.zl + bs, (long long)(out.row0_l + k) + out.ld * (out.col0_l + i), zl, acc);
        if (out.mirror && k != i) store(out.zl + bs, (long long)(out.row0_l + i) + out.ld * (out.col0_l + k), zl, acc);
    }
    if (out.zt) {
        store(out.zt + bs, (long long)(out.row0_t + k) + out.ld * (out.col0_t + i), zt, acc);
        if (out.mirror && k != i) store(out.zt + bs, (long long)(out.row0_t + i) + out.ld * (out.col0_t + k), zt, acc);
    }
}

// Path/electrode double integrals for the path voltage: thread per
// (electrode, path), grid.y over samples; jj[(smp * npaths + l) * m + e] =
// \int_0^1 \int_0^1 e^{-gamma r}/r (the pair rule above, tight table).
__global__ void __launch_bounds__(128) k_path_pairs(const double* __restrict__ elec, int m,
                                                    const double* __restrict__ paths, int npaths,
                                                    const SampleCoef* __restrict__ coef, double2* __restrict__ jj,
                                                    int* status) {
    __shared__ double sx[GL_TOTAL], sw[GL_TOTAL];
    for (int t = threadIdx.x; t < GL_TOTAL; t += blockDim.x) { sx[t] = g_glx[t]; sw[t] = g_glw[t]; }
    __syncthreads();
    GLTab gl{sx, sw};
    const long long n = (long long)m * npaths;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int smp = blockIdx.y;
    if (idx >= n) return;
    const int e = (int)(idx % m), l = (int)(idx / m);
    Seg S, R;
    ld_seg(paths + 11LL * l, S);
    ld_seg(elec + 11LL * e, R);
    const double2 j = pair_integral(S, R, coef[smp].gamma, TAGS_INTG_DOUBLE, true, gl, status);
    jj[((long long)smp * npaths + l) * m + e] = cscale(j, 1.0 / (S.len * R.len));
}

// ---- mixed form: plan-time pair classification + FP32 regular-pair fill --------

// Pair code (geometry only, computed once per plan):
//   bit 15      endpoints touch: Duffy rule in FP64
//   bit 14      coincident/overlapping segments (divergent integral)
//   bits 6..11  base Gauss-Legendre order of a panel pair
//   bits 0..5   panels per segment P (1..32)
constexpr uint16_t PC_TOUCH = 0x8000, PC_DEGEN = 0x4000;

TAGS_D uint16_t classify_pair(const Seg& S, const Seg& R) {
    const double lmax = fmax(S.len, R.len);
    int ia, ib;
    if (touching(R, S, 1e-9 * lmax, ia, ib)) {
        const double* ro = ia == 0 ? R.b : R.a;
        const double* so = ib == 0 ? S.b : S.a;
        double od = fmax(fabs(ro[0] - so[0]), fmax(fabs(ro[1] - so[1]), fabs(ro[2] - so[2])));
        return od <= 1e-9 * lmax ? PC_DEGEN : PC_TOUCH;
    }
    double dmin = seg_seg_dist(R.a, R.b, S.a, S.b);
    if (dmin <= 1e-12 * lmax) return PC_DEGEN;
    double ratio = dmin / lmax;
    int P = ratio >= 2.0 ? 1 : (int)fmin(32.0, ceil(2.0 / ratio));
    double rp = ratio * P;
    int qg = rp >= 8.0 ? 3 : rp >= 4.0 ? 4 : 5;
    return (uint16_t)(P | (qg << 6));
}

// Geometry of one (pair, kind) for the FP32 path, computed once per plan:
// receiver-minus-sender midpoint vector, its length split into two floats
// (hi + lo, ~2^-48 relative), and the ZL factor |d_i . d_k| (zero where the
// reference drops ZL: cos < DBL_EPSILON direct, cos <= DBL_EPSILON images).
struct PairRec {
    float dx, dy, dz, rch, rcl, fl;
};

__global__ void k_pair_plan(const double* __restrict__ elec, const double* __restrict__ img, int m, int has_img,
                            uint16_t* __restrict__ codes, PairRec* __restrict__ recs, int* __restrict__ ntouch,
                            int* __restrict__ touch_list) {
    const long long npairs = (long long)m * (m + 1) / 2;
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int i, k;
    pair_index(p, m, i, k);
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    uint16_t cc[2] = {0, 0};
    int special = 0;
    for (int kind = 0; kind < 2; ++kind) {
        PairRec rc{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if ((kind == 0 && k != i) || (kind == 1 && has_img)) {
            ld_seg((kind == 0 ? elec : img) + 11LL * k, R);
            cc[kind] = classify_pair(S, R);
            if (cc[kind] & (PC_TOUCH | PC_DEGEN)) special |= 1 << kind;
            double d[3] = {R.mid[0] - S.mid[0], R.mid[1] - S.mid[1], R.mid[2] - S.mid[2]};
            double r = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            float rh = (float)r;
            double cost = 0.0;
            for (int c = 0; c < 3; ++c) cost += (S.b[c] - S.a[c]) * (R.b[c] - R.a[c]);
            cost = fabs(cost);
            bool keep = kind == 0 ? !(cost < TAGS_DBL_EPSILON) : (cost > TAGS_DBL_EPSILON);
            rc = PairRec{(float)d[0], (float)d[1], (float)d[2], rh, (float)(r - (double)rh), keep ? (float)cost : 0.f};
        }
        recs[2 * p + kind] = rc;
    }
    codes[2 * p] = cc[0];
    codes[2 * p + 1] = cc[1];
    if (special) {
        int slot = atomicAdd(ntouch, 1);
        touch_list[2 * slot] = (int)p;
        touch_list[2 * slot + 1] = special;
    }
}

// Per-sample constants of the FP32 path: gamma as float pairs (hi + lo) and
// the scale factors in FP32.
struct SampleF32 {
    float grh, grl, gih, gil;
    float2 cL, cT, cLi, cTi;
};

__global__ void k_coef32(const SampleCoef* __restrict__ coef, int nsamp, SampleF32* __restrict__ out) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsamp) return;
    SampleCoef c = coef[q];
    SampleF32 o;
    o.grh = (float)c.gamma.x;
    o.grl = (float)(c.gamma.x - (double)o.grh);
    o.gih = (float)c.gamma.y;
    o.gil = (float)(c.gamma.y - (double)o.gih);
    o.cL = make_float2((float)c.cL.x, (float)c.cL.y);
    o.cT = make_float2((float)c.cT.x, (float)c.cT.y);
    o.cLi = make_float2((float)c.cLi.x, (float)c.cLi.y);
    o.cTi = make_float2((float)c.cTi.x, (float)c.cTi.y);
    out[q] = o;
}

// e^{-gamma r} in FP32 from float pairs (r = rh + rl, gamma = (grh + grl) +
// j (gih + gil)): the exponent and the phase are formed as float pairs
// (error-free products) and reduced exactly (2^-t split into integer and
// fraction, phase modulo 2 pi with a two-float 2 pi), so only the small
// reduced arguments meet FP32 rounding.
TAGS_D float2 anchor_df(float grh, float grl, float gih, float gil, float rh, float rl) {
    const float L2E_HI = 1.44269502162933349609f, L2E_LO = 1.925963033500011e-8f;
    const float TPI_HI = 6.28318548202514648438f, TPI_LO = -1.7484555314695172e-7f;
    // t = Re(gamma) r log2(e)
    float q = grh * rh;
    float qe = fmaf(grh, rh, -q) + fmaf(grh, rl, grl * rh);
    float th = q * L2E_HI;
    float te = fmaf(q, L2E_HI, -th) + fmaf(q, L2E_LO, qe * L2E_HI);
    float n = floorf(th);
    float f = (th - n) + te;
    float mag = ldexpf(exp2f(-f), -(int)fminf(n, 1000.f));
    // phase = Im(gamma) r, modulo 2 pi
    float p = gih * rh;
    float pe = fmaf(gih, rh, -p) + fmaf(gih, rl, gil * rh);
    float kq = rintf(p * 0.15915494309189535f);
    float red = fmaf(-kq, TPI_HI, p);
    red = fmaf(-kq, TPI_LO, red) + pe;
    float sn, cs;
    sincosf(red, &sn, &cs);
    return make_float2(mag * cs, -mag * sn);
}

// 2^x with the special-function unit's approximation (PTX ex2.approx.ftz:
// a few ulp, results below 2^-126 flushed to zero, which only happens for
// terms that are negligible against the panel's anchor).
TAGS_D float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr int FILL_WARPS = 4;              // warps per CTA
constexpr int FILL_SUB = 8;                // rows of one write sub-tile
constexpr int FILL_GEO = QMIX * QMIX;      // points of one panel pair, at most

struct FillWarpSmem {
    float2 geo[FILL_GEO];                  // (r_p - r_c, w_i w_j / r_p) of the current panel pair
    float4 anc[32];                        // panel-pair anchors (midpoint vector, |.| high part) of a chunk
    float ancl[32];                        // |.| low part
    float2 zl[FILL_SUB][33], zt[FILL_SUB][33];   // a sub-tile of outputs, [row][sample]
};

// Lower-triangle tiles of 32 rows: tile t -> (row block kb, column i); block
// rows kb < KB - 1 hold columns 0 .. 32 kb + 31, the last one all m columns.
TAGS_D void fill_tile(long long t, int m, int& kb, int& i) {
    const int KB = (m + 31) / 32;
    const long long full = 16LL * (KB - 1) * KB;
    if (t >= full) {
        kb = KB - 1;
        i = (int)(t - full);
        return;
    }
    int b = (int)floor((sqrt(1.0 + (double)t / 4.0) - 1.0) * 0.5);
    if (b < 0) b = 0;
    while (b > 0 && 16LL * b * (b + 1) > t) --b;
    while (16LL * (b + 1) * (b + 2) <= t) ++b;
    kb = b;
    i = (int)(t - 16LL * b * (b + 1));
}

// Mixed-form fill of the regular pairs, all in FP32, lower triangle only (the
// mirror is k_zmirror's). One warp per (column i, 32 rows, 32 samples): the
// lanes are the samples, so each quadrature point's geometry (offset from the
// panel-pair anchor and weight / r) is computed once, by the warp's lanes in
// parallel, into shared memory, and every sample applies its own
// e^{-gamma (r_p - r_c)} to it. Panel-pair anchors of split pairs are formed
// in FP64 once per warp (a lane per panel pair), never per sample. Outputs
// pass through a [row][sample] sub-tile so each store instruction writes 64
// contiguous bytes per sample. Pairs that share an endpoint (log-singular)
// and the self terms are left to k_fill_special64 (FP64). Five CTAs per SM (their shared memory allows five;
// 96 registers instead of 122): the point loop is latency-bound, so the extra
// warps pay for the few spilled values outside it.
__global__ void __launch_bounds__(FILL_WARPS * 32, 5) k_fill_mixed(
    const double* __restrict__ elec, const double* __restrict__ img, const float4* __restrict__ sdir,
    const float4* __restrict__ idir, int m, const uint16_t* __restrict__ codes,
    const PairRec* __restrict__ recs, const SampleF32* __restrict__ coef, int nsamp, float2* zl0, float2* zt0,
    long long bstride, int has_img, long long ntiles, int* status, const int* __restrict__ mom_ok, float2* zlo0,
    float2* ztlo0) {
    __shared__ float sxm[GL_MIX], swf[GL_MIX];
    __shared__ FillWarpSmem sw_all[FILL_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int smp = blockIdx.y * 32 + lane;
    // samples the moment fill covers (mom_ok) are left to it; every warp of a
    // CTA has the same 32 samples, so a CTA with none to do leaves as a whole
    const bool valid = smp < nsamp && !(mom_ok && mom_ok[smp]);
    if (!__any_sync(0xffffffffu, valid)) return;
    for (int t = threadIdx.x; t < GL_MIX; t += blockDim.x) {
        sxm[t] = g_glxm[t];
        swf[t] = g_glwm[t];
    }
    __syncthreads();
    FillWarpSmem& W = sw_all[warp];
    const long long tile = (long long)blockIdx.x * FILL_WARPS + warp;
    if (tile >= ntiles) return;                      // whole warp leaves together
    int kb, i;
    fill_tile(tile, m, kb, i);
    SampleF32 c{};
    if (valid) c = coef[smp];
    float gmax = valid ? sqrtf(c.grh * c.grh + c.gih * c.gih) : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gmax = fmaxf(gmax, __shfl_xor_sync(0xffffffffu, gmax, o));
    const float4 ds = sdir[i];
    const float3 hs1 = make_float3(ds.x, ds.y, ds.z);
    const long long pstart = (long long)i * (2LL * m - i + 1) / 2;     // pair index of (i, i)
    const int k_lo = max(i, 32 * kb), k_hi = min(m, 32 * kb + 32);
    const float kr = -1.44269502f * c.grh;
    for (int k0 = k_lo; k0 < k_hi; k0 += FILL_SUB) {
        const int kend = min(k_hi, k0 + FILL_SUB);
        for (int k = k0; k < kend; ++k) {
            const long long p = pstart + (k - i);
            // the self term of the diagonal is added in FP64 by k_fill_special64
            float2 zl = make_float2(0.f, 0.f), zt = make_float2(0.f, 0.f);
            for (int kind = 0; kind < 2; ++kind) {
                if (kind == 0 && k == i) continue;
                if (kind == 1 && !has_img) break;
                const uint16_t code = codes[2 * p + kind];
                if (code & (PC_TOUCH | PC_DEGEN)) continue;      // k_fill_special64
                const float4 dr = kind == 0 ? sdir[k] : idir[k];
                const PairRec rec = recs[2 * p + kind];
                const float lmax = fmaxf(ds.w, dr.w);
                const int P = min(32, max(max(code & 63, 1), (int)ceilf(fminf(gmax * lmax / 1.5f, 32.f))));
                const int qg = (code >> 6) & 63;
                const int qq = min(QMIX, qg + (int)ceilf(fminf(gmax * lmax / P, (float)QMIX)));
                const float* x = sxm + gl_off(qq);
                const float* w = swf + gl_off(qq);
                const float h = 1.f / (float)P;
                const float3 hr = make_float3(dr.x * h, dr.y * h, dr.z * h);
                const float3 hs = make_float3(hs1.x * h, hs1.y * h, hs1.z * h);
                const int npts = qq * qq;
                float2 acc = make_float2(0.f, 0.f);
                const int npp = P * P;
                for (int pp0 = 0; pp0 < npp; pp0 += 32) {
                    const int cnt = min(32, npp - pp0);
                    if (P > 1) {
                        // panel-pair anchors of this chunk in FP64, one per lane
                        // (the FP64 pipe is 1/64 of FP32 here: never per sample)
                        if (lane < cnt) {
                            const int pp = pp0 + lane, pi = pp / P, pj = pp - pi * P;
                            const double* SR = (kind == 0 ? elec : img) + 11LL * k;
                            const double* SS = elec + 11LL * i;
                            const double fr = (pi + 0.5) / P, fs = (pj + 0.5) / P;
                            double dd[3];
                            for (int cc = 0; cc < 3; ++cc)
                                dd[cc] = (SR[cc] + fr * (SR[3 + cc] - SR[cc])) - (SS[cc] + fs * (SS[3 + cc] - SS[cc]));
                            const double r = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                            const float rhf = (float)r;
                            W.anc[lane] = make_float4((float)dd[0], (float)dd[1], (float)dd[2], rhf);
                            W.ancl[lane] = (float)(r - (double)rhf);
                        }
                        __syncwarp();
                    }
                    for (int u = 0; u < cnt; ++u) {
                        // panel-pair anchor: midpoint vector and its length as a float pair
                        float3 D;
                        float rh, rl;
                        if (P == 1) {
                            D = make_float3(rec.dx, rec.dy, rec.dz);
                            rh = rec.rch;
                            rl = rec.rcl;
                        } else {
                            const float4 an4 = W.anc[u];
                            D = make_float3(an4.x, an4.y, an4.z);
                            rh = an4.w;
                            rl = W.ancl[u];
                        }
                        const float rc2 = rh * rh;
                        for (int t = lane; t < npts; t += 32) {
                            const int qi = t / qq, qj = t - qi * qq;
                            const float a = x[qi], b = x[qj];
                            // u = a hr - b hs: offset of the point pair from the panel centres
                            const float ux = fmaf(-b, hs.x, a * hr.x), uy = fmaf(-b, hs.y, a * hr.y),
                                        uz = fmaf(-b, hs.z, a * hr.z);
                            const float e = fmaf(2.f, fmaf(D.x, ux, fmaf(D.y, uy, D.z * uz)),
                                                 fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
                            const float tt = rc2 + e;
                            const float irp = rsqrtf(tt);                          // 1 / r_p
                            const float del = e * __frcp_rn(fmaf(tt, irp, rh));    // r_p - r_c
                            W.geo[t] = make_float2(del, w[qi] * w[qj] * irp);
                        }
                        __syncwarp();
                        float2 ps = make_float2(0.f, 0.f);
#pragma unroll 4
                        for (int t = 0; t < npts; ++t) {
                            const float2 g = W.geo[t];
                            const float mg = g.y * ex2_approx(kr * g.x);
                            float sn, cs;
                            __sincosf(c.gih * g.x, &sn, &cs);
                            ps.x = fmaf(mg, cs, ps.x);
                            ps.y = fmaf(-mg, sn, ps.y);
                        }
                        __syncwarp();
                        const float2 an = anchor_df(c.grh, c.grl, c.gih, c.gil, rh, rl);
                        acc = ffmac(an, ps, acc);
                    }
                    __syncwarp();                     // the chunk's anchors are read: free for the next
                }
                const float h2 = h * h;
                const float2 J = make_float2(acc.x * h2, acc.y * h2);
                const float2 cL = kind == 0 ? c.cL : c.cLi, cT = kind == 0 ? c.cT : c.cTi;
                zt = ffmac(cT, J, zt);
                zl = ffmac(make_float2(cL.x * rec.fl, cL.y * rec.fl), J, zl);
            }
            W.zl[k - k0][lane] = zl;
            W.zt[k - k0][lane] = zt;
        }
        __syncwarp();
        const int nrow = kend - k0;
        for (int idx = lane; idx < FILL_SUB * 32; idx += 32) {
            const int j = idx % FILL_SUB, sl = idx / FILL_SUB;
            const int ss = blockIdx.y * 32 + sl;
            if (j < nrow && ss < nsamp && !(mom_ok && mom_ok[ss])) {
                const float2 a = W.zl[j][sl], b = W.zt[j][sl];
                if (!isfinite(a.x + a.y + b.x + b.y)) raise_status(status, TAGS_ST_NONFINITE);
                const long long off = bstride * ss + (k0 + j) + (long long)m * i;
                zl0[off] = a;
                zt0[off] = b;
                if (zlo0) {
                    zlo0[off] = make_float2(0.f, 0.f);       // FP32 entries: no residue
                    ztlo0[off] = make_float2(0.f, 0.f);
                }
            }
        }
        __syncwarp();
    }
}

// Upper triangle of ZL and ZT from the lower one, 32 x 32 tiles through
// shared memory (coalesced reads and writes). A CTA moves one tile position
// of MIRROR_MATS matrices (ZL and ZT of consecutive samples), so each CTA
// carries enough traffic to hide its start-up.
// With pmax / psum (the high parts' pass) it also leaves the row statistics'
// partials: per matrix, row R and tile slot t (KB = ceil(m / 32) slots) the
// max and the sum of |Z[R][j]| over the 32 columns of block t, from the tile
// (R's block, t) for t below R's block, from the column below the diagonal in
// tile (t, R's block) for t above it, and from both halves of the diagonal
// tile at t = R's block: layout [mat][t][R]. Every sum has a fixed order.
constexpr int MIRROR_MATS = 8;
__global__ void __launch_bounds__(256) k_zmirror(float2* zl0, float2* zt0, long long bstride, int m, int nmat,
                                                 float* __restrict__ pmax, float* __restrict__ psum) {
    __shared__ float2 tile[2][32][33];
    __shared__ float rmx[2][8][32], rsm[2][8][32], cmx[2][32], csm[2][32];
    const long long t = blockIdx.x;
    // lower tiles by block row: row block bk holds column blocks 0 .. bk
    int bk = (int)floor((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    if (bk < 0) bk = 0;
    while (bk > 0 && (long long)bk * (bk + 1) / 2 > t) --bk;
    while ((long long)(bk + 1) * (bk + 2) / 2 <= t) ++bk;
    const int bi = (int)(t - (long long)bk * (bk + 1) / 2);
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int mat0 = blockIdx.y * MIRROR_MATS;
    const int KB = (m + 31) / 32;
    const int r = bk * 32 + tx;                        // this thread's row of the lower tile
    // the four lower entries of this thread in matrix mat (columns bi * 32 + ty + 8 jj),
    // loaded one matrix ahead so that they travel while the previous one is stored
    float2 v[4];
    auto load = [&](int mat) {
        const float2* Z = ((mat & 1) ? zt0 : zl0) + bstride * (mat >> 1);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int cc = bi * 32 + ty + 8 * jj;
            v[jj] = r < m && cc < m && r >= cc ? Z[r + (long long)m * cc] : make_float2(0.f, 0.f);
        }
    };
    if (mat0 < nmat) load(mat0);
    for (int q = 0; q < MIRROR_MATS; ++q) {
        const int mat = mat0 + q;                      // 2 x sample + (0: ZL, 1: ZT)
        if (mat >= nmat) break;
        float2* Z = ((mat & 1) ? zt0 : zl0) + bstride * (mat >> 1);
        float2 (*T)[33] = tile[q & 1];                 // two buffers: one barrier per matrix
        float rowmx = 0.f, rowsm = 0.f;                // row r over this thread's columns
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int j = ty + 8 * jj, cc = bi * 32 + j;
            if (r < m && cc < m && r > cc) T[j][tx] = v[jj];
            if (pmax) {
                // v is zero outside the lower triangle and the matrix
                const float a = sqrtf(v[jj].x * v[jj].x + v[jj].y * v[jj].y);
                rowmx = fmaxf(rowmx, a);
                rowsm += a;
                // column cc below the diagonal: row cc's entries in this tile
                float cm = r > cc ? a : 0.f, cs = cm;
                for (int o = 16; o > 0; o >>= 1) {
                    cm = fmaxf(cm, __shfl_xor_sync(0xffffffffu, cm, o));
                    cs += __shfl_xor_sync(0xffffffffu, cs, o);
                }
                if (tx == 0) {
                    cmx[q & 1][j] = cm;
                    csm[q & 1][j] = cs;
                }
            }
        }
        if (pmax) {
            rmx[q & 1][ty][tx] = rowmx;
            rsm[q & 1][ty][tx] = rowsm;
        }
        if (q + 1 < MIRROR_MATS && mat + 1 < nmat) load(mat + 1);
        __syncthreads();
        for (int j = ty; j < 32; j += 8) {
            const int cc = bi * 32 + tx, rr = bk * 32 + j;     // element (row cc, column rr) of the upper triangle
            if (rr < m && cc < m && rr > cc) Z[cc + (long long)m * rr] = T[tx][j];
        }
        if (pmax && ty < 2) {
            float mx = 0.f, sm = 0.f;
            if (ty == 0 || bk != bi) {
                // ty 0: the rows of block bk (their columns in block bi);
                // ty 1: the rows of block bi (their column parts), off the diagonal
                if (ty == 0) {
#pragma unroll
                    for (int w = 0; w < 8; ++w) {
                        mx = fmaxf(mx, rmx[q & 1][w][tx]);
                        sm += rsm[q & 1][w][tx];
                    }
                    if (bk == bi) {
                        mx = fmaxf(mx, cmx[q & 1][tx]);
                        sm += csm[q & 1][tx];
                    }
                } else {
                    mx = cmx[q & 1][tx];
                    sm = csm[q & 1][tx];
                }
                const int row = (ty == 0 ? bk : bi) * 32 + tx, slot = ty == 0 ? bi : bk;
                if (row < m) {
                    const long long o = ((long long)mat * KB + slot) * m + row;
                    pmax[o] = mx;
                    psum[o] = sm;
                }
            }
        }
    }
}

// Duffy moments of the touching kinds, once per plan (FP64). For a pair
// sharing an endpoint, j_touch sums w [phi(gamma rho1)/rho1 + phi(gamma rho2)/rho2]
// over the Duffy halves' nodes; with phi(x) = sum_n (-x)^n / (n + 1)! that is
//   J = sum_n (-gamma)^n / (n + 1)! M_n,   M_n = sum_q w_q (rho1^(n-1) + rho2^(n-1)),
// geometry only. rho <= L_a + L_b, so the series converges like that of
// e^{|gamma| (L_a + L_b)}: 24 terms cover |gamma| (L_a + L_b) up to ~3 at FP64
// accuracy. Warp per special entry, lane per node of a 32-point rule (more
// than the plain form's 16 + 2 |gamma| L for the same integrals).
constexpr int TM_Q = 32;

__global__ void __launch_bounds__(128) k_touch_moments(const double* __restrict__ elec, const double* __restrict__ img,
                                                       int m, const int2* __restrict__ ent, int nent,
                                                       double* __restrict__ tm) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int e = blockIdx.x * 4 + warp;
    if (e >= nent) return;
    const int2 en = ent[e];
    int i, k;
    pair_index(en.x, m, i, k);
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    for (int kind = 0; kind < 2; ++kind) {
        double acc[MOM_N];
#pragma unroll
        for (int n = 0; n < MOM_N; ++n) acc[n] = 0.0;
        bool ok = (en.y & (1 << kind)) != 0;
        int ia = 0, ib = 0;
        if (ok) {
            ld_seg((kind == 0 ? elec : img) + 11LL * k, R);
            ok = touching(R, S, 1e-9 * fmax(S.len, R.len), ia, ib);
        }
        if (ok) {
            double a[3], b[3];
            for (int d = 0; d < 3; ++d) {
                a[d] = ia == 0 ? R.b[d] - R.a[d] : R.a[d] - R.b[d];
                b[d] = ib == 0 ? S.b[d] - S.a[d] : S.a[d] - S.b[d];
            }
            const double t = g_glx[gl_off(TM_Q) + lane], w = g_glw[gl_off(TM_Q) + lane];
            const double u1[3] = {a[0] - t * b[0], a[1] - t * b[1], a[2] - t * b[2]};
            const double u2[3] = {t * a[0] - b[0], t * a[1] - b[1], t * a[2] - b[2]};
            const double r1 = sqrt(dot3(u1, u1)), r2 = sqrt(dot3(u2, u2));
            double v1 = w / r1, v2 = w / r2;
#pragma unroll
            for (int n = 0; n < MOM_N; ++n) {
                acc[n] = v1 + v2;
                v1 *= r1;
                v2 *= r2;
            }
        }
#pragma unroll
        for (int n = 0; n < MOM_N; ++n)
            for (int o = 16; o > 0; o >>= 1) acc[n] += __shfl_xor_sync(0xffffffffu, acc[n], o);
        if (lane == 0) {
#pragma unroll
            for (int n = 0; n < MOM_N; ++n) tm[((long long)e * 2 + kind) * MOM_N + n] = acc[n];
        }
    }
}

// The log-singular entries in FP64: for each special entry (a pair with a
// kind that shares an endpoint, or a diagonal entry) the touching kinds from
// their Duffy moments (k_touch_moments) as an FP64 series in gamma, or, for a
// warp of samples the 24-term series does not reach, the Duffy rule of
// j_touch at the plain form's order (16 + 2 |gamma| L) directly; and the
// static closed form for the self term, added to the FP32 value
// the regular fill left there for the regular kinds (lower triangle, hi in Z
// and lo in Zlo). The sum v is formed in FP64 and stored again as hi = fl(v)
// in Z and lo = fl(v - hi) in Zlo, which the refinement's residual reads. One warp per entry and
// 32 samples (lanes): the rule's nodes (rho and w / rho of both Duffy halves)
// are computed once per warp into shared memory.
constexpr int SPEC_WARPS = 4;

__global__ void __launch_bounds__(SPEC_WARPS * 32) k_fill_special64(
    const double* __restrict__ elec, const double* __restrict__ img, int m, const int2* __restrict__ ent, int nent,
    const SampleCoef* __restrict__ coef, int nsamp, float2* zl0, float2* zt0, float2* zlo0, float2* ztlo0,
    long long bstride, int* status, const double* __restrict__ tm, double tdmax) {
    __shared__ double2 nodes_all[SPEC_WARPS][2 * QMAX];      // (rho, w / rho)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double2* nodes = nodes_all[warp];
    const int e = blockIdx.x * SPEC_WARPS + warp;
    if (e >= nent) return;                            // whole warp leaves together
    const int smp = blockIdx.y * 32 + lane;
    const bool valid = smp < nsamp;
    SampleCoef c{};
    if (valid) c = coef[smp];
    const int2 en = ent[e];
    int i, k;
    pair_index(en.x, m, i, k);
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    double2 dl = cz(0.0, 0.0), dt = cz(0.0, 0.0);
    bool bad = false;
    // the moment series when every lane's sample needs at most MOM_N terms:
    // the first n with x^n / (n + 1)! <= 1e-17 e^{-x}, x = |gamma| (L_a + L_b)
    int ntw = 0;
    {
        const double xg = valid ? sqrt(cabs2(c.gamma)) * tdmax : 0.0, lim = 1e-17 * exp(-xg);
        double term = 1.0;
        while (ntw <= MOM_N && !(term <= lim && ntw > 4)) {
            ++ntw;
            term *= xg / (ntw + 1);
        }
        ntw = __reduce_max_sync(0xffffffffu, ntw);
    }
    const bool series = tm && ntw <= MOM_N;
    for (int kind = 0; kind < 2 && !bad; ++kind) {
        if (!(en.y & (1 << kind))) continue;
        ld_seg((kind == 0 ? elec : img) + 11LL * k, R);
        const double lmax = fmax(S.len, R.len);
        int ia, ib;
        bad = !touching(R, S, 1e-9 * lmax, ia, ib);       // coincident or overlapping
        if (!bad) {
            const double* ro = ia == 0 ? R.b : R.a;
            const double* so = ib == 0 ? S.b : S.a;
            bad = fmax(fabs(ro[0] - so[0]), fmax(fabs(ro[1] - so[1]), fabs(ro[2] - so[2]))) <= 1e-9 * lmax;
        }
        if (bad) break;
        if (series) {
            // J = sum_n (-gamma)^n / (n + 1)! M_n in FP64
            const double* M = tm + ((long long)e * 2 + kind) * MOM_N;
            double2 J = cz(0.0, 0.0), an = cz(1.0, 0.0);
            const double2 mg = cz(-c.gamma.x, -c.gamma.y);
            for (int n = 0; n < ntw; ++n) {
                const double Mn = M[n];
                J.x = fma(an.x, Mn, J.x);
                J.y = fma(an.y, Mn, J.y);
                an = cscale(cmul(an, mg), 1.0 / (n + 2));
            }
            double cost = 0.0;
            for (int d = 0; d < 3; ++d) cost += (S.b[d] - S.a[d]) * (R.b[d] - R.a[d]);
            cost = fabs(cost);
            const bool keep = kind == 0 ? !(cost < TAGS_DBL_EPSILON) : (cost > TAGS_DBL_EPSILON);
            const double2 cL = kind == 0 ? c.cL : c.cLi, cT = kind == 0 ? c.cT : c.cTi;
            dt = cadd(dt, cmul(cT, J));
            if (keep) dl = cadd(dl, cscale(cmul(cL, J), cost));
            continue;
        }
        int q = valid ? min(QMAX, 16 + 2 * (int)ceil(fmin(sqrt(cabs2(c.gamma)) * lmax, (double)QMAX))) : 0;
        q = __reduce_max_sync(0xffffffffu, q);
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) {
            a[d] = ia == 0 ? R.b[d] - R.a[d] : R.a[d] - R.b[d];
            b[d] = ib == 0 ? S.b[d] - S.a[d] : S.a[d] - S.b[d];
        }
        __syncwarp();
        for (int qi = lane; qi < q; qi += 32) {
            const double t = g_glx[gl_off(q) + qi], w = g_glw[gl_off(q) + qi];
            const double u1[3] = {a[0] - t * b[0], a[1] - t * b[1], a[2] - t * b[2]};
            const double u2[3] = {t * a[0] - b[0], t * a[1] - b[1], t * a[2] - b[2]};
            const double r1 = sqrt(dot3(u1, u1)), r2 = sqrt(dot3(u2, u2));
            nodes[2 * qi] = make_double2(r1, w / r1);
            nodes[2 * qi + 1] = make_double2(r2, w / r2);
        }
        __syncwarp();
        double2 J = cz(0.0, 0.0);
        if (valid) {
            for (int j = 0; j < 2 * q; ++j) {
                const double2 nd = nodes[j];
                const double2 ph = phi_c(cz(c.gamma.x * nd.x, c.gamma.y * nd.x));
                J.x = fma(nd.y, ph.x, J.x);
                J.y = fma(nd.y, ph.y, J.y);
            }
        }
        // ZL carries |d_i . d_k| (= |cos theta| L_i L_k), dropped where the
        // reference drops it (cos < DBL_EPSILON direct, <= DBL_EPSILON images)
        double cost = 0.0;
        for (int d = 0; d < 3; ++d) cost += (S.b[d] - S.a[d]) * (R.b[d] - R.a[d]);
        cost = fabs(cost);
        const bool keep = kind == 0 ? !(cost < TAGS_DBL_EPSILON) : (cost > TAGS_DBL_EPSILON);
        const double2 cL = kind == 0 ? c.cL : c.cLi, cT = kind == 0 ? c.cT : c.cTi;
        dt = cadd(dt, cmul(cT, J));
        if (keep) dl = cadd(dl, cscale(cmul(cL, J), cost));
    }
    if (!bad && (en.y & 4)) {
        // self term: the reference's static closed form (src/electrode.c:238-245, used at :346-348)
        const double v = self_integral_d(S);
        dl = cadd(dl, cscale(c.cL, v));
        dt = cadd(dt, cscale(c.cT, v / (S.len * S.len)));
    }
    if (bad) {
        if (lane == 0) raise_status(status, TAGS_ST_DEGENERATE_PAIR);
        dl = dt = cz(nan(""), nan(""));
    }
    if (!valid) return;
    if (!isfinite(dl.x + dl.y + dt.x + dt.y)) raise_status(status, TAGS_ST_NONFINITE);
    const long long idx = bstride * smp + k + (long long)m * i;      // lower triangle (k_zmirror copies it up)
    const float2 za = zl0[idx], zb = zt0[idx], la = zlo0[idx], lb = ztlo0[idx];
    const double vlr = ((double)za.x + (double)la.x) + dl.x, vli = ((double)za.y + (double)la.y) + dl.y;
    const double vtr = ((double)zb.x + (double)lb.x) + dt.x, vti = ((double)zb.y + (double)lb.y) + dt.y;
    const float2 hl = make_float2((float)vlr, (float)vli), ht = make_float2((float)vtr, (float)vti);
    zl0[idx] = hl;
    zt0[idx] = ht;
    zlo0[idx] = make_float2((float)(vlr - (double)hl.x), (float)(vli - (double)hl.y));
    ztlo0[idx] = make_float2((float)(vtr - (double)ht.x), (float)(vti - (double)ht.y));
}

// ---- mixed form: moment expansion of the regular pairs ---------------------------------
//
// For a (pair, kind) whose segments share no endpoint,
//   J(gamma) = \int_0^1 \int_0^1 e^{-gamma r} / r dt0 dt1
//            = e^{-gamma R} sum_n (-gamma)^n / n! N_n,   N_n = \int\int (r - R)^n / r dt0 dt1,
// expanded about R = b h, the multiple of h = 1/8 m nearest the midpoint
// distance. |r - R| <= (L_i + L_k) / 2 + h / 2 on the pair, so the series
// converges like that of e^{|gamma| dmax}: 16 terms reach 1e-14 at |gamma|
// dmax = 0.9 (1 m segments at 10 MHz in 1 mS/m soil). The moments N_n depend
// on the geometry only and are computed once per plan in FP64 (tensor
// Gauss-Legendre at the FP64 fill's orders plus MOM_EXTRA). Per sample a pass
// evaluates the series in two-float arithmetic (float pairs; the terms past
// MOM_HEAD, below 1e-5 of the sum, by Horner in FP32) and multiplies by
// e^{-gamma b h} from a per-sample table computed in FP64. The entries come
// out as hi + lo float pairs good to ~1e-12, where the FP32 quadrature of the
// same integrals (k_fill_mixed, kept for samples the series does not reach)
// is good to ~1e-7. FP32 rounding of the stored entries varies from sample to
// sample like noise, which the inverse Laplace transform amplifies by up to
// e^{c t}; the float pairs keep that noise at the FP64 level.

constexpr int MOM_HEAD = 8;                                  // terms kept as float pairs
constexpr int MOM_FLOATS = 2 * MOM_HEAD + (MOM_N - MOM_HEAD);   // 32 floats per (pair, kind)
constexpr int MOM_EXTRA = 6;                                 // orders above the FP64 fill's rule
static_assert(MOM_FLOATS == 32, "a (pair, kind) record is one 128-byte line");

struct MomRec {
    int b;            // expansion centre R = b h
    int regular;      // 1: the kind exists and shares no endpoint
    float fl_hi, fl_lo;   // ZL factor |d_i . d_k| as a float pair (0 where the reference drops ZL)
};

// Warp per (pair, kind): the lanes share the tensor rule's points; each lane
// accumulates all MOM_N moments of its points in FP64, then a butterfly sums
// them. Lane n writes term n (head terms as hi, lo float pairs).
__global__ void __launch_bounds__(128) k_moments(const double* __restrict__ elec, const double* __restrict__ img,
                                                 int m, int has_img, float* __restrict__ mom,
                                                 MomRec* __restrict__ rec) {
    __shared__ double sx[GL_TOTAL], sw[GL_TOTAL];
    for (int t = threadIdx.x; t < GL_TOTAL; t += blockDim.x) {
        sx[t] = g_glx[t];
        sw[t] = g_glw[t];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long npk = (long long)m * (m + 1);              // (pair, kind) records
    const long long pk = (long long)blockIdx.x * 4 + warp;
    if (pk >= npk) return;                                      // whole warp leaves together
    const long long p = pk >> 1;
    const int kind = (int)(pk & 1);
    int i, k;
    pair_index(p, m, i, k);
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    bool regular = (kind == 0 && k != i) || (kind == 1 && has_img);
    if (regular) {
        ld_seg((kind == 0 ? elec : img) + 11LL * k, R);
        regular = (classify_pair(S, R) & (PC_TOUCH | PC_DEGEN)) == 0;
    }
    float* out = mom + pk * MOM_FLOATS;
    if (!regular) {
        out[lane] = 0.f;
        if (lane == 0) rec[pk] = MomRec{0, 0, 0.f, 0.f};
        return;
    }
    double dm[3] = {R.mid[0] - S.mid[0], R.mid[1] - S.mid[1], R.mid[2] - S.mid[2]};
    const double rc = sqrt(dot3(dm, dm));
    const int b = (int)rint(rc / MOM_H);
    const double Rb = b * MOM_H;
    const double lmax = fmax(S.len, R.len);
    const double ratio = seg_seg_dist(R.a, R.b, S.a, S.b) / lmax;
    const int P = ratio >= 2.0 ? 1 : (int)fmin(32.0, ceil(2.0 / ratio));
    const int q = min(QMAX, order_for(ratio * P, 0.0, true) + MOM_EXTRA);
    const double* x = sx + gl_off(q);
    const double* w = sw + gl_off(q);
    double dr[3], ds[3];
    for (int c = 0; c < 3; ++c) {
        dr[c] = R.b[c] - R.a[c];
        ds[c] = S.b[c] - S.a[c];
    }
    const double h = 1.0 / P;
    double acc[MOM_N];
#pragma unroll
    for (int n = 0; n < MOM_N; ++n) acc[n] = 0.0;
    const int qq = q * q, npts = P * P * qq;
    for (int t = lane; t < npts; t += 32) {
        const int pp = t / qq, u = t - pp * qq;
        const int pi = pp / P, pj = pp - pi * P, qi = u / q, qj = u - qi * q;
        const double t0 = (pi + x[qi]) * h, t1 = (pj + x[qj]) * h;
        const double dx = (R.a[0] + t0 * dr[0]) - (S.a[0] + t1 * ds[0]);
        const double dy = (R.a[1] + t0 * dr[1]) - (S.a[1] + t1 * ds[1]);
        const double dz = (R.a[2] + t0 * dr[2]) - (S.a[2] + t1 * ds[2]);
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        const double d = r - Rb;
        double v = w[qi] * w[qj] * h * h / r;
#pragma unroll
        for (int n = 0; n < MOM_N; ++n) {
            acc[n] += v;
            v *= d;
        }
    }
#pragma unroll
    for (int n = 0; n < MOM_N; ++n)
        for (int o = 16; o > 0; o >>= 1) acc[n] += __shfl_xor_sync(0xffffffffu, acc[n], o);
    double mine = 0.0;
#pragma unroll
    for (int n = 0; n < MOM_N; ++n)
        if ((lane < 2 * MOM_HEAD ? lane >> 1 : lane - MOM_HEAD) == n) mine = acc[n];
    if (lane < 2 * MOM_HEAD) {
        const float hi = (float)mine;
        out[lane] = (lane & 1) ? (float)(mine - (double)hi) : hi;
    } else {
        out[lane] = (float)mine;
    }
    if (lane == 0) {
        double cost = fabs(dot3(ds, dr));
        const bool keep = kind == 0 ? !(cost < TAGS_DBL_EPSILON) : (cost > TAGS_DBL_EPSILON);
        if (!keep) cost = 0.0;
        const float fh = (float)cost;
        rec[pk] = MomRec{b, 1, fh, (float)(cost - (double)fh)};
    }
}

// ---- two-float (float pair) arithmetic --------------------------------------------
struct DF {
    float h, l;
};
TAGS_HD DF df_of(double v) {
    const float h = (float)v;
    return DF{h, (float)(v - (double)h)};
}
// a * b, the head product exact (FMA), the cross terms added to the tail
TAGS_D DF df_mul(DF a, DF b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return DF{p, e};
}
TAGS_D DF df_add(DF a, DF b) {
    const float s = a.h + b.h;
    const float z = s - a.h;
    const float e = (a.h - (s - z)) + (b.h - z);
    return DF{s, e + a.l + b.l};
}
TAGS_D DF df_neg(DF a) { return DF{-a.h, -a.l}; }
TAGS_D DF df_norm(DF a) {
    const float s = a.h + a.l;
    return DF{s, a.l - (s - a.h)};
}
struct CDF {
    DF re, im;
};
TAGS_D CDF cdf_mul(CDF a, CDF b) {
    return CDF{df_norm(df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im)))),
               df_norm(df_add(df_mul(a.re, b.im), df_mul(a.im, b.re)))};
}
TAGS_D CDF cdf_add(CDF a, CDF b) { return CDF{df_add(a.re, b.re), df_add(a.im, b.im)}; }
TAGS_HD CDF cdf_of(double2 v) { return CDF{df_of(v.x), df_of(v.y)}; }

// Per-sample constants of the moment fill.
struct MomCoef {
    float a[MOM_HEAD][4];      // (-gamma)^n / n!, n < MOM_HEAD: re (hi, lo), im (hi, lo)
    float2 g;                  // gamma (FP32), for the Horner tail
    float2 a8;                 // (-gamma)^MOM_HEAD / MOM_HEAD! (FP32)
    int nt;                    // terms this sample needs (<= MOM_N)
    int ok;                    // 1: the series reaches 1e-14 within MOM_N terms
};

// Terms of the series for 1e-14 at x = |gamma| dmax: the first n with
// x^n / n! <= 1e-14 e^{-x} (the sum is at least e^{-x} times its leading term's
// scale), at least MOM_HEAD + 1.
__global__ void k_mom_coef(const SampleCoef* __restrict__ coef, int nsamp, double dmax, MomCoef* __restrict__ out,
                           int* __restrict__ ok) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsamp) return;
    const SampleCoef c = coef[q];
    MomCoef o;
    double2 an = make_double2(1.0, 0.0);
    const double2 mg = make_double2(-c.gamma.x, -c.gamma.y);
    for (int n = 0; n < MOM_HEAD; ++n) {
        const DF r = df_of(an.x), im = df_of(an.y);
        o.a[n][0] = r.h;
        o.a[n][1] = r.l;
        o.a[n][2] = im.h;
        o.a[n][3] = im.l;
        an = cscale(cmul(an, mg), 1.0 / (n + 1));
    }
    o.a8 = make_float2((float)an.x, (float)an.y);
    o.g = make_float2((float)c.gamma.x, (float)c.gamma.y);
    const double xg = sqrt(cabs2(c.gamma)) * dmax;
    double term = 1.0;
    int nt = 0;
    const double lim = 1e-14 * exp(-xg);
    while (nt < 64 && !(term <= lim && nt > MOM_HEAD)) {
        term *= xg / (nt + 1);
        ++nt;
    }
    o.nt = nt;
    o.ok = nt <= MOM_N ? 1 : 0;
    out[q] = o;
    ok[q] = o.ok;
}

// The series' sample factors per bucket b and sample, formed in FP64 and
// stored as complex float pairs: tab[v][b][sample] = f_v e^{-gamma b h} with
// f_0 = cT (direct ZT), f_1 = cTi (image ZT), f_2 = cL (ZL, both kinds: ref_l
// = 1), so each (pair, kind) multiplies its series by one table value per
// matrix instead of by e^{-gamma b h} and then by the factor.
__global__ void k_mom_table(const SampleCoef* __restrict__ coef, int nsamp, int nb, int bstride,
                            float4* __restrict__ tab) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (q >= nsamp || b >= nb) return;
    const SampleCoef c = coef[q];
    const double2 e = cexp_d(make_double2(-c.gamma.x * b * MOM_H, -c.gamma.y * b * MOM_H));
    const double2 f[3] = {c.cT, c.cTi, c.cL};
    for (int v = 0; v < 3; ++v) {
        const double2 t = cmul(f[v], e);
        const DF r = df_of(t.x), im = df_of(t.y);
        tab[((long long)v * nb + b) * bstride + q] = make_float4(r.h, r.l, im.h, im.l);
    }
}

// J of one (pair, kind) for this lane's sample from the staged record and
// moments (shared memory, read by all lanes alike).
TAGS_D CDF mom_series(const float* __restrict__ mv, int nt, const MomCoef& c) {
    // tail: H = N_8 + (-gamma/9)(N_9 + (-gamma/10)(N_10 + ...)) by Horner in
    // FP32 (a term of the tail is a_n N_n = a_8 (a_n / a_8) N_n), times a_8
    float hr = 0.f, hi = 0.f;
    for (int n = nt - 1; n >= MOM_HEAD; --n) {
        const float f = -1.f / (float)(n + 1);
        const float tr = f * (c.g.x * hr - c.g.y * hi), ti = f * (c.g.x * hi + c.g.y * hr);
        hr = mv[2 * MOM_HEAD + n - MOM_HEAD] + tr;
        hi = ti;
    }
    const float tr = c.a8.x * hr - c.a8.y * hi, ti = c.a8.x * hi + c.a8.y * hr;
    DF sr{0.f, tr}, si{0.f, ti};
#pragma unroll
    for (int n = 0; n < MOM_HEAD; ++n) {
        const DF N{mv[2 * n], mv[2 * n + 1]};
        sr = df_add(sr, df_mul(DF{c.a[n][0], c.a[n][1]}, N));
        si = df_add(si, df_mul(DF{c.a[n][2], c.a[n][3]}, N));
    }
    return CDF{df_norm(sr), df_norm(si)};
}

constexpr int MOM_WARPS = 4;
struct MomWarpSmem {
    float mv[2][MOM_FLOATS];                      // moments of the row's two kinds
    MomRec rc[2];
    float2 zl[FILL_SUB][33], zt[FILL_SUB][33];    // outputs hi, [row][sample]
    float2 ll[FILL_SUB][33], lt[FILL_SUB][33];    // outputs lo
};

// Moment fill of the regular kinds, lower triangle, float pairs: Z gets hi,
// Zlo gets lo. Warp per (column i, 32 rows, 32 samples) as k_fill_mixed;
// samples whose series needs more than MOM_N terms are skipped (ok = 0) and
// left to k_fill_mixed. The diagonal's self term and the touching kinds are
// added afterwards by k_fill_special64.
__global__ void __launch_bounds__(MOM_WARPS * 32) k_fill_moment(
    int m, const float* __restrict__ mom, const MomRec* __restrict__ rec, const MomCoef* __restrict__ coef,
    const float4* __restrict__ tab, int tstride, int tnb, int nsamp, float2* zl0, float2* zt0, float2* zlo0,
    float2* ztlo0, long long bstride, long long ntiles, int* status) {
    __shared__ MomWarpSmem sw_all[MOM_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    MomWarpSmem& W = sw_all[warp];
    const long long tile = (long long)blockIdx.x * MOM_WARPS + warp;
    if (tile >= ntiles) return;                      // whole warp leaves together
    int kb, i;
    fill_tile(tile, m, kb, i);
    const int smp = blockIdx.y * 32 + lane;
    bool valid = smp < nsamp;
    MomCoef c{};
    if (valid) c = coef[smp];
    valid = valid && c.ok;
    if (!__any_sync(0xffffffffu, valid)) return;
    int ntw = valid ? c.nt : 0;
    ntw = __reduce_max_sync(0xffffffffu, ntw);
    const long long pstart = (long long)i * (2LL * m - i + 1) / 2;
    const int k_lo = max(i, 32 * kb), k_hi = min(m, 32 * kb + 32);
    // the rows' moments and records are read one row ahead into registers,
    // so their latency overlaps the series of the row before
    float nm0 = 0.f, nm1 = 0.f;
    MomRec nrc{0, 0, 0.f, 0.f};
    if (k_lo < k_hi) {
        const long long p = pstart + (k_lo - i);
        nm0 = mom[(2 * p) * MOM_FLOATS + lane];
        nm1 = mom[(2 * p + 1) * MOM_FLOATS + lane];
        if (lane < 2) nrc = rec[2 * p + lane];
    }
    for (int k0 = k_lo; k0 < k_hi; k0 += FILL_SUB) {
        const int kend = min(k_hi, k0 + FILL_SUB);
        for (int k = k0; k < kend; ++k) {
            const long long p = pstart + (k - i);
            __syncwarp();
            W.mv[0][lane] = nm0;
            W.mv[1][lane] = nm1;
            if (lane < 2) W.rc[lane] = nrc;
            __syncwarp();
            if (k + 1 < k_hi) {
                nm0 = mom[(2 * p + 2) * MOM_FLOATS + lane];
                nm1 = mom[(2 * p + 3) * MOM_FLOATS + lane];
                if (lane < 2) nrc = rec[2 * p + 2 + lane];
            }
            CDF zt{DF{0.f, 0.f}, DF{0.f, 0.f}}, zl = zt;
#pragma unroll
            for (int kind = 0; kind < 2; ++kind) {
                const MomRec rc = W.rc[kind];
                if (!rc.regular) continue;
                const CDF S = mom_series(W.mv[kind], ntw, c);
                // cT (or cTi) e^{-gamma b h} and cL e^{-gamma b h} from the table
                const float4 tt = valid ? tab[((long long)kind * tnb + rc.b) * tstride + smp]
                                        : make_float4(0.f, 0.f, 0.f, 0.f);
                zt = cdf_add(zt, cdf_mul(CDF{DF{tt.x, tt.y}, DF{tt.z, tt.w}}, S));
                const DF fl{rc.fl_hi, rc.fl_lo};
                if (fl.h != 0.f) {
                    const float4 tl = valid ? tab[((long long)2 * tnb + rc.b) * tstride + smp]
                                            : make_float4(0.f, 0.f, 0.f, 0.f);
                    const CDF lj = cdf_mul(CDF{DF{tl.x, tl.y}, DF{tl.z, tl.w}}, S);
                    zl = cdf_add(zl, CDF{df_mul(lj.re, fl), df_mul(lj.im, fl)});
                }
            }
            zl = CDF{df_norm(zl.re), df_norm(zl.im)};
            zt = CDF{df_norm(zt.re), df_norm(zt.im)};
            W.zl[k - k0][lane] = make_float2(zl.re.h, zl.im.h);
            W.zt[k - k0][lane] = make_float2(zt.re.h, zt.im.h);
            W.ll[k - k0][lane] = make_float2(zl.re.l, zl.im.l);
            W.lt[k - k0][lane] = make_float2(zt.re.l, zt.im.l);
        }
        __syncwarp();
        const int nrow = kend - k0;
        for (int idx = lane; idx < FILL_SUB * 32; idx += 32) {
            const int j = idx % FILL_SUB, sl = idx / FILL_SUB;
            const int ss = blockIdx.y * 32 + sl;
            const int ok_sl = __shfl_sync(0xffffffffu, valid ? 1 : 0, sl);     // every lane takes part
            if (j < nrow && ss < nsamp && ok_sl) {
                const float2 a = W.zl[j][sl], b = W.zt[j][sl];
                if (!isfinite(a.x + a.y + b.x + b.y)) raise_status(status, TAGS_ST_NONFINITE);
                const long long off = bstride * ss + (k0 + j) + (long long)m * i;
                zl0[off] = a;
                zt0[off] = b;
                zlo0[off] = W.ll[j][sl];
                ztlo0[off] = W.lt[j][sl];
            }
        }
        __syncwarp();
    }
}

__global__ void k_seg_dirs(const double* __restrict__ elec, const double* __restrict__ img, int m, int has_img,
                           float4* __restrict__ sdir, float4* __restrict__ idir) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    Seg S;
    ld_seg(elec + 11LL * i, S);
    sdir[i] = make_float4((float)(S.b[0] - S.a[0]), (float)(S.b[1] - S.a[1]), (float)(S.b[2] - S.a[2]), (float)S.len);
    if (has_img) {
        ld_seg(img + 11LL * i, S);
        idir[i] = make_float4((float)(S.b[0] - S.a[0]), (float)(S.b[1] - S.a[1]), (float)(S.b[2] - S.a[2]),
                              (float)S.len);
    } else {
        idir[i] = sdir[i];
    }
}

}  // namespace

// Gauss-Legendre nodes/weights by Newton iteration on P_q (host side).
void tags_gauss_legendre(int q, double* x, double* w) {
    for (int i = 0; i < q; ++i) {
        double z = cos(TAGS_PI * (i + 0.75) / (q + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int l = 2; l <= q; ++l) {
                double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
                p0 = p1;
                p1 = p2;
            }
            double pq = q == 1 ? z : p1, pqm1 = q == 1 ? 1.0 : p0;
            dp = q * (z * pq - pqm1) / (z * z - 1.0);
            double dz = pq / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        // recompute derivative at the converged root
        double p0 = 1.0, p1 = z;
        for (int l = 2; l <= q; ++l) {
            double p2 = ((2.0 * l - 1.0) * z * p1 - (l - 1.0) * p0) / l;
            p0 = p1;
            p1 = p2;
        }
        double pq = q == 1 ? z : p1, pqm1 = q == 1 ? 1.0 : p0;
        dp = q * (z * pq - pqm1) / (z * z - 1.0);
        x[i] = 0.5 * (1.0 - z);                 // ascending on [0,1]
        w[i] = 1.0 / ((1.0 - z * z) * dp * dp); // (2 / ((1-z^2) P'^2)) / 2
    }
}


int tags_fill_tables_init() {
    static double hx[GL_TOTAL], hw[GL_TOTAL];
    for (int q = 1; q <= QMAX; ++q) tags_gauss_legendre(q, hx + q * (q - 1) / 2, hw + q * (q - 1) / 2);
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glx, hx, sizeof(hx)));
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glw, hw, sizeof(hw)));
    static float fx[GL_MIX], fw[GL_MIX];
    for (int t = 0; t < GL_MIX; ++t) {
        fx[t] = (float)(hx[t] - 0.5);
        fw[t] = (float)hw[t];
    }
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glxm, fx, sizeof(fx)));
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glwm, fw, sizeof(fw)));
    return 0;
}

size_t tags_mixed_fill_workspace(int m) {
    const size_t np = (size_t)m * (m + 1) / 2;
    return np * 2 * (sizeof(uint16_t) + sizeof(PairRec)) + np * 2 * sizeof(int) + 2 * m * sizeof(float4) +
           4096 * sizeof(SampleF32) + 1024;
}

struct MixedFillWs {
    uint16_t* codes;
    PairRec* recs;
    int* list;
    int* nlist;
    float4* sdir;
    float4* idir;
    SampleF32* c32;
};

static MixedFillWs carve(void* ws, int m) {
    const size_t np = (size_t)m * (m + 1) / 2;
    char* b = reinterpret_cast<char*>(ws);
    MixedFillWs w;
    w.recs = reinterpret_cast<PairRec*>(b);
    b += np * 2 * sizeof(PairRec);
    w.sdir = reinterpret_cast<float4*>(b);
    b += m * sizeof(float4);
    w.idir = reinterpret_cast<float4*>(b);
    b += m * sizeof(float4);
    w.c32 = reinterpret_cast<SampleF32*>(b);
    b += 4096 * sizeof(SampleF32);
    w.list = reinterpret_cast<int*>(b);
    b += np * 2 * sizeof(int);
    w.nlist = reinterpret_cast<int*>(b);
    b += 16;
    w.codes = reinterpret_cast<uint16_t*>(b);
    return w;
}

int tags_launch_pair_plan(const double* d_elec, const double* d_img, int m, int has_img, void* ws, cudaStream_t st) {
    MixedFillWs w = carve(ws, m);
    const long long npairs = (long long)m * (m + 1) / 2;
    TAGS_CUDA_OK(cudaMemsetAsync(w.nlist, 0, sizeof(int), st));
    k_seg_dirs<<<(m + 127) / 128, 128, 0, st>>>(d_elec, d_img, m, has_img, w.sdir, w.idir);
    k_pair_plan<<<(unsigned)((npairs + 127) / 128), 128, 0, st>>>(d_elec, d_img, m, has_img, w.codes, w.recs, w.nlist,
                                                                 w.list);
    tags_note_launch(2);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_fill_mixed(const double* d_elec, const double* d_img, int m, void* ws, const SampleCoef* d_coef,
                           int nsamp, float2* d_zl, float2* d_zt, float2* d_zlo, float2* d_ztlo, long long bstride,
                           int has_img, const SpecialEntries& sp, const MomentFill& mf, int* d_status,
                           cudaStream_t st, float* rowpart) {
    if (m <= 0 || nsamp <= 0) return 0;
    if (nsamp > 4096 || nsamp > mf.batch)
        return tags_fail_cuda(cudaErrorInvalidValue, "fill_mixed: batch above capacity", __FILE__, __LINE__);
    MixedFillWs w = carve(ws, m);
    int pf = tags_prof_begin(TAGS_PROF_FILL_MIXED, st);
    MomCoef* mc = reinterpret_cast<MomCoef*>(mf.coef);
    k_mom_coef<<<(nsamp + 127) / 128, 128, 0, st>>>(d_coef, nsamp, mf.dmax, mc, mf.ok);
    k_mom_table<<<dim3((nsamp + 127) / 128, mf.nb), 128, 0, st>>>(d_coef, nsamp, mf.nb, mf.batch, mf.tab);
    k_coef32<<<(nsamp + 127) / 128, 128, 0, st>>>(d_coef, nsamp, w.c32);
    const int KB = (m + 31) / 32;
    const long long ntiles = 16LL * (KB - 1) * KB + m;
    dim3 grid((unsigned)((ntiles + MOM_WARPS - 1) / MOM_WARPS), (unsigned)((nsamp + 31) / 32));
    k_fill_moment<<<grid, MOM_WARPS * 32, 0, st>>>(m, mf.mom, reinterpret_cast<const MomRec*>(mf.rec), mc, mf.tab,
                                                   mf.batch, mf.nb, nsamp, d_zl, d_zt, d_zlo, d_ztlo, bstride, ntiles,
                                                   d_status);
    // samples the series does not reach: FP32 quadrature (warps with none leave at once)
    dim3 gq((unsigned)((ntiles + FILL_WARPS - 1) / FILL_WARPS), (unsigned)((nsamp + 31) / 32));
    k_fill_mixed<<<gq, FILL_WARPS * 32, 0, st>>>(d_elec, d_img, w.sdir, w.idir, m, w.codes, w.recs, w.c32, nsamp,
                                                 d_zl, d_zt, bstride, has_img, ntiles, d_status, mf.ok, d_zlo,
                                                 d_ztlo);
    dim3 gs((unsigned)((sp.n + SPEC_WARPS - 1) / SPEC_WARPS), (unsigned)((nsamp + 31) / 32));
    k_fill_special64<<<gs, SPEC_WARPS * 32, 0, st>>>(d_elec, d_img, m, sp.ent, sp.n, d_coef, nsamp, d_zl, d_zt, d_zlo,
                                                     d_ztlo, bstride, d_status, sp.tm, sp.tdmax);
    const dim3 gm((unsigned)((long long)KB * (KB + 1) / 2), (unsigned)((2 * nsamp + MIRROR_MATS - 1) / MIRROR_MATS));
    float* pmax = rowpart;
    float* psum = rowpart ? rowpart + (size_t)2 * nsamp * KB * m : nullptr;
    k_zmirror<<<gm, 256, 0, st>>>(d_zl, d_zt, bstride, m, 2 * nsamp, pmax, psum);
    k_zmirror<<<gm, 256, 0, st>>>(d_zlo, d_ztlo, bstride, m, 2 * nsamp, nullptr, nullptr);
    tags_prof_end(TAGS_PROF_FILL_MIXED, pf, st, 0.0, 0.0);
    tags_note_launch(8);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// Moments of every (pair, kind), once per plan, and the per-pass tables.
int tags_moment_fill_build(const double* d_elec, const double* d_img, int m, int has_img, const double* h_elec,
                           const double* h_img, int batch, MomentFill* mf, cudaStream_t st) {
    tags_moment_fill_free(mf);
    const long long npk = (long long)m * (m + 1);
    // |r - R| <= (L_i + L_k) / 2 + h / 2 <= Lmax + h / 2; buckets up to the
    // largest midpoint distance (bounding box of the midpoints and images)
    double lmax = 0.0, lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int e = 0; e < m; ++e) {
        lmax = fmax(lmax, h_elec[11 * e + 9]);
        for (int c = 0; c < 3; ++c) {
            const double v = h_elec[11 * e + 6 + c];
            lo[c] = fmin(lo[c], v);
            hi[c] = fmax(hi[c], v);
            if (has_img) {
                const double u = h_img[11 * e + 6 + c];
                lo[c] = fmin(lo[c], u);
                hi[c] = fmax(hi[c], u);
            }
        }
    }
    const double diag = sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                             (hi[2] - lo[2]) * (hi[2] - lo[2]));
    mf->dmax = lmax + 0.5 * MOM_H;
    mf->nb = (int)ceil(diag / MOM_H) + 2;
    mf->batch = batch;
    TAGS_CUDA_OK(cudaMalloc(&mf->mom, sizeof(float) * MOM_FLOATS * npk));
    TAGS_CUDA_OK(cudaMalloc(&mf->rec, sizeof(MomRec) * npk));
    TAGS_CUDA_OK(cudaMalloc(&mf->coef, sizeof(MomCoef) * batch));
    TAGS_CUDA_OK(cudaMalloc(&mf->ok, sizeof(int) * batch));
    TAGS_CUDA_OK(cudaMalloc(&mf->tab, sizeof(float4) * 3 * (size_t)mf->nb * batch));
    k_moments<<<(unsigned)((npk + 3) / 4), 128, 0, st>>>(d_elec, d_img, m, has_img, mf->mom,
                                                          reinterpret_cast<MomRec*>(mf->rec));
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

void tags_moment_fill_free(MomentFill* mf) {
    void* ptrs[] = {mf->mom, mf->rec, mf->coef, mf->ok, mf->tab};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    *mf = MomentFill{};
}

// The special entries from the pair plan's list of pairs with a touching (or
// degenerate) kind, plus every diagonal entry; sorted by pair index, so the
// list comes out in the same order on every build.
int tags_mixed_special_build(void* ws, int m, int batch, SpecialEntries* sp, cudaStream_t st) {
    MixedFillWs w = carve(ws, m);
    int nt = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(&nt, w.nlist, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    std::vector<int> tl(2 * (size_t)nt);
    if (nt > 0) {
        TAGS_CUDA_OK(cudaMemcpyAsync(tl.data(), w.list, sizeof(int) * 2 * nt, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    std::map<long long, int> kinds;
    for (int t = 0; t < nt; ++t) kinds[tl[2 * t]] |= tl[2 * t + 1] & 3;
    for (int i = 0; i < m; ++i) kinds[(long long)i * (2LL * m - i + 1) / 2] |= 4;
    const int n = (int)kinds.size();
    std::vector<int2> ent;
    ent.reserve(n);
    for (const auto& kv : kinds) ent.push_back(make_int2((int)kv.first, kv.second));
    tags_mixed_special_free(sp);
    TAGS_CUDA_OK(cudaMalloc(&sp->ent, sizeof(int2) * n));
    TAGS_CUDA_OK(cudaMemcpy(sp->ent, ent.data(), sizeof(int2) * n, cudaMemcpyHostToDevice));
    sp->n = n;
    (void)batch;
    return 0;
}

int tags_mixed_special_moments(const double* d_elec, const double* d_img, int m, double lmax, SpecialEntries* sp,
                               cudaStream_t st) {
    if (sp->tm) cudaFree(sp->tm);
    sp->tm = nullptr;
    if (sp->n <= 0) return 0;
    TAGS_CUDA_OK(cudaMalloc(&sp->tm, sizeof(double) * 2 * MOM_N * (size_t)sp->n));
    k_touch_moments<<<(unsigned)((sp->n + 3) / 4), 128, 0, st>>>(d_elec, d_img, m, sp->ent, sp->n, sp->tm);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    sp->tdmax = 2.0 * lmax;
    return 0;
}

void tags_mixed_special_free(SpecialEntries* sp) {
    void* ptrs[] = {sp->ent, sp->tm};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    *sp = SpecialEntries{};
}

int tags_mixed_touch_count(void* ws, int m, cudaStream_t st, int* out) {
    MixedFillWs w = carve(ws, m);
    TAGS_CUDA_OK(cudaMemcpyAsync(out, w.nlist, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

// ---- mHEM: per-sample rescale of static potentials ----------------------------
//
// The reference's mHEM examples (examples/three_grids.c:335-350) fill ZL/ZT
// per sample from static potentials computed once (INTG_MHEM integrals,
// direct and image) times e^{-gamma rbar} of the segments' midpoint distance:
//   ZL = iwu (e^{-gamma r} PL + ref_l e^{-gamma r'} PLi),
//   ZT = 1/(4 pi kappa) (e^{-gamma r} PT + ref_t e^{-gamma r'} PTi),
// r' the distance to the image; the coefficients come as cL = iwu, cLi =
// ref_l iwu, cT, cTi. pot holds PL, PT, PLi, PTi (lower triangles, element
// (k, i) at k + m i).

TAGS_D double mid_dist(const double* a, const double* b) {
    const double dx = a[6] - b[6], dy = a[7] - b[7], dz = a[8] - b[8];
    return sqrt(dx * dx + dy * dy + dz * dz);
}

__global__ void k_mhem_fp64(const double* __restrict__ elec, const double* __restrict__ img, int m,
                            const double2* __restrict__ pot, const SampleCoef* __restrict__ coef, int nsamp,
                            FillOut out, int has_img, int* status) {
    const long long npairs = (long long)m * (m + 1) / 2;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int smp = blockIdx.y;
    if (p >= npairs || smp >= nsamp) return;
    int i, k;
    pair_index(p, m, i, k);
    const SampleCoef c = coef[smp];
    const long long mm = (long long)m * m, e = k + (long long)m * i;
    const double2 ng = make_double2(-c.gamma.x, -c.gamma.y);
    const double2 e1 = cexp_d(cscale(ng, mid_dist(elec + 11LL * k, elec + 11LL * i)));
    double2 zl = cmul(cmul(e1, pot[e]), c.cL);
    double2 zt = cmul(cmul(e1, pot[mm + e]), c.cT);
    if (has_img) {
        const double2 e2 = cexp_d(cscale(ng, mid_dist(elec + 11LL * k, img + 11LL * i)));
        zl = cadd(zl, cmul(cmul(e2, pot[2 * mm + e]), c.cLi));
        zt = cadd(zt, cmul(cmul(e2, pot[3 * mm + e]), c.cTi));
    }
    if (!isfinite(zl.x + zl.y + zt.x + zt.y)) raise_status(status, TAGS_ST_NONFINITE);
    zl = cscale(zl, out.sign);
    zt = cscale(zt, out.sign);
    const long long bs = out.batch_stride * smp;
    store(out.zl + bs, (long long)(out.row0_l + k) + out.ld * (out.col0_l + i), zl, out.accumulate != 0);
    store(out.zt + bs, (long long)(out.row0_t + k) + out.ld * (out.col0_t + i), zt, out.accumulate != 0);
    if (out.mirror && k != i) {
        store(out.zl + bs, (long long)(out.row0_l + i) + out.ld * (out.col0_l + k), zl, out.accumulate != 0);
        store(out.zt + bs, (long long)(out.row0_t + i) + out.ld * (out.col0_t + k), zt, out.accumulate != 0);
    }
}

constexpr int MIX_SG = 4;   // samples per thread of the mHEM rescale

// Mixed form: the exponentials from the pair plan's two-float midpoint
// distances (anchor_df, exact range reduction), products in FP32; ZL at zl,
// ZT at zt (complex FP32, both triangles). A thread per (pair, sample group).
__global__ void __launch_bounds__(128) k_mhem_mixed(int m, const double2* __restrict__ pot,
                                                    const PairRec* __restrict__ recs,
                                                    const SampleF32* __restrict__ coef, int nsamp, float2* zl0,
                                                    float2* zt0, long long bstride, int has_img, int* status) {
    const long long npairs = (long long)m * (m + 1) / 2;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int s0 = blockIdx.y * MIX_SG;
    if (p >= npairs || s0 >= nsamp) return;
    int i, k;
    pair_index(p, m, i, k);
    const long long mm = (long long)m * m, e = k + (long long)m * i;
    const double2 pl = pot[e], pt = pot[mm + e];
    const float2 PL = make_float2((float)pl.x, (float)pl.y), PT = make_float2((float)pt.x, (float)pt.y);
    float2 PLi = make_float2(0.f, 0.f), PTi = make_float2(0.f, 0.f);
    if (has_img) {
        const double2 pli = pot[2 * mm + e], pti = pot[3 * mm + e];
        PLi = make_float2((float)pli.x, (float)pli.y);
        PTi = make_float2((float)pti.x, (float)pti.y);
    }
    const PairRec r1 = recs[2 * p], r2 = recs[2 * p + 1];     // r1 has r = 0 on the diagonal
#pragma unroll
    for (int q = 0; q < MIX_SG; ++q) {
        if (s0 + q >= nsamp) break;
        const SampleF32 c = coef[s0 + q];
        const float2 a1 = anchor_df(c.grh, c.grl, c.gih, c.gil, k == i ? 0.f : r1.rch, k == i ? 0.f : r1.rcl);
        float2 zl = fmulc(fmulc(a1, PL), c.cL), zt = fmulc(fmulc(a1, PT), c.cT);
        if (has_img) {
            const float2 a2 = anchor_df(c.grh, c.grl, c.gih, c.gil, r2.rch, r2.rcl);
            zl = ffmac(fmulc(a2, PLi), c.cLi, zl);
            zt = ffmac(fmulc(a2, PTi), c.cTi, zt);
        }
        if (!isfinite(zl.x + zl.y + zt.x + zt.y)) raise_status(status, TAGS_ST_NONFINITE);
        const long long bs = bstride * (s0 + q);
        zl0[bs + k + (long long)m * i] = zl;
        zt0[bs + k + (long long)m * i] = zt;
        if (k != i) {
            zl0[bs + i + (long long)m * k] = zl;
            zt0[bs + i + (long long)m * k] = zt;
        }
    }
}

// Static potentials of the mHEM fill (once per geometry): direct into pot[0..1],
// images into pot[2..3], lower triangles.
int tags_launch_mhem_potentials(const double* d_elec, const double* d_img, int m, int has_img, double2* d_pot,
                                SampleCoef* d_coef1, int* d_status, cudaStream_t st) {
    const long long mm = (long long)m * m;
    TAGS_CUDA_OK(cudaMemsetAsync(d_pot, 0, sizeof(double2) * 4 * mm, st));
    SampleCoef one{};          // scale factors are 1 for INTG_MHEM; gamma unused
    TAGS_CUDA_OK(cudaMemcpyAsync(d_coef1, &one, sizeof(one), cudaMemcpyHostToDevice, st));
    FillOut out{};
    out.zl = d_pot;
    out.zt = d_pot + mm;
    out.ld = m;
    out.sign = 1.0;
    int err = tags_launch_fill_fp64(d_elec, d_img, m, d_coef1, 1, out, TAGS_FILL_DIRECT, TAGS_INTG_MHEM, 1, d_status, st);
    if (!err && has_img) {
        out.zl = d_pot + 2 * mm;
        out.zt = d_pot + 3 * mm;
        err = tags_launch_fill_fp64(d_elec, d_img, m, d_coef1, 1, out, TAGS_FILL_IMAGE, TAGS_INTG_MHEM, 1, d_status,
                                    st);
    }
    return err;
}

int tags_launch_mhem_fp64(const double* d_elec, const double* d_img, int m, int has_img, const double2* d_pot,
                          const SampleCoef* d_coef, int nsamp, const FillOut& out, int* d_status, cudaStream_t st) {
    if (m <= 0 || nsamp <= 0) return 0;
    const long long npairs = (long long)m * (m + 1) / 2;
    int pf = tags_prof_begin(TAGS_PROF_FILL_FP64, st);
    k_mhem_fp64<<<dim3((unsigned)((npairs + 127) / 128), (unsigned)nsamp), 128, 0, st>>>(d_elec, d_img, m, d_pot,
                                                                                       d_coef, nsamp, out, has_img,
                                                                                       d_status);
    tags_prof_end(TAGS_PROF_FILL_FP64, pf, st, 0.0, 0.0);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_mhem_mixed(int m, int has_img, const double2* d_pot, void* ws, const SampleCoef* d_coef, int nsamp,
                           float2* d_zl, float2* d_zt, long long bstride, int* d_status, cudaStream_t st) {
    if (m <= 0 || nsamp <= 0) return 0;
    if (nsamp > 4096) return tags_fail_cuda(cudaErrorInvalidValue, "mhem_mixed: batch above 4096", __FILE__, __LINE__);
    MixedFillWs w = carve(ws, m);
    const long long npairs = (long long)m * (m + 1) / 2;
    int pf = tags_prof_begin(TAGS_PROF_FILL_MIXED, st);
    k_coef32<<<(nsamp + 127) / 128, 128, 0, st>>>(d_coef, nsamp, w.c32);
    k_mhem_mixed<<<dim3((unsigned)((npairs + 127) / 128), (unsigned)((nsamp + MIX_SG - 1) / MIX_SG)), 128, 0, st>>>(
        m, d_pot, w.recs, w.c32, nsamp, d_zl, d_zt, bstride, has_img, d_status);
    tags_prof_end(TAGS_PROF_FILL_MIXED, pf, st, 0.0, 0.0);
    tags_note_launch(2);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_fill_fp64(const double* d_elec, const double* d_img, int m, const SampleCoef* d_coef,
                          int nsamp, const FillOut& out, int mode, int itype, int tight, int* d_status,
                          cudaStream_t st) {
    if (m <= 0 || nsamp <= 0) return 0;
    const long long npairs = (long long)m * (m + 1) / 2;
    dim3 grid((unsigned)((npairs + 127) / 128), (unsigned)nsamp);
    int pf = tags_prof_begin(TAGS_PROF_FILL_FP64, st);
    k_fill_fp64<<<grid, 128, 0, st>>>(d_elec, d_img, m, d_coef, nsamp, out, mode, itype, tight, d_status);
    tags_prof_end(TAGS_PROF_FILL_FP64, pf, st, 0.0, 0.0);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_path_pairs(const double* d_elec, int m, const double* d_paths, int npaths, const SampleCoef* d_coef,
                           int nsamp, double2* d_jj, int* d_status, cudaStream_t st) {
    if (m <= 0 || npaths <= 0 || nsamp <= 0) return 0;
    if (nsamp > 65535) return tags_fail_cuda(cudaErrorInvalidValue, "path_pairs: more than 65535 samples", __FILE__,
                                             __LINE__);
    const long long n = (long long)m * npaths;
    k_path_pairs<<<dim3((unsigned)((n + 127) / 128), (unsigned)nsamp), 128, 0, st>>>(d_elec, m, d_paths, npaths,
                                                                                       d_coef, d_jj, d_status);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}
