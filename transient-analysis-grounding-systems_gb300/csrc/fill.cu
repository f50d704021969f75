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
#include "tags_common.cuh"
#include "tags_internal.h"

namespace {

constexpr int QMAX = 40;                      // largest Gauss-Legendre order tabulated
constexpr int GL_TOTAL = QMAX * (QMAX + 1) / 2;

__device__ double g_glx[GL_TOTAL];            // nodes on [0,1], order q at q(q-1)/2
__device__ double g_glw[GL_TOTAL];            // weights on [0,1]

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
    int extra = (int)ceil((tight ? 1.5 : 1.0) * gl);
    int q = base + extra;
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
        int q = 16 + 2 * (int)ceil(gabs * lmax);
        if (!tight) q = 10 + (int)ceil(gabs * lmax);
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
    // p enumerates (i, k), k >= i, column by column: start(i) = i(2m - i + 1)/2
    double b = 2.0 * m + 1.0;
    int ii = (int)floor((b - sqrt(fmax(b * b - 8.0 * (double)p, 0.0))) * 0.5);
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

__global__ void k_pair_plan(const double* __restrict__ elec, const double* __restrict__ img, int m, int has_img,
                            uint16_t* __restrict__ codes) {
    const long long npairs = (long long)m * (m + 1) / 2;
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    int i, k;
    pair_index(p, m, i, k);
    Seg S, R;
    ld_seg(elec + 11LL * i, S);
    uint16_t cd = 0, ci = 0;
    if (k != i) {
        ld_seg(elec + 11LL * k, R);
        cd = classify_pair(S, R);
    }
    if (has_img) {
        ld_seg(img + 11LL * k, R);
        ci = classify_pair(S, R);
    }
    codes[2 * p] = cd;
    codes[2 * p + 1] = ci;
}

// e^{-gamma r} for r in FP64, result FP32: the exponent and the phase are
// reduced in FP64 (2^-t with t split into integer and fraction, phase modulo
// 2 pi), the remaining small arguments are evaluated in FP32.
TAGS_D float2 anchor_f32(double2 gamma, double r) {
    const double LOG2E = 1.4426950408889634;
    double t = gamma.x * r * LOG2E;                  // e^{-Re(gamma) r} = 2^{-t}
    double ti = floor(t);
    float mag = ldexpf(exp2f(-(float)(t - ti)), -(int)fmin(ti, 1000.0));
    double ph = gamma.y * r;                         // e^{-j Im(gamma) r}
    ph -= TAGS_TWO_PI * rint(ph * (1.0 / TAGS_TWO_PI));
    float sn, cs;
    sincosf((float)ph, &sn, &cs);
    return make_float2(mag * cs, -mag * sn);
}

constexpr int MIX_SG = 8;   // samples per thread

// Mixed-form fill: one thread per (pair, group of up to MIX_SG samples).
// Regular pairs in FP32 (panel anchors in FP64), touching pairs in FP64.
// Writes ZL (at zl) and ZT (at zt), lower + mirrored upper, FP64 storage.
__global__ void __launch_bounds__(128, 1) k_fill_mixed(const double* __restrict__ elec, const double* __restrict__ img,
                                                    int m, const uint16_t* __restrict__ codes,
                                                    const SampleCoef* __restrict__ coef, int nsamp, FillOut out,
                                                    int has_img, int* status) {
    __shared__ double sx[GL_TOTAL], sw[GL_TOTAL];
    for (int t = threadIdx.x; t < GL_TOTAL; t += blockDim.x) { sx[t] = g_glx[t]; sw[t] = g_glw[t]; }
    __syncthreads();
    GLTab gl{sx, sw};
    const long long npairs = (long long)m * (m + 1) / 2;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int s0 = blockIdx.y * MIX_SG;
    if (p >= npairs || s0 >= nsamp) return;
    const int ns = min(MIX_SG, nsamp - s0);
    int i, k;
    pair_index(p, m, i, k);
    Seg S;
    ld_seg(elec + 11LL * i, S);
    const double ds[3] = {S.b[0] - S.a[0], S.b[1] - S.a[1], S.b[2] - S.a[2]};
    double2 zl[MIX_SG], zt[MIX_SG];
    double2 gam[MIX_SG];
    double gmax = 0.0;
#pragma unroll
    for (int q = 0; q < MIX_SG; ++q) {
        zl[q] = zt[q] = cz(0.0, 0.0);
        gam[q] = q < ns ? coef[s0 + q].gamma : cz(0.0, 0.0);
        gmax = fmax(gmax, sqrt(cabs2(gam[q])));
    }
    for (int kind = 0; kind < 2; ++kind) {
        if (kind == 1 && !has_img) break;
        Seg R;
        if (kind == 0 && k == i) {
            double intg = self_integral_d(S);
#pragma unroll
            for (int q = 0; q < MIX_SG; ++q) {
                if (q >= ns) break;
                SampleCoef c = coef[s0 + q];
                zl[q] = cscale(c.cL, intg);
                zt[q] = cscale(c.cT, intg / (S.len * S.len));
            }
            continue;
        }
        ld_seg((kind == 0 ? elec : img) + 11LL * k, R);
        const uint16_t code = codes[2 * p + kind];
        double cost = 0.0;
        for (int d = 0; d < 3; ++d) cost += ds[d] * (R.b[d] - R.a[d]);
        cost = fabs(cost);
        const double lsr = S.len * R.len;
        double2 J[MIX_SG];
        if (code & PC_DEGEN) {
            raise_status(status, TAGS_ST_DEGENERATE_PAIR);
#pragma unroll
            for (int q = 0; q < MIX_SG; ++q) J[q] = cz(nan(""), nan(""));
        } else if (code & PC_TOUCH) {
            int ia, ib;
            touching(R, S, 1e-9 * fmax(S.len, R.len), ia, ib);
#pragma unroll
            for (int q = 0; q < MIX_SG; ++q) {
                int qt = min(QMAX, 10 + (int)ceil(sqrt(cabs2(gam[q])) * fmax(S.len, R.len)));
                J[q] = q < ns ? j_touch(R, S, ia, ib, gam[q], false, qt, gl) : cz(0.0, 0.0);
            }
        } else {
            const int P = code & 63;
            const int qg = (code >> 6) & 63;
            const int qq = min(24, qg + (int)ceil(gmax * fmax(S.len, R.len) / P));
            const double* x = gl.x + gl_off(qq);
            const double* w = gl.w + gl_off(qq);
            const double h = 1.0 / (double)P;
            const double dr[3] = {R.b[0] - R.a[0], R.b[1] - R.a[1], R.b[2] - R.a[2]};
            const float3 hr = make_float3((float)(dr[0] * h), (float)(dr[1] * h), (float)(dr[2] * h));
            const float3 hs = make_float3((float)(ds[0] * h), (float)(ds[1] * h), (float)(ds[2] * h));
            float2 acc[MIX_SG];
            float gre[MIX_SG], gim[MIX_SG];
#pragma unroll
            for (int q = 0; q < MIX_SG; ++q) {
                acc[q] = make_float2(0.f, 0.f);
                gre[q] = (float)gam[q].x;
                gim[q] = (float)gam[q].y;
            }
            for (int pi = 0; pi < P; ++pi) {
                for (int pj = 0; pj < P; ++pj) {
                    double cr[3], dd[3];
                    for (int d = 0; d < 3; ++d) {
                        cr[d] = R.a[d] + (pi + 0.5) * h * dr[d];
                        dd[d] = cr[d] - (S.a[d] + (pj + 0.5) * h * ds[d]);
                    }
                    const double rc = sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                    const float3 D = make_float3((float)dd[0], (float)dd[1], (float)dd[2]);
                    const float rcf = (float)rc;
                    float2 psum[MIX_SG];
#pragma unroll
                    for (int q = 0; q < MIX_SG; ++q) psum[q] = make_float2(0.f, 0.f);
                    for (int qi = 0; qi < qq; ++qi) {
                        const float a = (float)(x[qi] - 0.5);
                        const float wi = (float)w[qi];
                        for (int qj = 0; qj < qq; ++qj) {
                            const float b = (float)(x[qj] - 0.5);
                            // u = a hr - b hs: offset of the point pair from the panel centres
                            float ux = a * hr.x - b * hs.x, uy = a * hr.y - b * hs.y, uz = a * hr.z - b * hs.z;
                            float e = 2.f * (D.x * ux + D.y * uy + D.z * uz) + (ux * ux + uy * uy + uz * uz);
                            float rp = sqrtf(rcf * rcf + e);
                            float del = e / (rp + rcf);                 // r_p - r_c without cancellation
                            float wt = wi * (float)w[qj] / rp;
#pragma unroll
                            for (int q = 0; q < MIX_SG; ++q) {
                                float mg = expf(-gre[q] * del);
                                float sn, cs;
                                sincosf(gim[q] * del, &sn, &cs);
                                psum[q].x = fmaf(wt * mg, cs, psum[q].x);
                                psum[q].y = fmaf(-wt * mg, sn, psum[q].y);
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < MIX_SG; ++q) {
                        if (q < ns) acc[q] = ffmac(anchor_f32(gam[q], rc), psum[q], acc[q]);
                    }
                }
            }
            const double h2 = h * h;
#pragma unroll
            for (int q = 0; q < MIX_SG; ++q) J[q] = cz((double)acc[q].x * h2, (double)acc[q].y * h2);
        }
#pragma unroll
        for (int q = 0; q < MIX_SG; ++q) {
            if (q >= ns) break;
            SampleCoef c = coef[s0 + q];
            double2 intg = cscale(J[q], lsr);
            double2 cL = kind == 0 ? c.cL : c.cLi, cT = kind == 0 ? c.cT : c.cTi;
            zt[q] = cadd(zt[q], cmul(cscale(cT, 1.0 / lsr), intg));
            bool keep = kind == 0 ? !(cost < TAGS_DBL_EPSILON) : (cost > TAGS_DBL_EPSILON);
            if (keep) zl[q] = cadd(zl[q], cscale(cmul(cL, intg), cost / lsr));
        }
    }
#pragma unroll
    for (int q = 0; q < MIX_SG; ++q) {
        if (q >= ns) break;
        const int smp = s0 + q;
        const long long bs = out.batch_stride * smp;
        double2 l = cscale(zl[q], out.sign), t = cscale(zt[q], out.sign);
        if (!isfinite(l.x + l.y + t.x + t.y)) raise_status(status, TAGS_ST_NONFINITE);
        out.zl[bs + (long long)(out.row0_l + k) + out.ld * (out.col0_l + i)] = l;
        out.zt[bs + (long long)(out.row0_t + k) + out.ld * (out.col0_t + i)] = t;
        if (out.mirror && k != i) {
            out.zl[bs + (long long)(out.row0_l + i) + out.ld * (out.col0_l + k)] = l;
            out.zt[bs + (long long)(out.row0_t + i) + out.ld * (out.col0_t + k)] = t;
        }
    }
}

// Gauss-Legendre nodes/weights by Newton iteration on P_q (host side).
void gauss_legendre(int q, double* x, double* w) {
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

}  // namespace

int tags_fill_tables_init() {
    static double hx[GL_TOTAL], hw[GL_TOTAL];
    for (int q = 1; q <= QMAX; ++q) gauss_legendre(q, hx + q * (q - 1) / 2, hw + q * (q - 1) / 2);
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glx, hx, sizeof(hx)));
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_glw, hw, sizeof(hw)));
    return 0;
}

int tags_launch_pair_plan(const double* d_elec, const double* d_img, int m, int has_img, uint16_t* d_codes,
                          cudaStream_t st) {
    const long long npairs = (long long)m * (m + 1) / 2;
    k_pair_plan<<<(unsigned)((npairs + 127) / 128), 128, 0, st>>>(d_elec, d_img, m, has_img, d_codes);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_fill_mixed(const double* d_elec, const double* d_img, int m, const uint16_t* d_codes,
                           const SampleCoef* d_coef, int nsamp, const FillOut& out, int has_img, int* d_status,
                           cudaStream_t st) {
    if (m <= 0 || nsamp <= 0) return 0;
    const long long npairs = (long long)m * (m + 1) / 2;
    dim3 grid((unsigned)((npairs + 127) / 128), (unsigned)((nsamp + MIX_SG - 1) / MIX_SG));
    int pf = tags_prof_begin(TAGS_PROF_FILL_MIXED, st);
    k_fill_mixed<<<grid, 128, 0, st>>>(d_elec, d_img, m, d_codes, d_coef, nsamp, out, has_img, d_status);
    tags_prof_end(TAGS_PROF_FILL_MIXED, pf, st, 0.0, 0.0);
    tags_note_launch();
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
