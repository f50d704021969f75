// Mixed-precision batched solve of the immittance system.
//
// Same system as the reference's solve_immittance (src/linalg.c:112-139):
//     W_G = [ 0   A^T  B^T ]      x = [U; I_L; I_T],  b = [I_E; 0; 0]
//           [ A  -ZL   0   ]
//           [ B   0   -ZT  ]
// solved here as follows:
//   0. impedance blocks as float pairs (hi in Z, lo in Zlo), good to ~1e-13:
//      regular pairs from the moment expansion (FP64 geometry moments, series
//      in float pairs), pairs sharing an endpoint (log-singular) and the
//      diagonal's closed form in FP64 per sample; the refinement solves this
//      matrix, the factorisation uses its FP32 high parts;
//   1. static symmetric ordering P: ZL rows, ZT rows, then node rows, so that
//      the elimination meets the impedance blocks (large diagonals) before the
//      zero Y_E block and needs no pivot search;
//   2. symmetric scaling D = diag(1/sqrt(max_j |W'_ij|)), W'' = D P W P^T D;
//   3. LDL^T of W'' without pivoting, complex FP32 storage, trailing updates
//      and triangular-solve panels on the tensor cores (ldl_tc.cu);
//   4. iterative refinement: x in FP64, r = b - W x with the exact incidence
//      (sparse, +-1 / 0.5) in FP64 and the impedance blocks times x in
//      two-float arithmetic (about 2^-44 relative), the correction from the
//      FP32 factors; a sample stops once its predicted error is below the
//      tolerance (1e-9 |x|) or its corrections stop shrinking. The stopping
//      decision runs on the device (k_ir_decide) after each correction and
//      before the residual, which only the samples that go on then form; one
//      refinement step is a fixed launch sequence that a CUDA graph repeats
//      under a conditional while-node. The first step's right-hand side is b,
//      zero in the impedance rows, and its forward sweep starts at the node
//      rows;
//   5. samples that do not converge are re-solved by the plain FP64 path
//      (LU with partial pivoting).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

TAGS_D void atomic_max_nonneg(double* addr, double v) {
    // IEEE order of non-negative doubles matches the order of their bits
    atomicMax(reinterpret_cast<unsigned long long*>(addr), (unsigned long long)__double_as_longlong(v));
}

// Row maxima (and row sums) of the impedance blocks: Z is symmetric, so row k
// equals column k (contiguous). One warp per (row, block, sample).
__global__ void k_rowstats(const float2* __restrict__ Z, int m, double* __restrict__ scale, double* __restrict__ rsum,
                           float* __restrict__ scalef, int N) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    int blk = blockIdx.y;       // 0 = ZL, 1 = ZT
    int b = blockIdx.z;
    if (warp >= m) return;
    const float2* col = Z + (size_t)b * 2 * m * m + (size_t)blk * m * m + (size_t)m * warp;
    float mx = 0.f, sm = 0.f;       // a scaling and a norm estimate: FP32 is plenty
    for (int j = lane; j < m; j += 32) {
        const float2 z = col[j];
        const float a = sqrtf(z.x * z.x + z.y * z.y);
        mx = fmaxf(mx, a);
        sm += a;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        sm += __shfl_down_sync(0xffffffffu, sm, o);
    }
    if (lane == 0) {
        double inc = blk == 0 ? 1.0 : 0.5;            // incidence entries of the row
        int row = blk * m + warp;                      // reordered index
        const double sc = 1.0 / sqrt(fmax((double)mx, inc));
        scale[(size_t)b * N + row] = sc;
        scalef[(size_t)b * N + row] = (float)sc;             // the build's copy (no FP64 per element there)
        rsum[(size_t)b * N + row] = (double)sm + 2.0 * inc;
    }
}

// The same statistics from the partials the fill's mirror pass leaves
// (max and sum of |Z[R][j]| per row R and 32-column block t, [mat][t][R]):
// the max over t, the sum over t in order. One thread per (row, block, sample).
__global__ void k_rowstats_part(const float* __restrict__ pmax, const float* __restrict__ psum, int m,
                                double* __restrict__ scale, double* __restrict__ rsum, float* __restrict__ scalef,
                                int N) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, blk = blockIdx.y, b = blockIdx.z;
    if (r >= m) return;
    const int KB = (m + 31) / 32;
    const long long base = (long long)(2 * b + blk) * KB * m + r;
    float mx = 0.f, sm = 0.f;
    for (int t = 0; t < KB; ++t) {
        mx = fmaxf(mx, pmax[base + (long long)t * m]);
        sm += psum[base + (long long)t * m];
    }
    const double inc = blk == 0 ? 1.0 : 0.5;            // incidence entries of the row
    const int row = blk * m + r;                          // reordered index
    const double sc = 1.0 / sqrt(fmax((double)mx, inc));
    scale[(size_t)b * N + row] = sc;
    scalef[(size_t)b * N + row] = (float)sc;
    rsum[(size_t)b * N + row] = (double)sm + 2.0 * inc;
}

// Node rows: max |entry| = 1 (A) so the scale is 1; row sum = sum over
// incident segments of (1 + 0.5).
__global__ void k_rowstats_nodes(const int* __restrict__ node_ptr, int n, int m, double* __restrict__ scale,
                                 double* __restrict__ rsum, float* __restrict__ scalef, int N) {
    int nd = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (nd >= n) return;
    scale[(size_t)b * N + 2 * m + nd] = 1.0;
    scalef[(size_t)b * N + 2 * m + nd] = 1.f;
    rsum[(size_t)b * N + 2 * m + nd] = 1.5 * (double)(node_ptr[nd + 1] - node_ptr[nd]);
}

// W'' (complex FP32, column-major N x N, reordered and scaled), lower triangle.
// A CTA writes BUILD_COLS columns of one sample, rows j .. N-1 of column j, in
// at most three plain row ranges: the column's impedance block (-Z d_i d_j),
// the zero ZT rows of a ZL column, and the node rows, which are zero but for
// the segment's incidence entries (start +1 / end -1 in the ZL columns, 0.5 in
// the ZT columns; node rows have scale 1), written after a barrier.
constexpr int BUILD_COLS = 4;      // columns of W'' per CTA (enough traffic per CTA to hide its start-up)

__global__ void __launch_bounds__(256) k_build(const float2* __restrict__ Z, const Incidence inc,
                                               const float* __restrict__ scale, int m, int n,
                                               float2* __restrict__ A) {
    const int N = n + 2 * m;
    const int b = blockIdx.y;
    const float* d = scale + (size_t)b * N;
    const float2* Zb = Z + (size_t)b * 2 * m * m;
    const float2 zero = make_float2(0.f, 0.f);
    for (int c = 0; c < BUILD_COLS; ++c) {
        const int j = blockIdx.x * BUILD_COLS + c;
        if (j >= N) break;
        float2* Aj = A + (size_t)b * N * N + (size_t)j * N;
        if (j >= 2 * m) {                                   // node columns: rows j .. N-1 are zero
            for (int i = j + (int)threadIdx.x; i < N; i += blockDim.x) Aj[i] = zero;
            continue;
        }
        const float dj = d[j];
        const int bj = j < m ? 0 : 1, e = j - bj * m;
        // zc[i] = Z_bj(i - bj m, e) for rows i of the column's impedance block
        const float2* zc = Zb + (size_t)bj * m * m + (size_t)m * e - (size_t)bj * m;
        for (int i = j + (int)threadIdx.x; i < (bj + 1) * m; i += blockDim.x) {
            const float2 z = zc[i];
            const float sc = d[i] * dj;
            Aj[i] = make_float2(-z.x * sc, -z.y * sc);
        }
        if (bj == 0)
            for (int i = m + (int)threadIdx.x; i < 2 * m; i += blockDim.x) Aj[i] = zero;
        for (int i = 2 * m + (int)threadIdx.x; i < N; i += blockDim.x) Aj[i] = zero;
        __syncthreads();                                    // the zeros land before the entries
        if (threadIdx.x == 0)
            for (int q = inc.seg_ptr[e]; q < inc.seg_ptr[e + 1]; ++q) {
                const float a = bj == 0 ? (float)inc.seg_a[q] : 0.5f;
                Aj[2 * m + inc.seg_node[q]] = make_float2(a * dj, 0.f);
            }
    }
}

TAGS_D int orig_of(int ip, int m, int n) {
    // reordered index -> original W_G index
    return ip < 2 * m ? n + ip : ip - 2 * m;
}

// rf = D P r (FP32)
// (first kernel of a refinement step: also clears the step's reductions)
__global__ void k_ir_rhs(const double2* __restrict__ r, const double* __restrict__ scale, int m, int n,
                         float2* __restrict__ rf, double* __restrict__ norms, double* __restrict__ dots) {
    const int N = n + 2 * m;
    int ip = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (blockIdx.x == 0 && threadIdx.x < 2) norms[4 * b + threadIdx.x] = 0.0;
    if (blockIdx.x == 0 && threadIdx.x < 4) dots[4 * b + threadIdx.x] = 0.0;
    if (ip >= N) return;
    double2 v = r[(size_t)b * N + orig_of(ip, m, n)];
    double s = scale[(size_t)b * N + ip];
    rf[(size_t)b * N + ip] = make_float2((float)(v.x * s), (float)(v.y * s));
}

// x += P^T D y (FP64); norms[b*4 + 0] = max|dx|, [1] = max|x|. From the
// third step on also dots[b*4 + 0..3] = (Re, Im of sum conj(yp) y, sum |yp|^2,
// sum |y|^2) against the previous step's correction yp, kept in yprev. 256
// threads per CTA.
__global__ void __launch_bounds__(256) k_ir_update(const float2* __restrict__ y, const double* __restrict__ scale,
                                                   int m, int n, double2* __restrict__ x, double* __restrict__ norms,
                                                   const int* __restrict__ active, float2* __restrict__ yprev,
                                                   double* __restrict__ dots, const int* __restrict__ step) {
    __shared__ double red[8][4];
    const int N = n + 2 * m;
    int ip = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (!active[b]) return;                                // the whole CTA
    const bool dot = *step >= 2;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    if (ip < N) {
        double s = scale[(size_t)b * N + ip];
        float2 yv = y[(size_t)b * N + ip];
        double2 dx = make_double2((double)yv.x * s, (double)yv.y * s);
        size_t o = (size_t)b * N + orig_of(ip, m, n);
        double2 xv = cadd(x[o], dx);
        x[o] = xv;
        atomic_max_nonneg(norms + 4 * b + 0, fabs(dx.x) + fabs(dx.y));
        atomic_max_nonneg(norms + 4 * b + 1, fabs(xv.x) + fabs(xv.y));
        float2* yp = yprev + (size_t)b * N + ip;
        if (dot) {
            const float2 pv = *yp;
            a[0] = (double)pv.x * yv.x + (double)pv.y * yv.y;
            a[1] = (double)pv.x * yv.y - (double)pv.y * yv.x;
            a[2] = (double)pv.x * pv.x + (double)pv.y * pv.y;
            a[3] = (double)yv.x * yv.x + (double)yv.y * yv.y;
        }
        *yp = yv;
    }
    if (!dot) return;                                      // the whole CTA
#pragma unroll
    for (int k = 0; k < 4; ++k)
        for (int o = 16; o > 0; o >>= 1) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 4; ++k) red[threadIdx.x >> 5][k] = a[k];
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w][threadIdx.x];
        atomicAdd(dots + 4 * b + threadIdx.x, t);
    }
}


// r = b - W x with the structure of W_G; norms[2] = max|r|.
// Node rows (sparse incidence, exact +-1 / 0.5) in FP64.
__global__ void k_residual_nodes(const Incidence inc, int m, int n, const double2* __restrict__ bvec,
                                 const double2* __restrict__ x, double2* __restrict__ r, double* __restrict__ norms,
                                 const int* __restrict__ active) {
    const int N = n + 2 * m;
    int row = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (row >= n || !active[b]) return;
    const double2* xb = x + (size_t)b * N;
    double2 acc = make_double2(0.0, 0.0);
    for (int q = inc.node_ptr[row]; q < inc.node_ptr[row + 1]; ++q) {
        int e = inc.node_seg[q];
        double a = inc.node_a[q];
        double2 il = xb[n + e], it = xb[n + m + e];
        acc.x += a * il.x + 0.5 * it.x;
        acc.y += a * il.y + 0.5 * it.y;
    }
    double2 rv = csub(bvec[(size_t)b * N + row], acc);
    r[(size_t)b * N + row] = rv;
    atomic_max_nonneg(norms + 4 * b + 2, fabs(rv.x) + fabs(rv.y));
}

// Two-float accumulator: the running FP32 sum hi of the products' leading
// parts and, in lo, every rounding error (of the products, exact by FMA, and of
// the additions to hi, exact by TwoSum). lo stays ~2^-24 of hi, so its own
// rounding is negligible and no renormalisation is needed until the end.
struct F2 {
    float hi, lo;
};
// a += z * (xh + xl) for real z (exact in FP32) and a two-float x
TAGS_D F2 f2_mac(F2 a, float z, float xh, float xl) {
    const float p = z * xh;
    float e = fmaf(z, xh, -p);
    e = fmaf(z, xl, e);
    const float s = a.hi + p;                 // TwoSum(a.hi, p)
    const float v = s - a.hi;
    const float t = (a.hi - (s - v)) + (p - v);
    a.hi = s;
    a.lo += t + e;
    return a;
}

// Impedance rows: r_k = b_k - (incidence terms - sum_j Z_kj x_j). The dense
// product runs in two-float arithmetic on the FP32 pipe (Z is exact in FP32,
// x is split into float pairs), so its result is accurate to ~2^-44 of
// |Z| |x| without FP64 arithmetic in the m^2 loop.
constexpr int RES_CHUNK = 1024;
// Zlo (may be null, as for the mHEM fill): the low parts of the entries, which
// are float pairs (hi in Z): their products with x's high parts go into the
// low accumulator, so the residual is that of the float-pair values.
__global__ void __launch_bounds__(128) k_residual_z(const float2* __restrict__ Z, const float2* __restrict__ Zlo,
                                                    const Incidence inc, int m, int n,
                                                    const double2* __restrict__ bvec, const double2* __restrict__ x,
                                                    double2* __restrict__ r, double* __restrict__ norms,
                                                    const int* __restrict__ active) {
    __shared__ float4 xs[RES_CHUNK];        // re_hi, re_lo, im_hi, im_lo
    const int N = n + 2 * m;
    const int blk = blockIdx.y & 1, b = blockIdx.y >> 1;
    if (!active[b]) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const double2* xb = x + (size_t)b * N;
    const float2* Zb = Z + (size_t)b * 2 * m * m + (size_t)blk * m * m;
    const float2* Lb = Zlo ? Zlo + (size_t)b * 2 * m * m + (size_t)blk * m * m : nullptr;
    F2 ar{0.f, 0.f}, ai{0.f, 0.f};
    for (int j0 = 0; j0 < m; j0 += RES_CHUNK) {
        const int nj = min(RES_CHUNK, m - j0);
        __syncthreads();
        for (int t = threadIdx.x; t < nj; t += blockDim.x) {
            double2 v = xb[n + blk * m + j0 + t];
            float rh = (float)v.x, ih = (float)v.y;
            xs[t] = make_float4(rh, (float)(v.x - rh), ih, (float)(v.y - ih));
        }
        __syncthreads();
        if (k < m) {
            const float2* zc = Zb + k + (size_t)m * j0;
            int j = 0;
            if (Lb) {
                const float2* lc = Lb + k + (size_t)m * j0;
                for (; j + 8 <= nj; j += 8) {
                    float2 z[8], l[8];                     // sixteen loads in flight
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        z[q] = zc[(size_t)m * (j + q)];
                        l[q] = lc[(size_t)m * (j + q)];
                    }
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const float4 xv = xs[j + q];
                        ar = f2_mac(ar, z[q].x, xv.x, xv.y);
                        ar = f2_mac(ar, -z[q].y, xv.z, xv.w);
                        ai = f2_mac(ai, z[q].x, xv.z, xv.w);
                        ai = f2_mac(ai, z[q].y, xv.x, xv.y);
                        // low parts (|lo| <= 2^-24 |hi|): FP32 products into the low sums
                        ar.lo = fmaf(l[q].x, xv.x, fmaf(-l[q].y, xv.z, ar.lo));
                        ai.lo = fmaf(l[q].x, xv.z, fmaf(l[q].y, xv.x, ai.lo));
                    }
                }
                for (; j < nj; ++j) {
                    const float2 z = zc[(size_t)m * j], l = lc[(size_t)m * j];
                    const float4 xv = xs[j];
                    ar = f2_mac(ar, z.x, xv.x, xv.y);
                    ar = f2_mac(ar, -z.y, xv.z, xv.w);
                    ai = f2_mac(ai, z.x, xv.z, xv.w);
                    ai = f2_mac(ai, z.y, xv.x, xv.y);
                    ar.lo = fmaf(l.x, xv.x, fmaf(-l.y, xv.z, ar.lo));
                    ai.lo = fmaf(l.x, xv.z, fmaf(l.y, xv.x, ai.lo));
                }
            }
            for (; j + 8 <= nj; j += 8) {
                float2 z[8];                               // eight loads in flight
#pragma unroll
                for (int q = 0; q < 8; ++q) z[q] = zc[(size_t)m * (j + q)];
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 xv = xs[j + q];
                    // (zr + i zi)(xr + i xi) = (zr xr - zi xi) + i (zr xi + zi xr)
                    ar = f2_mac(ar, z[q].x, xv.x, xv.y);
                    ar = f2_mac(ar, -z[q].y, xv.z, xv.w);
                    ai = f2_mac(ai, z[q].x, xv.z, xv.w);
                    ai = f2_mac(ai, z[q].y, xv.x, xv.y);
                }
            }
            for (; j < nj; ++j) {
                const float2 z = zc[(size_t)m * j];
                const float4 xv = xs[j];
                ar = f2_mac(ar, z.x, xv.x, xv.y);
                ar = f2_mac(ar, -z.y, xv.z, xv.w);
                ai = f2_mac(ai, z.x, xv.z, xv.w);
                ai = f2_mac(ai, z.y, xv.x, xv.y);
            }
        }
    }
    if (k >= m) return;
    const int row = n + blk * m + k;
    double2 acc = make_double2(0.0, 0.0);
    for (int q = inc.seg_ptr[k]; q < inc.seg_ptr[k + 1]; ++q) {
        double2 u = xb[inc.seg_node[q]];
        double a = blk == 0 ? (double)inc.seg_a[q] : 0.5;
        acc.x += a * u.x;
        acc.y += a * u.y;
    }
    acc.x -= (double)ar.hi + (double)ar.lo;
    acc.y -= (double)ai.hi + (double)ai.lo;
    double2 rv = csub(bvec[(size_t)b * N + row], acc);
    r[(size_t)b * N + row] = rv;
    atomic_max_nonneg(norms + 4 * b + 2, fabs(rv.x) + fabs(rv.y));
}

__global__ void k_copy_c(const double2* __restrict__ src, double2* __restrict__ dst, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = src[t];
}

__global__ void k_max_rows(const double* __restrict__ rsum, int N, double* __restrict__ norms) {
    int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= N) return;
    atomic_max_nonneg(norms + 4 * b + 3, rsum[(size_t)b * N + i]);
}

// Refinement state of a pass (device): per sample active / converged /
// iterations, previous correction size, max row sum of W, backward error;
// the step counter and the continue flag.
struct IrState {
    int* active;
    int* conv;
    int* iters;
    double* prev_dx;
    double* wnorm;
    double* berr;
    int* step;       // steps done
    int* cont;       // 1 while another step is wanted
    int* extr;       // per sample: the step of its last extrapolation (k_ir_extrap)
    int* nact;       // samples that refine in the coming step
    double* lam;     // per sample: |lambda| of that extrapolation
    double tol;      // stopping tolerance (relative error left in x)
};

// Stopping test after a correction of max-norm dx, |x| = xn (max norm). pdx:
// the previous correction's size (> 0; infinite before the first), or, after
// an extrapolated step, minus the slow mode's |lambda|. The error left after
// this correction is about rho dx for the measured contraction rho = dx / pdx
// (rho <= 1/4), or the mode's tail |lambda| / (1 - |lambda|) dx; stop when four
// times that is below tol |x| (default 1e-9: the residual sees the impedance
// entries as float pairs good to ~1e-13, so what refinement leaves is the
// solution's error against FP64; the inverse Laplace transform amplifies
// sample-to-sample errors by up to e^{c t}; with the fp16-pair factors'
// contraction of ~1e-5, two steps already predict ~4e-10), or when the
// correction itself is below tol / 10 |x|. Step 0 starts from x = 0 (dx_0 = |x_0|), so it never
// stops on the estimate.
TAGS_D bool ir_converged(int step, double dx, double xn, double pdx, double tol) {
    if (dx <= 0.1 * tol * xn) return true;
    if (step >= 1 && pdx > 0.0) {
        const double rho = dx / pdx;
        return rho <= 0.25 && 4.0 * rho * dx <= tol * xn;
    }
    if (pdx < 0.0) {
        const double l = -pdx;
        return 4.0 * l / (1.0 - l) * dx <= tol * xn;
    }
    return false;
}

IrState ir_state(tags_plan_s* p) {
    const int b = p->batch;
    IrState s;
    s.active = p->d_iri;
    s.conv = p->d_iri + b;
    s.iters = p->d_iri + 2 * b;
    s.step = p->d_iri + 3 * b;
    s.cont = p->d_iri + 3 * b + 1;
    s.extr = p->d_iri + 3 * b + 2;
    s.nact = p->d_iri + 4 * b + 2;
    s.prev_dx = p->d_ird;
    s.wnorm = p->d_ird + b;
    s.berr = p->d_ird + 2 * b;
    s.lam = p->d_ird + 3 * b;
    s.tol = p->ir_tol;
    return s;
}

// Extrapolation against one slow mode. At low frequencies the scaled system
// keeps a mode (the grid's common potential) that the FP32 factors reproduce
// poorly, and the corrections then shrink by a nearly constant complex factor:
// y_k ~ lambda y_{k-1} (measured: cosine^2 = 1.000 between successive
// corrections, |lambda| from 0.02 to 0.5). When the last two corrections are
// that close to parallel (cosine >= 0.9, 0.01 <= |lambda| <= 0.95) and the
// sample is not stopping at this step anyway, the error left in x is about
// lambda / (1 - lambda) times the last correction, which is added (Aitken's
// step, one vector). Never on two steps running (the correction after an
// extrapolated step says nothing about lambda), and from the third step on.
// The residual that follows is computed from scratch, so a poor estimate costs
// a step, not accuracy. Same grid as k_ir_update.
__global__ void k_ir_extrap(const float2* __restrict__ y, const double* __restrict__ scale, int m, int n,
                            double2* __restrict__ x, const double* __restrict__ norms, const double* __restrict__ dots,
                            IrState s) {
    const int N = n + 2 * m;
    const int ip = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (!s.active[b]) return;
    const int step = *s.step;
    if (step < 2 || s.extr[b] == step - 1) return;
    if (ir_converged(step, norms[4 * b + 0], norms[4 * b + 1], s.prev_dx[b], s.tol)) return;
    const double re = dots[4 * b], im = dots[4 * b + 1], pp = dots[4 * b + 2], yy = dots[4 * b + 3];
    if (!(pp > 0.0) || !(yy > 0.0) || re * re + im * im < 0.81 * pp * yy) return;
    const double lr = re / pp, li = im / pp, l2 = lr * lr + li * li;
    if (!(l2 >= 1e-4 && l2 <= 0.9025)) return;
    const double dr = 1.0 - lr, di = -li, dd = dr * dr + di * di;
    const double gr = (lr * dr + li * di) / dd, gi = (li * dr - lr * di) / dd;      // lambda / (1 - lambda)
    if (ip == 0) {
        s.extr[b] = step;
        s.lam[b] = sqrt(l2);
    }
    if (ip >= N) return;
    const double sc = scale[(size_t)b * N + ip];
    const float2 yv = y[(size_t)b * N + ip];
    const double dxr = (double)yv.x * sc, dxi = (double)yv.y * sc;
    const size_t o = (size_t)b * N + orig_of(ip, m, n);
    double2 xv = x[o];
    xv.x += gr * dxr - gi * dxi;
    xv.y += gr * dxi + gi * dxr;
    x[o] = xv;
}

// A sample refines unless its static-order factorisation hit a zero pivot
// or a tensor-core wait ran out (FP64 fallback), or an fp16 split value left
// its range (the pass is factorised again with bf16 pieces).
__global__ void k_ir_init(const double* __restrict__ norms, const int* __restrict__ info,
                          const int* __restrict__ tc_err, int nb, IrState s) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q == 0) {
        *s.step = 0;
        *s.cont = 1;
        *s.nact = nb;
    }
    if (q >= nb) return;
    s.active[q] = info[q] == 0 && tc_err[0] == 0 && tc_err[1] == 0;
    s.conv[q] = 0;
    s.iters[q] = 0;
    s.prev_dx[q] = INFINITY;
    s.wnorm[q] = norms[4 * q + 3];
    s.berr[q] = 0.0;
    s.extr[q] = -10;
}

// After a step's correction, before its residual: per sample, stop on
// ir_converged (the correction times the measured contraction predicts an
// error under the tolerance), or once the corrections stop shrinking
// (accepted when the backward error is below 1e-12); NaN goes to the
// fallback. Samples that stop here skip the residual of their final iterate:
// the backward error kept is that of the iterate before the final correction
// (norms[2] / (|W| norms[3]), formed by the previous step's residual), which
// the correction then shrinks by about the measured contraction. For samples
// that go on, norms[2] is cleared for this step's residual and norms[3] takes
// |x|. One CTA. Sets the continue flag and, inside a graph, the while-node
// condition.
__global__ void __launch_bounds__(1024) k_ir_decide(double* __restrict__ norms, int nb, int max_steps, IrState s,
                                                    cudaGraphConditionalHandle cond, int set_cond) {
    __shared__ int going;
    const int step = *s.step;
    if (threadIdx.x == 0) going = 0;
    __syncthreads();
    for (int q = threadIdx.x; q < nb; q += blockDim.x) {
        if (!s.active[q]) continue;
        s.iters[q] = step + 1;
        const double dx = norms[4 * q + 0], xn = norms[4 * q + 1];
        // step 0 starts from x = 0: no residual of an earlier iterate yet
        const double be = step >= 1 ? norms[4 * q + 2] / (s.wnorm[q] * norms[4 * q + 3] + 1e-300) : 0.0;
        s.berr[q] = be;
        if (!(dx == dx) || !(xn == xn)) { s.active[q] = 0; continue; }
        bool more = true;
        if (s.extr[q] == step) {
            // extrapolated in this step: x moved by more than dx; the next
            // step measures its error against the mode's contraction
            s.prev_dx[q] = -s.lam[q];
        } else {
            const double pdx = s.prev_dx[q];
            if (ir_converged(step, dx, xn, pdx, s.tol)) {
                s.active[q] = 0;
                s.conv[q] = 1;
                more = false;
            } else if (step >= 2 && pdx > 0.0 && dx > 0.5 * pdx) {
                s.conv[q] = be <= 1e-12;
                s.active[q] = 0;
                more = false;
            } else {
                s.prev_dx[q] = dx;
            }
        }
        if (more) {
            norms[4 * q + 2] = 0.0;
            norms[4 * q + 3] = xn;
            atomicAdd(&going, 1);
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int c = going > 0 && step + 1 < max_steps;
        *s.step = step + 1;
        *s.cont = c;
        *s.nact = going;
        if (set_cond) cudaGraphSetConditional(cond, c ? 1u : 0u);
    }
}

}  // namespace

int tags_mixed_alloc(tags_plan_s* p) {
    const size_t b = p->batch, N = p->N, m = p->m;
    TAGS_CUDA_OK(cudaMalloc(&p->d_fillws, tags_mixed_fill_workspace(p->m)));
    int err = tags_launch_pair_plan(p->d_elec, p->d_img, p->m, p->has_images, p->d_fillws, p->stream);
    if (err) return err;
    err = tags_mixed_touch_count(p->d_fillws, p->m, p->stream, &p->n_touch);
    if (err) return err;
    err = tags_mixed_special_build(p->d_fillws, p->m, (int)b, &p->spec, p->stream);
    if (err) return err;
    {
        double lmax = 0.0;
        for (int e = 0; e < p->m; ++e) lmax = std::max(lmax, p->h_elec[11 * (size_t)e + 9]);
        err = tags_mixed_special_moments(p->d_elec, p->d_img, p->m, lmax, &p->spec, p->stream);
        if (err) return err;
    }
    err = tags_moment_fill_build(p->d_elec, p->has_images ? p->d_img : p->d_elec, p->m, p->has_images,
                                 p->h_elec.data(), p->has_images ? p->h_img.data() : p->h_elec.data(), (int)b, &p->mom,
                                 p->stream);
    if (err) return err;
    TAGS_CUDA_OK(cudaMalloc(&p->d_Zlo, sizeof(float2) * 2 * m * m * b));
    TAGS_CUDA_OK(cudaMemset(p->d_Zlo, 0, sizeof(float2) * 2 * m * m * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_Z, sizeof(float2) * 2 * m * m * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_rowpart, sizeof(float) * 2 * 2 * b * ((m + 31) / 32) * m));
    TAGS_CUDA_OK(cudaMalloc(&p->d_A, sizeof(float2) * N * N * b));
    // scale + row sums (FP64), then an FP32 copy of the scale
    TAGS_CUDA_OK(cudaMalloc(&p->d_scale, sizeof(double) * 2 * N * b + sizeof(float) * N * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_r, sizeof(double2) * 2 * N * b));      // residual + right-hand side
    TAGS_CUDA_OK(cudaMalloc(&p->d_rf, sizeof(float2) * N * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_norms, sizeof(double) * 4 * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_iri, sizeof(int) * (4 * b + 3)));
    TAGS_CUDA_OK(cudaMalloc(&p->d_yprev, sizeof(float2) * N * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_dots, sizeof(double) * 4 * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_ird, sizeof(double) * 4 * b));
    const size_t ws = tags_ldl_tc_workspace((int)N, (int)b);
    TAGS_CUDA_OK(cudaMalloc(&p->d_ldlws, ws));
    TAGS_CUDA_OK(cudaMemset(p->d_ldlws, 0, ws));
    TAGS_CUDA_OK(cudaMalloc(&p->d_ldlerr, 2 * sizeof(int)));     // [0] wait ran out, [1] fp16 range
    TAGS_CUDA_OK(cudaMemset(p->d_ldlerr, 0, 2 * sizeof(int)));
    // one-time kernel attributes and driver entry points, outside any capture
    return tags_ldl_tc_prepare();
}

int tags_mixed_free(tags_plan_s* p) {
    void* ptrs[] = {p->d_Z,      p->d_A,      p->d_scale, p->d_r,      p->d_rf,  p->d_norms,   p->d_fillws,
                    p->d_ldlws, p->d_ldlerr, p->d_iri,  p->d_ird, p->d_yprev, p->d_dots, p->d_rowpart};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    tags_mixed_special_free(&p->spec);
    tags_moment_fill_free(&p->mom);
    if (p->d_Zlo) cudaFree(p->d_Zlo);
    p->d_Zlo = nullptr;
    p->d_Z = nullptr;
    p->d_A = nullptr;
    p->d_yprev = nullptr;
    p->d_dots = nullptr;
    p->d_rowpart = nullptr;
    return 0;
}

// Re-solve sample `q` of the current pass in plain FP64 (partial pivoting).
static int fallback_plain(tags_plan_s* p, int q, cudaStream_t st) {
    TagsRange range("tags FP64 re-solve");
    const long long N = p->N, NN = N * N;
    if (!p->d_fbW) {
        if (cudaMalloc(&p->d_fbW, sizeof(double2) * NN) != cudaSuccess ||
            cudaMalloc(&p->d_fbpiv, sizeof(int) * (N + 1)) != cudaSuccess) {
            cudaGetLastError();
            if (p->d_fbW) cudaFree(p->d_fbW);
            p->d_fbW = nullptr;
            return tags_fail(TAGS_E_NOMEM, "device allocation failed (FP64 fallback)");
        }
    }
    double2* W = p->d_fbW;
    int* ipiv = p->d_fbpiv;
    TAGS_CUDA_OK(cudaMemsetAsync(W, 0, sizeof(double2) * NN, st));
    int err = tags_wg_incidence(W, N, NN, 1, p->d_cond, p->n, p->m, st);
    if (err) return err;
    FillOut out{};
    out.zl = W;
    out.zt = W;
    out.ld = N;
    out.row0_l = out.col0_l = p->n;
    out.row0_t = out.col0_t = p->n + p->m;
    out.sign = -1.0;
    out.mirror = 1;
    err = tags_plan_fill_fp64(p, p->d_coef + q, 1, out, st);
    if (err) return err;
    err = tags_lu_z(W, (int)N, N, NN, 1, 1, ipiv, p->d_info + q, st);
    if (err) return err;
    double2* x = p->d_x + (size_t)q * N;
    const double2* bvec = p->d_r + (size_t)p->batch * N + (size_t)q * N;
    TAGS_CUDA_OK(cudaMemcpyAsync(x, bvec, sizeof(double2) * N, cudaMemcpyDeviceToDevice, st));
    return tags_lu_solve_z(W, (int)N, N, NN, 1, ipiv, x, 1, N, N, st);
}

int tags_plan_rhs(tags_plan_s* p, double2* d_X, const double2* d_ie, int inj_node, int nb, cudaStream_t st);
int tags_plan_coef(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur, int nb, cudaStream_t st);

int tags_mixed_fallback_one(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur,
                            const double2* d_ie, int inj_node, double2* x_out, int* info_out, cudaStream_t st) {
    int err = tags_plan_coef(p, d_s, d_kappa, mur, 1, st);          // coefficients in slot 0
    double2* b0 = p->d_r + (size_t)p->batch * p->N;                    // saved right-hand side, slot 0
    if (!err) err = tags_plan_rhs(p, b0, d_ie, inj_node, 1, st);
    if (!err) err = fallback_plain(p, 0, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaMemcpyAsync(x_out, p->d_x, sizeof(double2) * p->N, cudaMemcpyDeviceToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(info_out, p->d_info, sizeof(int), cudaMemcpyDeviceToDevice, st));
    return 0;
}

// ---- one pass of nb samples, in four stages -------------------------------------
// The right-hand side b is in d_x when a pass starts (written by the plan).

static constexpr int kMaxSteps = 40;      // upper bound of tags_plan_s::max_steps

// b saved, x = 0, impedance fill, scaling, FP32 working matrix, its LDL^T
int tags_mixed_factor(tags_plan_s* p, int nb, cudaStream_t st) {
    const int m = p->m, n = p->n, N = p->N;
    const size_t NN = (size_t)N * N;
    double* d_rsum = p->d_scale + (size_t)p->batch * N;
    double2* d_b = p->d_r + (size_t)p->batch * N;
    k_copy_c<<<(unsigned)(((long long)nb * N + 255) / 256), 256, 0, st>>>(p->d_x, d_b, (long long)nb * N);
    tags_note_launch();
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_x, 0, sizeof(double2) * N * nb, st));
    // 1. impedance blocks (full symmetric, complex FP32), direct + images: double
    //    line integrals, or the mHEM rescale of the static potentials
    TagsRange range("tags fill");
    int err = p->fill_model == TAGS_INTG_MHEM
                  ? tags_launch_mhem_mixed(m, p->has_images, p->d_pot, p->d_fillws, p->d_coef, nb, p->d_Z,
                                           p->d_Z + (size_t)m * m, 2LL * m * m, p->d_status, st)
                  : tags_launch_fill_mixed(p->d_elec, p->d_img, m, p->d_fillws, p->d_coef, nb, p->d_Z,
                                           p->d_Z + (size_t)m * m, p->d_Zlo, p->d_Zlo + (size_t)m * m, 2LL * m * m,
                                           p->has_images, p->spec, p->mom, p->d_status, st, p->d_rowpart);
    if (err) return err;
    range.next("tags assemble");
    // 2. scaling
    float* d_scalef = reinterpret_cast<float*>(p->d_scale + 2 * (size_t)p->batch * N);
    if (p->fill_model == TAGS_INTG_MHEM)
        k_rowstats<<<dim3((m * 32 + 255) / 256, 2, nb), 256, 0, st>>>(p->d_Z, m, p->d_scale, d_rsum, d_scalef, N);
    else       // from the partials of the fill's mirror pass
        k_rowstats_part<<<dim3((m + 255) / 256, 2, nb), 256, 0, st>>>(
            p->d_rowpart, p->d_rowpart + (size_t)2 * nb * ((m + 31) / 32) * m, m, p->d_scale, d_rsum, d_scalef, N);
    k_rowstats_nodes<<<dim3((n + 127) / 128, nb), 128, 0, st>>>(p->inc.node_ptr, n, m, p->d_scale, d_rsum, d_scalef,
                                                                N);
    tags_note_launch(2);
    // 3. FP32 working matrix and its LDL^T (no pivoting)
    int pf = tags_prof_begin(TAGS_PROF_BUILD, st);
    k_build<<<dim3((unsigned)((N + BUILD_COLS - 1) / BUILD_COLS), nb), 256, 0, st>>>(p->d_Z, p->inc, d_scalef, m, n,
                                                                                  p->d_A);
    tags_prof_end(TAGS_PROF_BUILD, pf, st, 0.0, (8.0 * 0.5 * N * (N + 1.0) + 32.0 * m * m) * nb);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    range.next("tags factor");
    return tags_ldl_tc(p->d_A, N, N, (long long)NN, nb, p->batch, p->d_ldlws, p->d_info, p->d_ldlerr, m,
                       p->split_pieces, p->group_panels, st, p->tc_pairs);
}

// r = b, max row sum of W per sample, refinement state
int tags_mixed_ir_setup(tags_plan_s* p, int nb, cudaStream_t st) {
    TagsRange range("tags refine setup");
    const int N = p->N;
    double* d_rsum = p->d_scale + (size_t)p->batch * N;
    double2* d_b = p->d_r + (size_t)p->batch * N;
    k_copy_c<<<(unsigned)(((long long)nb * N + 255) / 256), 256, 0, st>>>(d_b, p->d_r, (long long)nb * N);
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_norms, 0, sizeof(double) * 4 * nb, st));
    k_max_rows<<<dim3((N + 255) / 256, nb), 256, 0, st>>>(d_rsum, N, p->d_norms);
    k_ir_init<<<(nb + 255) / 256, 256, 0, st>>>(p->d_norms, p->d_info, p->d_ldlerr, nb, ir_state(p));
    tags_note_launch(3);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// One refinement step: correction from the factors, x update, stopping
// decision, residual of the new iterate for the samples that go on. A fixed
// launch sequence (graph-capturable).
int tags_mixed_ir_step(tags_plan_s* p, int nb, cudaStream_t st, cudaGraphConditionalHandle cond, int set_cond) {
    TagsRange range("tags refine step");
    const int m = p->m, n = p->n, N = p->N;
    const size_t NN = (size_t)N * N;
    double2* d_b = p->d_r + (size_t)p->batch * N;
    const IrState s = ir_state(p);
    dim3 gv((N + 255) / 256, nb);
    k_ir_rhs<<<gv, 256, 0, st>>>(p->d_r, p->d_scale, m, n, p->d_rf, p->d_norms, p->d_dots);
    tags_note_launch();
    // samples that stopped refining skip the sweeps (their x is left alone);
    // the first step's right-hand side is b, zero in the 2m impedance rows
    // that the order ZL, ZT, nodes puts first
    int err = tags_ldl_solve_c(p->d_A, N, N, (long long)NN, nb, p->batch, p->d_ldlws, p->d_rf, N, m, st, s.active,
                               s.step, 2 * m, s.nact);
    if (err) return err;
    k_ir_update<<<gv, 256, 0, st>>>(p->d_rf, p->d_scale, m, n, p->d_x, p->d_norms, s.active, p->d_yprev, p->d_dots,
                                    s.step);
    k_ir_extrap<<<gv, 256, 0, st>>>(p->d_rf, p->d_scale, m, n, p->d_x, p->d_norms, p->d_dots, s);
    k_ir_decide<<<1, 1024, 0, st>>>(p->d_norms, nb, std::min(p->max_steps, kMaxSteps), s, cond, set_cond);
    int pf = tags_prof_begin(TAGS_PROF_RESID, st);
    k_residual_nodes<<<dim3((n + 255) / 256, nb), 256, 0, st>>>(p->inc, m, n, d_b, p->d_x, p->d_r, p->d_norms,
                                                                s.active);
    const float2* zlo = p->fill_model == TAGS_INTG_MHEM ? nullptr : p->d_Zlo;
    k_residual_z<<<dim3((m + 127) / 128, 2 * nb), 128, 0, st>>>(p->d_Z, zlo, p->inc, m, n, d_b, p->d_x, p->d_r,
                                                                p->d_norms, s.active);
    // 2 m^2 complex products (4 real multiply-adds each) and a read of Z in FP32
    tags_prof_end(TAGS_PROF_RESID, pf, st, 16.0 * m * (double)m * nb, 16.0 * m * (double)m * nb);
    tags_note_launch(5);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// Read the refinement state back, re-solve what did not converge in FP64.
int tags_mixed_finish(tags_plan_s* p, int nb, cudaStream_t st, int* h_iters, double* h_berr, int* h_conv,
                      int* h_steps) {
    const int b = p->batch;
    std::vector<int> iri(3 * b + 2);
    std::vector<double> ird(3 * b);
    int tc_errs[2] = {0, 0};
    int status = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(iri.data(), p->d_iri, sizeof(int) * (3 * b + 2), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(ird.data(), p->d_ird, sizeof(double) * 3 * b, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(tc_errs, p->d_ldlerr, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(&status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (status & TAGS_ST_NONFINITE) {
        // a non-finite input reached the fill (the run reports it): no
        // re-solve in FP64, and no switch to bf16 pieces over a NaN that only
        // looks like a value outside the fp16 range
        TAGS_CUDA_OK(cudaMemsetAsync(p->d_ldlerr, 0, 2 * sizeof(int), st));
        if (h_steps) *h_steps = iri[3 * b];
        for (int q = 0; q < nb; ++q) {
            h_iters[q] = iri[2 * b + q];
            h_conv[q] = iri[b + q];
            h_berr[q] = ird[2 * b + q];
        }
        return 0;
    }
    if (tc_errs[1] && !tc_errs[0]) {
        // an fp16 split value left its range: this plan uses three bf16
        // pieces from now on (its graphs are recaptured), and the pass is
        // solved again from its right-hand side
        TAGS_CUDA_OK(cudaMemsetAsync(p->d_ldlerr, 0, 2 * sizeof(int), st));
        p->split_pieces = 3;
        tags_plan_drop_graphs(p);
        const double2* d_b = p->d_r + (size_t)p->batch * p->N;
        TAGS_CUDA_OK(cudaMemcpyAsync(p->d_x, d_b, sizeof(double2) * p->N * nb, cudaMemcpyDeviceToDevice, st));
        int err = tags_mixed_solve_batch(p, nb, nullptr, h_iters, h_berr, h_conv, st);
        if (h_steps) *h_steps = 0;
        return err;
    }
    const int tc_err = tc_errs[0];
    if (tc_err) {
        // a tensor-core wait ran out: the pass went to the FP64 path
        tags_fail(TAGS_E_CUDA, "tensor-core factorisation reported a timeout; samples re-solved in FP64");
        TAGS_CUDA_OK(cudaMemsetAsync(p->d_ldlerr, 0, 2 * sizeof(int), st));
    }
    if (h_steps) *h_steps = iri[3 * b];
    for (int q = 0; q < nb; ++q) {
        h_iters[q] = iri[2 * b + q];
        h_conv[q] = iri[b + q];
        h_berr[q] = ird[2 * b + q];
        if (!h_conv[q]) {
            int err = fallback_plain(p, q, st);
            if (err) return err;
        }
    }
    // converged samples report success; fallbacks keep their own LU info
    for (int q = 0; q < nb; ++q)
        if (h_conv[q]) TAGS_CUDA_OK(cudaMemsetAsync(p->d_info + q, 0, sizeof(int), st));
    return 0;
}

int tags_plan_coef(tags_plan_s* p, const double2* d_s, const double2* d_kappa, double mur, int nb, cudaStream_t st);

// Diagnostic: the mixed fill of ns <= batch samples, returned as the values the
// refinement's residual uses (FP32 entries, FP64 hi + lo on the special ones).
extern "C" int tags_debug_mixed_fill(tags_plan plan, const tags_cdouble* s, const tags_cdouble* kappa, double mur,
                                     size_t ns, tags_cdouble* zl, tags_cdouble* zt) {
    tags_plan_s* p = plan;
    if (!p || p->precision == TAGS_PLAIN_FP64 || !s || !kappa || !zl || !zt || ns == 0 || (int)ns > p->batch)
        return tags_fail(TAGS_E_ARG, "tags_debug_mixed_fill: invalid argument (mixed plan, 1 <= ns <= batch)");
    if (p->fill_model != TAGS_INTG_DOUBLE) return tags_fail(TAGS_E_ARG, "tags_debug_mixed_fill: INTG_DOUBLE fill only");
    const int m = p->m, nb = (int)ns;
    cudaStream_t st = p->stream;
    TAGS_CUDA_OK(cudaMemcpyAsync(p->d_sin, s, sizeof(double2) * nb, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(p->d_sin + p->batch, kappa, sizeof(double2) * nb, cudaMemcpyHostToDevice, st));
    int err = tags_plan_coef(p, p->d_sin, p->d_sin + p->batch, mur, nb, st);
    if (!err)
        err = tags_launch_fill_mixed(p->d_elec, p->d_img, m, p->d_fillws, p->d_coef, nb, p->d_Z, p->d_Z + (size_t)m * m,
                                     p->d_Zlo, p->d_Zlo + (size_t)m * m, 2LL * m * m, p->has_images, p->spec, p->mom,
                                     p->d_status, st);
    if (err) return err;
    const size_t mm = (size_t)m * m;
    std::vector<float2> z(2 * mm * nb), lo(2 * mm * nb);
    TAGS_CUDA_OK(cudaMemcpyAsync(z.data(), p->d_Z, sizeof(float2) * z.size(), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(lo.data(), p->d_Zlo, sizeof(float2) * lo.size(), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    double* ol = reinterpret_cast<double*>(zl);
    double* ot = reinterpret_cast<double*>(zt);
    for (int b = 0; b < nb; ++b)
        for (size_t e = 0; e < mm; ++e) {
            const size_t a = (size_t)b * 2 * mm + e, c = a + mm, o = (size_t)b * mm + e;
            ol[2 * o] = (double)z[a].x + (double)lo[a].x;
            ol[2 * o + 1] = (double)z[a].y + (double)lo[a].y;
            ot[2 * o] = (double)z[c].x + (double)lo[c].x;
            ot[2 * o + 1] = (double)z[c].y + (double)lo[c].y;
        }
    return 0;
}

// The pass without a graph: the host follows the device's continue flag.
int tags_mixed_solve_batch(tags_plan_s* p, int nb, const double2*, int* h_iters, double* h_berr, int* h_conv,
                           cudaStream_t st) {
    int err = tags_mixed_factor(p, nb, st);
    if (!err) err = tags_mixed_ir_setup(p, nb, st);
    if (err) return err;
    cudaGraphConditionalHandle none = 0;
    for (int step = 0; step < std::min(p->max_steps, kMaxSteps); ++step) {
        err = tags_mixed_ir_step(p, nb, st, none, 0);
        if (err) return err;
        int cont = 0;
        TAGS_CUDA_OK(cudaMemcpyAsync(&cont, p->d_iri + 3 * p->batch + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
        if (!cont) break;
    }
    return tags_mixed_finish(p, nb, st, h_iters, h_berr, h_conv, nullptr);
}
