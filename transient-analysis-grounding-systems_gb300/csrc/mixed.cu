// Mixed-precision batched solve of the immittance system.
//
// Same system as the reference's solve_immittance (src/linalg.c:112-139):
//     W_G = [ 0   A^T  B^T ]      x = [U; I_L; I_T],  b = [I_E; 0; 0]
//           [ A  -ZL   0   ]
//           [ B   0   -ZT  ]
// solved here as follows:
//   0. impedance blocks: regular pairs in FP32 (anchors from two-float
//      products), pairs sharing an endpoint (log-singular) in FP64, the
//      diagonal in its closed form; stored as complex FP32, which is the
//      matrix the refinement solves (its entries carry the fill's ~1e-7 error);
//   1. static symmetric ordering P: ZL rows, ZT rows, then node rows, so that
//      the elimination meets the impedance blocks (large diagonals) before the
//      zero Y_E block and needs no pivot search;
//   2. symmetric scaling D = diag(1/sqrt(max_j |W'_ij|)), W'' = D P W P^T D;
//   3. LDL^T of W'' without pivoting, complex FP32 storage, trailing updates
//      and triangular-solve panels on the tensor cores (ldl_tc.cu);
//   4. iterative refinement in FP64: r = b - W x is evaluated in FP64 from the
//      FP64 impedance blocks and the exact incidence (sparse, +-1 / 0.5), the
//      correction from the FP32 factors, until the correction is below
//      4 eps |x| or stops shrinking;
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
                           int N) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    int blk = blockIdx.y;       // 0 = ZL, 1 = ZT
    int b = blockIdx.z;
    if (warp >= m) return;
    const float2* col = Z + (size_t)b * 2 * m * m + (size_t)blk * m * m + (size_t)m * warp;
    double mx = 0.0, sm = 0.0;
    for (int j = lane; j < m; j += 32) {
        float2 z = col[j];
        double a = sqrtf(z.x * z.x + z.y * z.y);
        mx = fmax(mx, a);
        sm += a;
    }
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        sm += __shfl_down_sync(0xffffffffu, sm, o);
    }
    if (lane == 0) {
        double inc = blk == 0 ? 1.0 : 0.5;            // incidence entries of the row
        int row = blk * m + warp;                      // reordered index
        scale[(size_t)b * N + row] = 1.0 / sqrt(fmax(mx, inc));
        rsum[(size_t)b * N + row] = sm + 2.0 * inc;
    }
}

// Node rows: max |entry| = 1 (A) so the scale is 1; row sum = sum over
// incident segments of (1 + 0.5).
__global__ void k_rowstats_nodes(const int* __restrict__ node_ptr, int n, int m, double* __restrict__ scale,
                                 double* __restrict__ rsum, int N) {
    int nd = blockIdx.x * blockDim.x + threadIdx.x;
    int b = blockIdx.y;
    if (nd >= n) return;
    scale[(size_t)b * N + 2 * m + nd] = 1.0;
    rsum[(size_t)b * N + 2 * m + nd] = 1.5 * (double)(node_ptr[nd + 1] - node_ptr[nd]);
}

// W'' (complex FP32, column-major N x N, reordered and scaled), lower triangle.
// Grid: x over 256-row chunks, y over columns, z over samples.
__global__ void __launch_bounds__(256) k_build(const float2* __restrict__ Z, const signed char* __restrict__ cond,
                                               const double* __restrict__ scale, int m, int n,
                                               float2* __restrict__ A) {
    const int N = n + 2 * m;
    const int j = blockIdx.y, b = blockIdx.z;
    const int i = j + blockIdx.x * blockDim.x + threadIdx.x;     // rows i >= j only
    if (i >= N) return;
    const double* d = scale + (size_t)b * N;
    const float2* Zb = Z + (size_t)b * 2 * m * m;
    float vx = 0.f, vy = 0.f;
    const int bi = i < m ? 0 : (i < 2 * m ? 1 : 2);
    const int bj = j < m ? 0 : (j < 2 * m ? 1 : 2);
    if (bi < 2 && bj == bi) {
        const float2 z = Zb[(size_t)bi * m * m + (i - bi * m) + (size_t)m * (j - bj * m)];
        vx = -z.x;
        vy = -z.y;
    } else if (bi == 2 && bj < 2) {
        const int c = cond[(size_t)(i - 2 * m) * m + (j - bj * m)];
        if (c) vx = bj == 0 ? (c == 1 ? 1.f : -1.f) : 0.5f;
    }
    const float s = (float)(d[i] * d[j]);
    A[(size_t)b * N * N + (size_t)j * N + i] = make_float2(vx * s, vy * s);
}

TAGS_D int orig_of(int ip, int m, int n) {
    // reordered index -> original W_G index
    return ip < 2 * m ? n + ip : ip - 2 * m;
}

// rf = D P r (FP32)
__global__ void k_ir_rhs(const double2* __restrict__ r, const double* __restrict__ scale, int m, int n,
                         float2* __restrict__ rf) {
    const int N = n + 2 * m;
    int ip = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (ip >= N) return;
    double2 v = r[(size_t)b * N + orig_of(ip, m, n)];
    double s = scale[(size_t)b * N + ip];
    rf[(size_t)b * N + ip] = make_float2((float)(v.x * s), (float)(v.y * s));
}

// x += P^T D y (FP64); norms[b*4 + 0] = max|dx|, [1] = max|x|
__global__ void k_ir_update(const float2* __restrict__ y, const double* __restrict__ scale, int m, int n,
                            double2* __restrict__ x, double* __restrict__ norms, const int* __restrict__ active) {
    const int N = n + 2 * m;
    int ip = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (ip >= N || !active[b]) return;
    double s = scale[(size_t)b * N + ip];
    float2 yv = y[(size_t)b * N + ip];
    double2 dx = make_double2((double)yv.x * s, (double)yv.y * s);
    size_t o = (size_t)b * N + orig_of(ip, m, n);
    double2 xv = cadd(x[o], dx);
    x[o] = xv;
    atomic_max_nonneg(norms + 4 * b + 0, fabs(dx.x) + fabs(dx.y));
    atomic_max_nonneg(norms + 4 * b + 1, fabs(xv.x) + fabs(xv.y));
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

// Two-float helpers: a value is hi + lo with |lo| <= ulp(hi)/2 (~2^-48 relative).
struct F2 {
    float hi, lo;
};
TAGS_D F2 f2_add(F2 a, float p, float e) {
    // a + (p + e), p the leading part of a product, e its rounding error
    float s = a.hi + p;
    float v = s - a.hi;
    float t = (a.hi - (s - v)) + (p - v);
    t += a.lo + e;
    F2 o;
    o.hi = s + t;
    o.lo = t - (o.hi - s);
    return o;
}
// a += z * (xh + xl) for real z (exact in FP32) and a two-float x
TAGS_D F2 f2_mac(F2 a, float z, float xh, float xl) {
    float p = z * xh;
    float e = fmaf(z, xh, -p);
    e = fmaf(z, xl, e);
    return f2_add(a, p, e);
}

// Impedance rows: r_k = b_k - (incidence terms - sum_j Z_kj x_j). The dense
// product runs in two-float arithmetic on the FP32 pipe (Z is exact in FP32,
// x is split into float pairs), so its result is accurate to ~2^-44 of
// |Z| |x| without FP64 arithmetic in the m^2 loop.
constexpr int RES_CHUNK = 1024;
__global__ void __launch_bounds__(256) k_residual_z(const float2* __restrict__ Z, const Incidence inc, int m, int n,
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
            for (int j = 0; j < nj; ++j) {
                const float2 z = Zb[k + (size_t)m * (j0 + j)];
                const float4 xv = xs[j];
                // (zr + i zi)(xr + i xi) = (zr xr - zi xi) + i (zr xi + zi xr)
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

}  // namespace

int tags_mixed_alloc(tags_plan_s* p) {
    const size_t b = p->batch, N = p->N, m = p->m;
    TAGS_CUDA_OK(cudaMalloc(&p->d_fillws, tags_mixed_fill_workspace(p->m)));
    int err = tags_launch_pair_plan(p->d_elec, p->d_img, p->m, p->has_images, p->d_fillws, p->stream);
    if (err) return err;
    err = tags_mixed_touch_count(p->d_fillws, p->m, p->stream, &p->n_touch);
    if (err) return err;
    TAGS_CUDA_OK(cudaMalloc(&p->d_Z, sizeof(float2) * 2 * m * m * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_A, sizeof(float2) * N * N * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_scale, sizeof(double) * 2 * N * b));   // scale + row sums
    TAGS_CUDA_OK(cudaMalloc(&p->d_r, sizeof(double2) * 2 * N * b));      // residual + right-hand side
    TAGS_CUDA_OK(cudaMalloc(&p->d_rf, sizeof(float2) * N * b));
    TAGS_CUDA_OK(cudaMalloc(&p->d_norms, sizeof(double) * 4 * b + sizeof(int) * b));
    const size_t ws = tags_ldl_tc_workspace((int)N, (int)b);
    TAGS_CUDA_OK(cudaMalloc(&p->d_ldlws, ws));
    TAGS_CUDA_OK(cudaMemset(p->d_ldlws, 0, ws));
    TAGS_CUDA_OK(cudaMalloc(&p->d_ldlerr, sizeof(int)));
    TAGS_CUDA_OK(cudaMemset(p->d_ldlerr, 0, sizeof(int)));
    return 0;
}

int tags_mixed_free(tags_plan_s* p) {
    void* ptrs[] = {p->d_Z, p->d_A, p->d_scale, p->d_r, p->d_rf, p->d_norms, p->d_fillws, p->d_ldlws, p->d_ldlerr};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    p->d_Z = nullptr;
    p->d_A = nullptr;
    return 0;
}

// Re-solve sample `q` of the current pass in plain FP64 (partial pivoting).
static int fallback_plain(tags_plan_s* p, int q, cudaStream_t st) {
    DeviceCtx* c = tags_ctx();
    const long long N = p->N, NN = N * N;
    double2* W = (double2*)c->scratch(10, sizeof(double2) * NN);
    int* ipiv = (int*)c->scratch(11, sizeof(int) * (N + 1));
    if (!W || !ipiv) return tags_fail(TAGS_E_NOMEM, "device allocation failed (fallback)");
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
    err = tags_launch_fill_fp64(p->d_elec, p->d_img, p->m, p->d_coef + q, 1, out,
                                p->has_images ? TAGS_FILL_BOTH : TAGS_FILL_DIRECT, TAGS_INTG_DOUBLE, 1, p->d_status, st);
    if (err) return err;
    err = tags_lu_z(W, (int)N, N, NN, 1, 1, ipiv, p->d_info + q, st);
    if (err) return err;
    double2* x = p->d_x + (size_t)q * N;
    const double2* bvec = p->d_r + (size_t)p->batch * N + (size_t)q * N;
    TAGS_CUDA_OK(cudaMemcpyAsync(x, bvec, sizeof(double2) * N, cudaMemcpyDeviceToDevice, st));
    return tags_lu_solve_z(W, (int)N, N, NN, 1, ipiv, x, 1, N, N, st);
}

int tags_mixed_solve_batch(tags_plan_s* p, int nb, const double2*, int* h_iters, double* h_berr, int* h_conv,
                           cudaStream_t st) {
    const int m = p->m, n = p->n, N = p->N;
    const size_t NN = (size_t)N * N;
    double* d_rsum = p->d_scale + (size_t)p->batch * N;
    double2* d_b = p->d_r + (size_t)p->batch * N;
    int* d_active = reinterpret_cast<int*>(p->d_norms + 4 * p->batch);
    // right-hand side b (written by the plan into d_x), then x = 0
    k_copy_c<<<(unsigned)(((long long)nb * N + 255) / 256), 256, 0, st>>>(p->d_x, d_b, (long long)nb * N);
    tags_note_launch();
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_x, 0, sizeof(double2) * N * nb, st));
    // 1. impedance blocks (full symmetric, complex FP32), direct + images
    int err = tags_launch_fill_mixed(p->d_elec, p->d_img, m, p->d_fillws, p->d_coef, nb, p->d_Z, p->d_Z + (size_t)m * m,
                                     2LL * m * m, p->has_images, p->n_touch, p->d_status, st);
    if (err) return err;
    // 2. scaling
    k_rowstats<<<dim3((m * 32 + 255) / 256, 2, nb), 256, 0, st>>>(p->d_Z, m, p->d_scale, d_rsum, N);
    k_rowstats_nodes<<<dim3((n + 127) / 128, nb), 128, 0, st>>>(p->inc.node_ptr, n, m, p->d_scale, d_rsum, N);
    tags_note_launch(2);
    // 3. FP32 working matrix and its LU (no pivoting)
    int pf = tags_prof_begin(TAGS_PROF_BUILD, st);
    k_build<<<dim3((unsigned)((N + 255) / 256), N, nb), 256, 0, st>>>(p->d_Z, p->d_cond, p->d_scale, m, n, p->d_A);
    tags_prof_end(TAGS_PROF_BUILD, pf, st, 0.0, (8.0 * 0.5 * N * (N + 1.0) + 32.0 * m * m) * nb);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    err = tags_ldl_tc(p->d_A, N, N, (long long)NN, nb, p->batch, p->d_ldlws, p->d_info, p->d_ldlerr, m,
                      p->split_pieces, st);
    if (err) return err;
    // 4. refinement
    std::vector<int> active(nb, 1), conv(nb, 0), iters(nb, 0);
    std::vector<double> prev_dx(nb, INFINITY), hn(4 * nb);
    std::vector<int> info(nb);
    int tc_err = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(info.data(), p->d_info, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(&tc_err, p->d_ldlerr, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (tc_err) {
        // a tensor-core wait ran out: the whole pass goes to the FP64 path
        tags_fail(TAGS_E_CUDA, "tensor-core factorisation reported a timeout; samples re-solved in FP64");
        TAGS_CUDA_OK(cudaMemsetAsync(p->d_ldlerr, 0, sizeof(int), st));
        for (int q = 0; q < nb; ++q) active[q] = 0;
    }
    for (int q = 0; q < nb; ++q)
        if (info[q] != 0) active[q] = 0;   // zero pivot in the static order: straight to the fallback
    // r = b initially
    k_copy_c<<<(unsigned)(((long long)nb * N + 255) / 256), 256, 0, st>>>(d_b, p->d_r, (long long)nb * N);
    tags_note_launch();
    TAGS_CUDA_OK(cudaMemsetAsync(p->d_norms, 0, sizeof(double) * 4 * nb, st));
    k_max_rows<<<dim3((N + 255) / 256, nb), 256, 0, st>>>(d_rsum, N, p->d_norms);
    tags_note_launch();
    std::vector<double> wnorm(nb);
    TAGS_CUDA_OK(cudaMemcpyAsync(hn.data(), p->d_norms, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    for (int q = 0; q < nb; ++q) wnorm[q] = hn[4 * q + 3];
    const int max_it = 40;
    for (int it = 0; it < max_it; ++it) {
        bool any = false;
        for (int q = 0; q < nb; ++q) any |= active[q] != 0;
        if (!any) break;
        TAGS_CUDA_OK(cudaMemcpyAsync(d_active, active.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemsetAsync(p->d_norms, 0, sizeof(double) * 4 * nb, st));
        dim3 gv((N + 255) / 256, nb);
        k_ir_rhs<<<gv, 256, 0, st>>>(p->d_r, p->d_scale, m, n, p->d_rf);
        tags_note_launch();
        err = tags_ldl_solve_c(p->d_A, N, N, (long long)NN, nb, p->batch, p->d_ldlws, p->d_rf, N, m, st);
        if (err) return err;
        k_ir_update<<<gv, 256, 0, st>>>(p->d_rf, p->d_scale, m, n, p->d_x, p->d_norms, d_active);
        pf = tags_prof_begin(TAGS_PROF_RESID, st);
        k_residual_nodes<<<dim3((n + 255) / 256, nb), 256, 0, st>>>(p->inc, m, n, d_b, p->d_x, p->d_r, p->d_norms,
                                                                    d_active);
        k_residual_z<<<dim3((m + 255) / 256, 2 * nb), 256, 0, st>>>(p->d_Z, p->inc, m, n, d_b, p->d_x, p->d_r,
                                                                    p->d_norms, d_active);
        // 2 m^2 complex products (4 real multiply-adds each) and a read of Z in FP32
        tags_prof_end(TAGS_PROF_RESID, pf, st, 16.0 * m * (double)m * nb, 16.0 * m * (double)m * nb);
        tags_note_launch(2);
        TAGS_CUDA_OK(cudaGetLastError());
        TAGS_CUDA_OK(cudaMemcpyAsync(hn.data(), p->d_norms, sizeof(double) * 4 * nb, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
        for (int q = 0; q < nb; ++q) {
            if (!active[q]) continue;
            iters[q] = it + 1;
            double dx = hn[4 * q + 0], xn = hn[4 * q + 1], rn = hn[4 * q + 2];
            h_berr[q] = rn / (wnorm[q] * xn + 1e-300);
            if (!(dx == dx) || !(xn == xn)) { active[q] = 0; continue; }       // NaN: fallback
            // the residual is accurate to ~2^-44 |W| |x| (two-float products): stop
            // once the correction is below that level or stops shrinking
            if (dx <= 1e-13 * xn) { active[q] = 0; conv[q] = 1; continue; }
            if (it >= 2 && dx > 0.5 * prev_dx[q]) {
                if (h_berr[q] <= 1e-12) conv[q] = 1;
                active[q] = 0;
                continue;
            }
            prev_dx[q] = dx;
        }
    }
    // 5. fallback for samples that did not converge
    for (int q = 0; q < nb; ++q) {
        h_iters[q] = iters[q];
        h_conv[q] = conv[q];
        if (!conv[q]) {
            err = fallback_plain(p, q, st);
            if (err) return err;
        }
    }
    // converged samples report success; fallbacks keep their own LU info
    for (int q = 0; q < nb; ++q)
        if (conv[q]) TAGS_CUDA_OK(cudaMemsetAsync(p->d_info + q, 0, sizeof(int), st));
    return 0;
}
