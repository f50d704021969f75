// Batched dense complex LU factorisation and triangular solves (CUDA cores).
//
// Replaces the reference's dense solve of the immittance system,
// solve_immittance -> zsysv('L') (src/linalg.c:112-139). The plain FP64 form
// uses LU with partial pivoting on the symmetrised W_G (row interchanges as in
// LAPACK's getrf: pivot = first index of max |Re|+|Im|). The same kernels,
// instantiated for complex FP32 and without pivoting, serve the mixed form's
// statically ordered factorisation. Right-looking blocked algorithm with a
// panel width NB: panel factorisation, row interchanges, triangular solve of
// the block row, trailing update C -= L21 * U12.
//
// Layout: column-major, leading dimension ld, one matrix per blockIdx.z
// (pointer + z * stride). ipiv is 0-based global row indices.
#include <mutex>
#include <type_traits>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

template <typename T> struct Cx;
template <> struct Cx<double2> {
    using R = double;
    static TAGS_D double2 zero() { return make_double2(0.0, 0.0); }
    static TAGS_D double2 mul(double2 a, double2 b) { return cmul(a, b); }
    static TAGS_D double2 fma(double2 a, double2 b, double2 c) { return cfma(a, b, c); }
    static TAGS_D double2 sub(double2 a, double2 b) { return csub(a, b); }
    static TAGS_D double abs1(double2 a) { return fabs(a.x) + fabs(a.y); }
    static TAGS_D double2 inv(double2 a) { return cdiv(make_double2(1.0, 0.0), a); }
    static TAGS_D bool is_zero(double2 a) { return a.x == 0.0 && a.y == 0.0; }
};
template <> struct Cx<float2> {
    using R = float;
    static TAGS_D float2 zero() { return make_float2(0.f, 0.f); }
    static TAGS_D float2 mul(float2 a, float2 b) { return fmulc(a, b); }
    static TAGS_D float2 fma(float2 a, float2 b, float2 c) { return ffmac(a, b, c); }
    static TAGS_D float2 sub(float2 a, float2 b) { return fsub(a, b); }
    static TAGS_D float abs1(float2 a) { return fabsf(a.x) + fabsf(a.y); }
    static TAGS_D float2 inv(float2 a) {
        double2 r = cdiv(make_double2(1.0, 0.0), make_double2(a.x, a.y));
        return make_float2((float)r.x, (float)r.y);
    }
    static TAGS_D bool is_zero(float2 a) { return a.x == 0.f && a.y == 0.f; }
};
// negation for the subtraction in the trailing update
TAGS_D double2 negc(double2 a) { return make_double2(-a.x, -a.y); }
TAGS_D float2 negc(float2 a) { return make_float2(-a.x, -a.y); }

constexpr int PANEL_THREADS = 512;

// Factor the panel A[j0:n, j0:j0+jb] in place (unblocked, column by column).
// One CTA per matrix. With `pivot`, rows are interchanged inside the panel
// only; the rest of the matrix is swapped by k_laswp afterwards.
template <typename T>
__global__ void __launch_bounds__(PANEL_THREADS) k_panel(T* __restrict__ A0, int n, long long ld, long long stride,
                                                          int j0, int jb, int pivot, int* __restrict__ ipiv0,
                                                          int* __restrict__ info0) {
    using C = Cx<T>;
    using R = typename C::R;
    T* A = A0 + stride * blockIdx.z;
    int* ipiv = ipiv0 ? ipiv0 + (long long)n * blockIdx.z : nullptr;
    int* info = info0 + blockIdx.z;
    __shared__ R s_val[PANEL_THREADS / 32];
    __shared__ int s_idx[PANEL_THREADS / 32];
    __shared__ T s_row[128];
    __shared__ int s_p;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int c = j0; c < j0 + jb; ++c) {
        int p = c;
        if (pivot) {
            R best = -1;
            int bi = n;
            for (int r = c + tid; r < n; r += blockDim.x) {
                R v = C::abs1(A[r + ld * c]);
                if (v > best) { best = v; bi = r; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                R ov = __shfl_down_sync(0xffffffffu, best, o);
                int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) { s_val[warp] = best; s_idx[warp] = bi; }
            __syncthreads();
            if (tid == 0) {
                R b = s_val[0];
                int i = s_idx[0];
                for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
                    if (s_val[w] > b || (s_val[w] == b && s_idx[w] < i)) { b = s_val[w]; i = s_idx[w]; }
                s_p = (i < n) ? i : c;
            }
            __syncthreads();
            p = s_p;
            if (tid == 0 && ipiv) ipiv[c] = p;
            if (p != c) {
                for (int cc = j0 + tid; cc < j0 + jb; cc += blockDim.x) {
                    T t = A[c + ld * cc];
                    A[c + ld * cc] = A[p + ld * cc];
                    A[p + ld * cc] = t;
                }
            }
            __syncthreads();
        } else if (tid == 0 && ipiv) {
            ipiv[c] = c;
        }
        // pivot row of the panel to shared memory
        for (int cc = c + tid; cc < j0 + jb; cc += blockDim.x) s_row[cc - j0] = A[c + ld * cc];
        __syncthreads();
        T piv = s_row[c - j0];
        if (C::is_zero(piv)) {
            if (tid == 0 && *info == 0) *info = c + 1;
            __syncthreads();
            continue;
        }
        T ip = C::inv(piv);
        for (int r = c + 1 + tid; r < n; r += blockDim.x) {
            T l = C::mul(A[r + ld * c], ip);
            A[r + ld * c] = l;
            T nl = negc(l);
            for (int cc = c + 1; cc < j0 + jb; ++cc) A[r + ld * cc] = C::fma(nl, s_row[cc - j0], A[r + ld * cc]);
        }
        __syncthreads();
    }
}

// Apply the interchanges ipiv[j0:j0+jb] to the columns outside the panel.
template <typename T>
__global__ void k_laswp(T* __restrict__ A0, int n, long long ld, long long stride, int j0, int jb,
                        const int* __restrict__ ipiv0) {
    T* A = A0 + stride * blockIdx.z;
    const int* ipiv = ipiv0 + (long long)n * blockIdx.z;
    int col = blockIdx.x * blockDim.x + threadIdx.x;
    int ncols = n - jb;
    if (col >= ncols) return;
    int j = col < j0 ? col : col + jb;
    for (int c = j0; c < j0 + jb; ++c) {
        int p = ipiv[c];
        if (p != c) {
            T t = A[c + ld * j];
            A[c + ld * j] = A[p + ld * j];
            A[p + ld * j] = t;
        }
    }
}

// U12 = L11^{-1} A12, L11 = unit lower jb x jb at (j0, j0), columns j0+jb..n.
// One CTA per 32 columns; the block row tile lives in shared memory.
template <typename T, int NB>
__global__ void __launch_bounds__(256) k_trsm_row(T* __restrict__ A0, int n, long long ld, long long stride,
                                                  int j0, int jb) {
    using C = Cx<T>;
    T* A = A0 + stride * blockIdx.z;
    __shared__ T sL[NB][NB + 1];
    __shared__ T sX[NB][33];
    const int c0 = j0 + jb + blockIdx.x * 32;
    const int ncol = min(32, n - c0);
    if (ncol <= 0) return;
    for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
        int r = t % jb, c = t / jb;
        sL[r][c] = A[(j0 + r) + ld * (j0 + c)];
    }
    for (int t = threadIdx.x; t < jb * 32; t += blockDim.x) {
        int r = t % jb, c = t / jb;
        sX[r][c] = c < ncol ? A[(j0 + r) + ld * (c0 + c)] : C::zero();
    }
    __syncthreads();
    for (int k = 0; k < jb; ++k) {
        for (int t = threadIdx.x; t < (jb - k - 1) * 32; t += blockDim.x) {
            int r = k + 1 + t / 32, c = t % 32;
            sX[r][c] = C::fma(negc(sL[r][k]), sX[k][c], sX[r][c]);
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < jb * 32; t += blockDim.x) {
        int r = t % jb, c = t / jb;
        if (c < ncol) A[(j0 + r) + ld * (c0 + c)] = sX[r][c];
    }
}

// Trailing update C -= L21 * U12 over rows/cols [j0+jb, n). 64x64 output tile,
// 256 threads with a 4x4 register tile, K = jb <= NB in one shared stage.
template <typename T, int NB>
__global__ void __launch_bounds__(256) k_gemm_update(T* __restrict__ A0, int n, long long ld, long long stride,
                                                     int j0, int jb) {
    using C = Cx<T>;
    T* A = A0 + stride * blockIdx.z;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sA = reinterpret_cast<T*>(smem_raw);          // [NB][64]  (k-major: sA[k*64 + r])
    T* sB = sA + NB * 64;                            // [NB][64]  (sB[k*64 + c])
    const int base = j0 + jb;
    const int r0 = base + blockIdx.y * 64, c0 = base + blockIdx.x * 64;
    if (r0 >= n || c0 >= n) return;
    for (int t = threadIdx.x; t < jb * 64; t += blockDim.x) {
        int r = t & 63, k = t >> 6;
        int gr = r0 + r;
        sA[k * 64 + r] = gr < n ? A[gr + ld * (j0 + k)] : C::zero();
        int c = t & 63, kk = t >> 6;
        int gc = c0 + c;
        // U12 row (j0+kk) read along columns: element (j0+kk, gc)
        sB[kk * 64 + c] = gc < n ? A[(j0 + kk) + ld * gc] : C::zero();
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = C::zero();
    for (int k = 0; k < jb; ++k) {
        T av[4], bv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) av[a] = sA[k * 64 + ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) bv[b] = sB[k * 64 + tx + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] = C::fma(av[a], bv[b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        int gr = r0 + ty + 16 * a;
        if (gr >= n) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            int gc = c0 + tx + 16 * b;
            if (gc < n) {
                long long idx = gr + ld * gc;
                A[idx] = C::sub(A[idx], acc[a][b]);
            }
        }
    }
}

// ---- triangular solves with nrhs columns (x overwritten) ---------------------

// Apply ipiv forward (LAPACK laswp order) to the right-hand sides.
template <typename T>
__global__ void k_rhs_swap(T* __restrict__ X0, int n, int nrhs, long long ldx, long long xstride,
                           const int* __restrict__ ipiv0) {
    T* X = X0 + xstride * blockIdx.z;
    const int* ipiv = ipiv0 + (long long)n * blockIdx.z;
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nrhs) return;
    for (int c = 0; c < n; ++c) {
        int p = ipiv[c];
        if (p != c) {
            T t = X[c + ldx * j];
            X[c + ldx * j] = X[p + ldx * j];
            X[p + ldx * j] = t;
        }
    }
}

// Solve the jb x jb diagonal block at j0 (lower unit or upper non-unit) for
// every right-hand side; one CTA per matrix.
template <typename T, int NB>
__global__ void __launch_bounds__(256) k_trsv_diag(const T* __restrict__ A0, int n, long long ld, long long stride,
                                                   T* __restrict__ X0, int nrhs, long long ldx, long long xstride,
                                                   int j0, int jb, int upper) {
    using C = Cx<T>;
    const T* A = A0 + stride * blockIdx.z;
    T* X = X0 + xstride * blockIdx.z;
    __shared__ T sL[NB][NB + 1];
    __shared__ T sx[NB][9];
    for (int t = threadIdx.x; t < jb * jb; t += blockDim.x) {
        int r = t % jb, c = t / jb;
        sL[r][c] = A[(j0 + r) + ld * (j0 + c)];
    }
    for (int j = 0; j < nrhs; j += 8) {
        int nj = min(8, nrhs - j);
        __syncthreads();
        for (int t = threadIdx.x; t < jb * nj; t += blockDim.x) {
            int r = t % jb, c = t / jb;
            sx[r][c] = X[(j0 + r) + ldx * (j + c)];
        }
        __syncthreads();
        if (!upper) {
            for (int k = 0; k < jb; ++k) {
                for (int t = threadIdx.x; t < (jb - k - 1) * nj; t += blockDim.x) {
                    int r = k + 1 + t / nj, c = t % nj;
                    sx[r][c] = C::fma(negc(sL[r][k]), sx[k][c], sx[r][c]);
                }
                __syncthreads();
            }
        } else {
            for (int k = jb - 1; k >= 0; --k) {
                if (threadIdx.x < nj) sx[k][threadIdx.x] = C::mul(sx[k][threadIdx.x], C::inv(sL[k][k]));
                __syncthreads();
                for (int t = threadIdx.x; t < k * nj; t += blockDim.x) {
                    int r = t / nj, c = t % nj;
                    sx[r][c] = C::fma(negc(sL[r][k]), sx[k][c], sx[r][c]);
                }
                __syncthreads();
            }
        }
        for (int t = threadIdx.x; t < jb * nj; t += blockDim.x) {
            int r = t % jb, c = t / jb;
            X[(j0 + r) + ldx * (j + c)] = sx[r][c];
        }
    }
}

// X[rows] -= A[rows, j0:j0+jb] * X[j0:j0+jb]; rows = [j0+jb, n) (lower) or
// [0, j0) (upper). One thread per (row, rhs).
template <typename T>
__global__ void k_trsv_update(const T* __restrict__ A0, int n, long long ld, long long stride,
                              T* __restrict__ X0, int nrhs, long long ldx, long long xstride, int j0, int jb,
                              int upper) {
    using C = Cx<T>;
    const T* A = A0 + stride * blockIdx.z;
    T* X = X0 + xstride * blockIdx.z;
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    int rbeg = upper ? 0 : j0 + jb, rend = upper ? j0 : n;
    r += rbeg;
    if (r >= rend || j >= nrhs) return;
    T acc = C::zero();
    for (int k = 0; k < jb; ++k) acc = C::fma(A[r + ld * (j0 + k)], X[(j0 + k) + ldx * j], acc);
    X[r + ldx * j] = C::sub(X[r + ldx * j], acc);
}

constexpr int NB = 32;

}  // namespace

// Kernel attributes of the LU, set once per process before any launch (and
// so before any graph capture).
int tags_lu_prepare() {
    static std::once_flag once;
    static int rc = 0;
    std::call_once(once, [] {
        const int g64 = (int)(2 * NB * 64 * sizeof(double2)), g32 = (int)(2 * NB * 64 * sizeof(float2));
        if (cudaFuncSetAttribute(k_gemm_update<double2, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, g64) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_gemm_update<float2, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, g32) !=
                cudaSuccess)
            rc = tags_fail(TAGS_E_CUDA, "cudaFuncSetAttribute(k_gemm_update) failed");
    });
    return rc;
}

namespace {

template <typename T>
int lu_impl(T* A, int n, long long ld, long long stride, int batch, int pivot, int* ipiv, int* info,
            cudaStream_t st) {
    TAGS_CUDA_OK(cudaMemsetAsync(info, 0, sizeof(int) * batch, st));
    const size_t gsmem = 2 * NB * 64 * sizeof(T);
    if (int e = tags_lu_prepare()) return e;
    for (int j0 = 0; j0 < n; j0 += NB) {
        int jb = min(NB, n - j0);
        k_panel<T><<<dim3(1, 1, batch), PANEL_THREADS, 0, st>>>(A, n, ld, stride, j0, jb, pivot, ipiv, info);
        tags_note_launch();
        if (pivot) {
            int ncols = n - jb;
            if (ncols > 0) {
                k_laswp<T><<<dim3((ncols + 127) / 128, 1, batch), 128, 0, st>>>(A, n, ld, stride, j0, jb, ipiv);
                tags_note_launch();
            }
        }
        int rest = n - j0 - jb;
        if (rest > 0) {
            k_trsm_row<T, NB><<<dim3((rest + 31) / 32, 1, batch), 256, 0, st>>>(A, n, ld, stride, j0, jb);
            tags_note_launch();
            dim3 g((rest + 63) / 64, (rest + 63) / 64, batch);
            int pf = std::is_same<T, double2>::value ? tags_prof_begin(TAGS_PROF_LU64_GEMM, st) : -1;
            k_gemm_update<T, NB><<<g, 256, gsmem, st>>>(A, n, ld, stride, j0, jb);
            // rank-jb update of a rest x rest block: 8 rest^2 jb real flops
            tags_prof_end(TAGS_PROF_LU64_GEMM, pf, st, 8.0 * rest * (double)rest * jb * batch,
                          (32.0 * rest * (double)rest + 32.0 * rest * jb) * batch);
            tags_note_launch();
        }
    }
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

template <typename T>
int lu_solve_impl(const T* A, int n, long long ld, long long stride, int batch, const int* ipiv, T* X, int nrhs,
                  long long ldx, long long xstride, cudaStream_t st) {
    if (ipiv) {
        k_rhs_swap<T><<<dim3((nrhs + 31) / 32, 1, batch), 32, 0, st>>>(X, n, nrhs, ldx, xstride, ipiv);
        tags_note_launch();
    }
    for (int j0 = 0; j0 < n; j0 += NB) {
        int jb = min(NB, n - j0);
        k_trsv_diag<T, NB><<<dim3(1, 1, batch), 256, 0, st>>>(A, n, ld, stride, X, nrhs, ldx, xstride, j0, jb, 0);
        tags_note_launch();
        int rest = n - j0 - jb;
        if (rest > 0) {
            k_trsv_update<T><<<dim3((rest + 127) / 128, nrhs, batch), 128, 0, st>>>(A, n, ld, stride, X, nrhs, ldx,
                                                                                 xstride, j0, jb, 0);
            tags_note_launch();
        }
    }
    int last = ((n - 1) / NB) * NB;
    for (int j0 = last; j0 >= 0; j0 -= NB) {
        int jb = min(NB, n - j0);
        k_trsv_diag<T, NB><<<dim3(1, 1, batch), 256, 0, st>>>(A, n, ld, stride, X, nrhs, ldx, xstride, j0, jb, 1);
        tags_note_launch();
        if (j0 > 0) {
            k_trsv_update<T><<<dim3((j0 + 127) / 128, nrhs, batch), 128, 0, st>>>(A, n, ld, stride, X, nrhs, ldx,
                                                                               xstride, j0, jb, 1);
            tags_note_launch();
        }
    }
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

}  // namespace

int tags_lu_z(double2* A, int n, long long ld, long long stride, int batch, int pivot, int* ipiv, int* info,
              cudaStream_t st) {
    return lu_impl<double2>(A, n, ld, stride, batch, pivot, ipiv, info, st);
}
int tags_lu_c(float2* A, int n, long long ld, long long stride, int batch, int pivot, int* ipiv, int* info,
              cudaStream_t st) {
    return lu_impl<float2>(A, n, ld, stride, batch, pivot, ipiv, info, st);
}
int tags_lu_solve_z(const double2* A, int n, long long ld, long long stride, int batch, const int* ipiv, double2* X,
                    int nrhs, long long ldx, long long xstride, cudaStream_t st) {
    return lu_solve_impl<double2>(A, n, ld, stride, batch, ipiv, X, nrhs, ldx, xstride, st);
}
int tags_lu_solve_c(const float2* A, int n, long long ld, long long stride, int batch, const int* ipiv, float2* X,
                    int nrhs, long long ldx, long long xstride, cudaStream_t st) {
    return lu_solve_impl<float2>(A, n, ld, stride, batch, ipiv, X, nrhs, ldx, xstride, st);
}
