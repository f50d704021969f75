// Immittance-system assembly on the device.
//
// Replaces fill_incidence_imm (src/linalg.c:12-86) and fill_impedance_imm
// (src/linalg.c:88-110). The incidence of node n on segment e is decided
// exactly as the reference does (|coordinate difference| <= 1e-5 per axis,
// start tested before end) and kept as a small integer code; all W_G entries
// are then written from those codes (+1 / -1 for A, 0.5 for B).
#include "tags_common.cuh"
#include "tags_internal.h"

namespace {

__global__ void k_incidence_codes(const double* __restrict__ elec, int m, const double* __restrict__ nodes, int n,
                                  signed char* __restrict__ cond) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * m) return;
    int nd = (int)(t / m), e = (int)(t % m);
    const double* s = elec + 11LL * e;
    const double* p = nodes + 3LL * nd;
    const double tol = 1e-5;
    bool st = fabs(s[0] - p[0]) <= tol && fabs(s[1] - p[1]) <= tol && fabs(s[2] - p[2]) <= tol;
    bool en = fabs(s[3] - p[0]) <= tol && fabs(s[4] - p[1]) <= tol && fabs(s[5] - p[2]) <= tol;
    cond[t] = st ? 1 : (en ? 2 : 0);
}

// Writes the incidence entries of W_G (original ordering, leading dim ld):
// A at rows n+e, col nd; B at rows n+m+e; and the transposes.
__global__ void k_wg_incidence(double2* __restrict__ W0, long long ld, long long stride,
                               const signed char* __restrict__ cond, int n, int m) {
    double2* W = W0 + stride * blockIdx.y;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * m) return;
    int nd = (int)(t / m), e = (int)(t % m);
    int c = cond[t];
    if (!c) return;
    double av = c == 1 ? 1.0 : -1.0;
    W[(n + e) + ld * nd] = cz(av, 0.0);
    W[(n + m + e) + ld * nd] = cz(0.5, 0.0);
    W[nd + ld * (n + e)] = cz(av, 0.0);
    W[nd + ld * (n + m + e)] = cz(0.5, 0.0);
}

// fill_impedance_imm: -ZL and -ZT (whole m x m blocks as stored) into W_G,
// zero ZL/ZT coupling blocks and zero Y_E.
__global__ void k_wg_impedance(double2* __restrict__ W, long long ld, const double2* __restrict__ zl,
                               const double2* __restrict__ zt, int m, int n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long tot = (long long)m * m;
    if (t < tot) {
        int i = (int)(t % m), k = (int)(t / m);
        W[(i + n) + ld * (k + n)] = cneg(zl[i + (long long)m * k]);
        W[(i + n) + ld * (k + n + m)] = cz(0.0, 0.0);
        W[(i + n + m) + ld * (k + n)] = cz(0.0, 0.0);
        W[(i + n + m) + ld * (k + n + m)] = cneg(zt[i + (long long)m * k]);
    }
    if (t < (long long)n * n) {
        int i = (int)(t % n), k = (int)(t / n);
        W[i + ld * k] = cz(0.0, 0.0);
    }
}

// Mirror the lower triangle onto the upper one (zsysv('L') reads only the
// lower half; the LU factorises the full symmetric matrix).
__global__ void k_symmetrize_lower(double2* __restrict__ W0, int N, long long ld, long long stride) {
    double2* W = W0 + stride * blockIdx.z;
    int r = blockIdx.x * 32 + threadIdx.x;     // row of the upper element
    int c = blockIdx.y * 32 + threadIdx.y;     // col of the upper element
    if (r < N && c < N && c > r) W[r + ld * c] = W[c + ld * r];
}

}  // namespace

int tags_incidence_codes(const double* d_elec, int m, const double* d_nodes, int n, signed char* d_cond,
                         cudaStream_t st) {
    long long tot = (long long)n * m;
    if (tot == 0) return 0;
    k_incidence_codes<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(d_elec, m, d_nodes, n, d_cond);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_wg_incidence(double2* d_W, long long ld, long long stride, int batch, const signed char* d_cond, int n,
                      int m, cudaStream_t st) {
    long long tot = (long long)n * m;
    if (tot == 0) return 0;
    k_wg_incidence<<<dim3((unsigned)((tot + 255) / 256), batch), 256, 0, st>>>(d_W, ld, stride, d_cond, n, m);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_wg_impedance(double2* d_W, long long ld, const double2* d_zl, const double2* d_zt, int m, int n,
                      cudaStream_t st) {
    long long tot = (long long)m * m > (long long)n * n ? (long long)m * m : (long long)n * n;
    if (tot == 0) return 0;
    k_wg_impedance<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(d_W, ld, d_zl, d_zt, m, n);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_symmetrize_lower(double2* d_W, int N, long long ld, long long stride, int batch, cudaStream_t st) {
    if (N <= 0) return 0;
    dim3 g((N + 31) / 32, (N + 31) / 32, batch);
    k_symmetrize_lower<<<g, dim3(32, 32), 0, st>>>(d_W, N, ld, stride);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}
