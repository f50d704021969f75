// Numerical Laplace transform pair in FP64 on the device.
//
// Replaces laplace_trans / inv_laplace_trans (src/auxiliary.c:239-329) and the
// batched inverse of the examples (examples/three_grids.c:447-465), which use
// FFTW r2c/c2r. Here the transforms are direct sums over an FP64 twiddle
// table indexed by (j*k mod nt), so the result does not depend on an FFT
// factorisation and stays accurate to ~nt*eps:
//   forward  G[k] = sum_j f[j] dt e^{-c t_j} e^{-2 pi i jk/nt},   k < nt/2+1
//   inverse  f[j] = (sum_k sigma_k G[k] e^{+2 pi i jk/nt} over the Hermitian
//            extension) * e^{c t_j} / (nt dt),   c = Re s_0,
// with the reference's data windows sigma (src/auxiliary.c:279-317).
#include "tags_common.cuh"
#include "tags_internal.h"

namespace {

__global__ void k_twiddles(double2* __restrict__ tw, long long nt) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nt) return;
    double s, c;
    // angle 2 pi q / nt in [0, 2 pi); sincospi keeps it exact at the quadrants
    sincospi(2.0 * (double)q / (double)nt, &s, &c);
    tw[q] = make_double2(c, s);
}

__device__ double window(int filter, double w, double omega) {
    double alpha;
    switch (filter) {
    case 1: alpha = TAGS_PI * w / omega; return 0.42 + 0.5 * cos(alpha) + 0.08 * cos(2 * alpha);
    case 2: return (1 + cos(TAGS_PI * w / omega)) / 2;
    case 3: alpha = TAGS_PI * w / omega; return sin(alpha) / alpha;
    case 4: return 1.0 - (w / omega) * (w / omega);
    default: return 1.0;
    }
}

// One thread per (time index j, series). g: ns values per series, series
// stride gstride; f: nt values per series, stride fstride.
__global__ void k_inlt(const double2* __restrict__ g, long long gstride, long long ns, const double2* __restrict__ s,
                       const double2* __restrict__ tw, long long nt, double tmax, int filter, double* __restrict__ f,
                       long long fstride, int nseries) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int srs = blockIdx.y;
    if (j >= nt || srs >= nseries) return;
    const double2* G = g + gstride * srs;
    const double omega = s[ns - 1].y;
    const long long half = nt / 2;
    double acc = G[0].x * window(filter, s[0].y, omega);
    long long kmax = (nt % 2 == 0) ? half - 1 : half;
    for (long long k = 1; k <= kmax; ++k) {
        long long q = (j * k) % nt;
        double2 t = tw[q];
        double sg = window(filter, s[k].y, omega);
        double2 v = G[k];
        acc += 2.0 * sg * (v.x * t.x - v.y * t.y);
    }
    if (nt % 2 == 0 && nt > 1) acc += ((j & 1) ? -1.0 : 1.0) * G[half].x * window(filter, s[half].y, omega);
    const double dt = tmax / (double)(nt - 1);
    const double c = s[0].x;
    f[fstride * srs + j] = acc * exp(c * (double)j * dt) / ((double)nt * dt);
}

// Batched inverse in the examples' layout (examples/three_grids.c:229-242,
// :447-465): g[series + k nser] (sample-major), f[series + j nser], scaled by
// e^{c t_j} / (nt dt). One thread per (series, time index): threads run along
// the series, so the reads of g and the writes of f are contiguous and the
// twiddle is the same for the whole block.
__global__ void k_inlt_rows(const double2* __restrict__ g, long long ns, const double2* __restrict__ s,
                            const double2* __restrict__ tw, long long nt, double tmax, int filter,
                            double* __restrict__ f, long long nser) {
    const long long srs = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long j = blockIdx.y;
    if (srs >= nser || j >= nt) return;
    const double omega = s[ns - 1].y;
    const long long half = nt / 2;
    double acc = g[srs].x * window(filter, s[0].y, omega);
    const long long kmax = (nt % 2 == 0) ? half - 1 : half;
    for (long long k = 1; k <= kmax; ++k) {
        const double2 t = tw[(j * k) % nt];
        const double2 v = g[srs + k * nser];
        acc += 2.0 * window(filter, s[k].y, omega) * (v.x * t.x - v.y * t.y);
    }
    if (nt % 2 == 0 && nt > 1) acc += ((j & 1) ? -1.0 : 1.0) * g[srs + half * nser].x * window(filter, s[half].y, omega);
    const double dt = tmax / (double)(nt - 1);
    f[srs + j * nser] = acc * exp(s[0].x * (double)j * dt) / ((double)nt * dt);
}

// Forward transform with the damping of the numerical Laplace transform.
__global__ void k_nlt(const double* __restrict__ f, long long fstride, long long nt, const double2* __restrict__ tw,
                      double tmax, double2* __restrict__ g, long long gstride, int nseries) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int srs = blockIdx.y;
    long long ns = nt / 2 + 1;
    if (k >= ns || srs >= nseries) return;
    const double* F = f + fstride * srs;
    const double c = log((double)nt * (double)nt) / tmax;
    const double dt = tmax / (double)(nt - 1);
    double re = 0.0, im = 0.0;
    for (long long j = 0; j < nt; ++j) {
        double v = F[j] * dt * exp(-c * (double)j * dt);
        double2 t = tw[(j * k) % nt];
        re += v * t.x;
        im -= v * t.y;
    }
    g[gstride * srs + k] = make_double2(re, im);
}

}  // namespace

int tags_twiddles(double2* d_tw, long long nt, cudaStream_t st) {
    k_twiddles<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(d_tw, nt);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_inlt(const double2* d_g, long long gstride, long long ns, const double2* d_s, const double2* d_tw,
                     long long nt, double tmax, int filter, double* d_f, long long fstride, int nseries,
                     cudaStream_t st) {
    dim3 grid((unsigned)((nt + 127) / 128), nseries);
    k_inlt<<<grid, 128, 0, st>>>(d_g, gstride, ns, d_s, d_tw, nt, tmax, filter, d_f, fstride, nseries);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_inlt_rows(const double2* d_g, long long ns, const double2* d_s, const double2* d_tw, long long nt,
                          double tmax, int filter, double* d_f, long long nser, cudaStream_t st) {
    dim3 grid((unsigned)((nser + 127) / 128), (unsigned)nt);
    k_inlt_rows<<<grid, 128, 0, st>>>(d_g, ns, d_s, d_tw, nt, tmax, filter, d_f, nser);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

int tags_launch_nlt(const double* d_f, long long fstride, long long nt, const double2* d_tw, double tmax,
                    double2* d_g, long long gstride, int nseries, cudaStream_t st) {
    long long ns = nt / 2 + 1;
    dim3 grid((unsigned)((ns + 127) / 128), nseries);
    k_nlt<<<grid, 128, 0, st>>>(d_f, fstride, nt, d_tw, tmax, d_g, gstride, nseries);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}
