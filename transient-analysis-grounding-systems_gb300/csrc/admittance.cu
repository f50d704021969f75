// Drop-ins for the reference's nodal admittance formulation, the solve its
// mHEM examples use (src/linalg.c:142-350, called from
// examples/three_grids.c:270-392):
//   fill_incidence_adm   A (+1 start, -1 end) and B (0.5), m x n column-major,
//                        from the exact node-matching codes, written in the
//                        reference's order with its checks;
//   calculate_yla_ytb    yla = ZL^{-1} A, ytb = ZT^{-1} B; ZL and ZT (lower
//                        triangles) are overwritten by their inverses, as
//                        zsytrf + zsytri leave them;
//   fill_impedance_adm2  YN = A^T yla + B^T ytb;
//   fill_impedance_adm   both steps;
//   solve_admittance     zsysv('L') semantics on YN (the factors are not
//                        written back).
// FP64 on the GPU: LU with partial pivoting of the symmetrised blocks
// (lu.cu), solves with all n columns of A (B) as right-hand sides, and YN as
// a sparse gather (A and B hold a few nonzeros per column). Host buffers in
// and out, as the reference's callers pass them.
#include <cstdio>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

// yn[i + n j] = sum over nonzeros (e, a) of column i of A: a yla[e + m j],
// plus the same over B with ytb. One thread per (i, j).
__global__ void k_adm_gather(const int* __restrict__ aptr, const int* __restrict__ aidx,
                             const double2* __restrict__ aval, const int* __restrict__ bptr,
                             const int* __restrict__ bidx, const double2* __restrict__ bval,
                             const double2* __restrict__ yla, const double2* __restrict__ ytb, int m, int n,
                             double2* __restrict__ yn) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= n) return;
    double2 acc = make_double2(0.0, 0.0);
    for (int q = aptr[i]; q < aptr[i + 1]; ++q) acc = cfma(aval[q], yla[aidx[q] + (long long)m * j], acc);
    for (int q = bptr[i]; q < bptr[i + 1]; ++q) acc = cfma(bval[q], ytb[bidx[q] + (long long)m * j], acc);
    yn[i + (long long)n * j] = acc;
}

__global__ void k_identity(double2* __restrict__ X, int m) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * m) return;
    X[t] = make_double2(t % m == t / m ? 1.0 : 0.0, 0.0);
}

// Nonzeros of the columns of a dense m x n matrix, column by column.
struct ColList {
    std::vector<int> ptr, idx;
    std::vector<double2> val;
};

ColList columns_of(const tags_cdouble* a, size_t m, size_t n) {
    ColList c;
    c.ptr.assign(n + 1, 0);
    for (size_t i = 0; i < n; ++i) {
        for (size_t e = 0; e < m; ++e) {
            const tags_cdouble v = a[e + m * i];
            if (v.re != 0.0 || v.im != 0.0) {
                c.idx.push_back((int)e);
                c.val.push_back(make_double2(v.re, v.im));
            }
        }
        c.ptr[i + 1] = (int)c.idx.size();
    }
    return c;
}

// Z^{-1} B into X (m x nrhs) and, if zinv, Z^{-1} into zinv (m x m): Z is
// the symmetric matrix whose lower triangle is in z (host, column-major).
int sym_solve(const tags_cdouble* z, const tags_cdouble* rhs, size_t m, size_t nrhs, tags_cdouble* x,
              tags_cdouble* zinv, int slot, cudaStream_t st) {
    DeviceCtx* c = tags_ctx();
    double2* d_Z = (double2*)c->scratch(slot, sizeof(double2) * m * m);
    double2* d_X = (double2*)c->scratch(slot + 1, sizeof(double2) * (m * (nrhs > m ? nrhs : m) + 1));
    int* d_ipiv = (int*)c->scratch(5, sizeof(int) * (m + 1));
    if (!d_Z || !d_X || !d_ipiv) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    TAGS_CUDA_OK(cudaMemcpyAsync(d_Z, z, sizeof(double2) * m * m, cudaMemcpyHostToDevice, st));
    int err = tags_symmetrize_lower(d_Z, (int)m, (long long)m, 0, 1, st);
    if (!err) err = tags_lu_z(d_Z, (int)m, (long long)m, 0, 1, 1, d_ipiv, d_ipiv + m, st);
    if (err) return err;
    int info = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(&info, d_ipiv + m, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (info > 0) return info;        // an exactly singular block, as zsytrf reports it
    if (nrhs) {
        TAGS_CUDA_OK(cudaMemcpyAsync(d_X, rhs, sizeof(double2) * m * nrhs, cudaMemcpyHostToDevice, st));
        err = tags_lu_solve_z(d_Z, (int)m, (long long)m, 0, 1, d_ipiv, d_X, (int)nrhs, (long long)m, 0, st);
        if (err) return err;
        TAGS_CUDA_OK(cudaMemcpyAsync(x, d_X, sizeof(double2) * m * nrhs, cudaMemcpyDeviceToHost, st));
    }
    if (zinv) {
        k_identity<<<(unsigned)((m * m + 255) / 256), 256, 0, st>>>(d_X, (int)m);
        tags_note_launch();
        err = tags_lu_solve_z(d_Z, (int)m, (long long)m, 0, 1, d_ipiv, d_X, (int)m, (long long)m, 0, st);
        if (err) return err;
        TAGS_CUDA_OK(cudaMemcpyAsync(zinv, d_X, sizeof(double2) * m * m, cudaMemcpyDeviceToHost, st));
    }
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

int yla_ytb_impl(tags_cdouble* yla, tags_cdouble* ytb, tags_cdouble* zl, tags_cdouble* zt, const tags_cdouble* a,
                 const tags_cdouble* b, size_t m, size_t n, cudaStream_t st) {
    std::vector<tags_cdouble> inv(m * m);
    for (int blk = 0; blk < 2; ++blk) {
        tags_cdouble* z = blk == 0 ? zl : zt;
        int info = sym_solve(z, blk == 0 ? a : b, m, n, blk == 0 ? yla : ytb, inv.data(), 6, st);
        if (info) return info;
        // the inverse replaces the lower triangle, as zsytri writes it (src/linalg.c:278-289)
        for (size_t k = 0; k < m; ++k)
            for (size_t i = k; i < m; ++i) z[i + m * k] = inv[i + m * k];
    }
    return 0;
}

int adm2_impl(tags_cdouble* yn, const tags_cdouble* yla, const tags_cdouble* ytb, const tags_cdouble* a,
              const tags_cdouble* b, size_t m, size_t n, cudaStream_t st) {
    DeviceCtx* c = tags_ctx();
    const ColList ca = columns_of(a, m, n), cb = columns_of(b, m, n);
    const size_t na = ca.idx.size(), nbz = cb.idx.size();
    double2* d_y = (double2*)c->scratch(6, sizeof(double2) * (2 * m * n + 1));
    double2* d_yn = (double2*)c->scratch(7, sizeof(double2) * (n * n + 1));
    int* d_i = (int*)c->scratch(8, sizeof(int) * (2 * (n + 1) + na + nbz + 2));
    double2* d_v = (double2*)c->scratch(9, sizeof(double2) * (na + nbz + 2));
    if (!d_y || !d_yn || !d_i || !d_v) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    int *aptr = d_i, *bptr = d_i + (n + 1), *aidx = d_i + 2 * (n + 1), *bidx = aidx + na;
    TAGS_CUDA_OK(cudaMemcpyAsync(d_y, yla, sizeof(double2) * m * n, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_y + m * n, ytb, sizeof(double2) * m * n, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(aptr, ca.ptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(bptr, cb.ptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    if (na) {
        TAGS_CUDA_OK(cudaMemcpyAsync(aidx, ca.idx.data(), sizeof(int) * na, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_v, ca.val.data(), sizeof(double2) * na, cudaMemcpyHostToDevice, st));
    }
    if (nbz) {
        TAGS_CUDA_OK(cudaMemcpyAsync(bidx, cb.idx.data(), sizeof(int) * nbz, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_v + na, cb.val.data(), sizeof(double2) * nbz, cudaMemcpyHostToDevice, st));
    }
    k_adm_gather<<<dim3((unsigned)((n + 127) / 128), (unsigned)n), 128, 0, st>>>(
        aptr, aidx, d_v, bptr, bidx, d_v + na, d_y, d_y + m * n, (int)m, (int)n, d_yn);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    TAGS_CUDA_OK(cudaMemcpyAsync(yn, d_yn, sizeof(double2) * n * n, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

}  // namespace

extern "C" int fill_incidence_adm(tags_cdouble* a, tags_cdouble* b, const Electrode* electrodes,
                                  size_t num_electrodes, const double* nodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    const size_t m = num_electrodes, n = num_nodes;
    if (n == 0) return 0;
    if (!a || !b || !electrodes || !nodes) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    std::vector<signed char> cond(n * m);
    if (m) {
        double* d_elec = (double*)c->scratch(0, sizeof(Electrode) * m);
        double* d_nodes = (double*)c->scratch(2, sizeof(double) * 3 * n);
        signed char* d_cond = (signed char*)c->scratch(1, n * m + 1);
        if (!d_elec || !d_nodes || !d_cond) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
        TAGS_CUDA_OK(cudaMemcpyAsync(d_elec, electrodes, sizeof(Electrode) * m, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_nodes, nodes, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        int err = tags_incidence_codes(d_elec, (int)m, d_nodes, (int)n, d_cond, st);
        if (err) return err;
        TAGS_CUDA_OK(cudaMemcpyAsync(cond.data(), d_cond, n * m, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    // written node by node, stopping after the first node without incidence
    // (src/linalg.c:157-192)
    long long suma = 0;
    double sumb = 0.0;
    for (size_t nd = 0; nd < n; ++nd) {
        bool none = true;
        for (size_t e = 0; e < m; ++e) {
            const int cd = cond[nd * m + e];
            const size_t pos = m * nd + e;
            // the reference's write order (b before a at a match) and read-back
            // sums, so that a == b (src/linalg.h:90) leaves A and the same code
            if (cd == 1) { b[pos] = {0.5, 0.0}; a[pos] = {1.0, 0.0}; }
            else if (cd == 2) { b[pos] = {0.5, 0.0}; a[pos] = {-1.0, 0.0}; }
            else { a[pos] = {0.0, 0.0}; b[pos] = {0.0, 0.0}; }
            suma += (long long)a[pos].re;
            sumb += b[pos].re;
            if (cd) none = false;
        }
        if (none) {
            char msg[96];
            snprintf(msg, sizeof(msg), "No electrode is connected to node[%i]\n", (int)nd);
            tags_msg(msg);
            return 1;
        }
    }
    if (suma != 0) {
        char msg[96];
        snprintf(msg, sizeof(msg), "incidence matrix A is wrong. sum(A) = %lli != 0\n", suma);
        tags_msg(msg);
        return (int)-suma;
    }
    if (sumb != (double)m) {
        char msg[128];
        snprintf(msg, sizeof(msg), "incidence matrix B is wrong. sum(B) = %.1f != %.1f\n", sumb, (double)m);
        tags_msg(msg);
        return (int)(sumb - (double)m);
    }
    return 0;
}

extern "C" int calculate_yla_ytb(tags_cdouble* yla, tags_cdouble* ytb, tags_cdouble* zl, tags_cdouble* zt,
                                 tags_cdouble* a, tags_cdouble* b, size_t num_electrodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    const size_t m = num_electrodes, n = num_nodes;
    if (m == 0) return 0;
    if (!yla || !ytb || !zl || !zt || !a || !b) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    return yla_ytb_impl(yla, ytb, zl, zt, a, b, m, n, c->stream);
}

extern "C" int fill_impedance_adm2(tags_cdouble* yn, tags_cdouble* yla, tags_cdouble* ytb, tags_cdouble* a,
                                   tags_cdouble* b, size_t num_electrodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    const size_t m = num_electrodes, n = num_nodes;
    if (n == 0) return 0;
    if (!yn || !yla || !ytb || !a || !b) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    return adm2_impl(yn, yla, ytb, a, b, m, n, c->stream);
}

extern "C" int fill_impedance_adm(tags_cdouble* yn, tags_cdouble* zl, tags_cdouble* zt, tags_cdouble* a,
                                  tags_cdouble* b, size_t num_electrodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    const size_t m = num_electrodes, n = num_nodes;
    if (n == 0) return 0;
    if (!yn || !zl || !zt || !a || !b) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    std::vector<tags_cdouble> yla(m * n), ytb(m * n);
    int info = yla_ytb_impl(yla.data(), ytb.data(), zl, zt, a, b, m, n, c->stream);
    if (info) return info;
    return adm2_impl(yn, yla.data(), ytb.data(), a, b, m, n, c->stream);
}

extern "C" int solve_admittance(tags_cdouble* yn, tags_cdouble* ic, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    const size_t n = num_nodes;
    if (n == 0) return 0;
    if (!yn || !ic) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    std::vector<tags_cdouble> x(n);
    int info = sym_solve(yn, ic, n, 1, x.data(), nullptr, 3, c->stream);
    if (info > 0) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "The diagonal element of the triangular factor of YN,\nU(%i,%i) is zero, so that YN is singular;\n"
                 "the solution could not be computed.\n",
                 info, info);
        tags_msg(msg);
        return info;
    }
    if (info) return info;
    for (size_t i = 0; i < n; ++i) ic[i] = x[i];
    return 0;
}
