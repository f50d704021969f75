// C-ABI of the GB300 HEM library: the reference-named drop-in entry points and
// the batched plan API declared in include/tags_gpu.h.
//
// Drop-ins copy the caller's host buffers to the device, run the kernels and
// copy the results back with the reference's memory contract (lower triangles
// only, accumulation where the reference accumulates, untouched elsewhere).
// Calls are serialised by a process-wide mutex; each uses the library's own
// stream on the caller's current device.
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

using zd = std::complex<double>;

namespace {

std::atomic<long long> g_launches{0};
thread_local long long t_launches = 0;    // this host thread's share (graph capture subtracts its own)
std::atomic<int> g_quiet{-1};
thread_local std::string g_last_error;
std::mutex g_mutex;

bool quiet() {
    int q = g_quiet.load();
    if (q < 0) {
        const char* e = getenv("TAGS_GPU_QUIET");
        q = (e && *e && *e != '0') ? 1 : 0;
        g_quiet.store(q);
    }
    return q != 0;
}

}  // namespace

void tags_note_launch(long long n) {
    g_launches += n;
    t_launches += n;
}

long long tags_thread_launch_count() { return t_launches; }

// drop-ins in other translation units share the scratch slots, so they
// serialise on the same lock
std::mutex& tags_dropin_mutex() { return g_mutex; }

int tags_fail_cuda(cudaError_t e, const char* what, const char* file, int line) {
    char buf[512];
    snprintf(buf, sizeof(buf), "CUDA error %s (%s) at %s:%d in %s", cudaGetErrorName(e), cudaGetErrorString(e), file,
             line, what);
    g_last_error = buf;
    if (!quiet()) fprintf(stderr, "tags_gpu: %s\n", buf);
    return TAGS_E_CUDA;
}

int tags_fail(int code, const char* msg) {
    g_last_error = msg;
    if (!quiet()) fprintf(stderr, "tags_gpu: %s\n", msg);
    return code;
}

void tags_msg(const char* msg) {
    if (!quiet()) fputs(msg, stdout);
}

// ---- per-device context ------------------------------------------------------

DeviceCtx* tags_ctx() {
    static DeviceCtx ctxs[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    DeviceCtx& c = ctxs[dev];
    if (!c.ready) {
        if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        if (tags_fill_tables_init() != 0) return nullptr;
        if (cudaMalloc(&c.status, sizeof(int) * 4) != cudaSuccess) return nullptr;
        c.device = dev;
        c.ready = true;
    }
    return &c;
}

// Grow-only device scratch owned by the context.
void* DeviceCtx::scratch(int slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (scratch_bytes[slot] < bytes) {
        if (scratch_ptr[slot]) cudaFree(scratch_ptr[slot]);
        scratch_ptr[slot] = nullptr;
        scratch_bytes[slot] = 0;
        if (cudaMalloc(&scratch_ptr[slot], bytes) != cudaSuccess) return nullptr;
        scratch_bytes[slot] = bytes;
    }
    return scratch_ptr[slot];
}

SampleCoef tags_sample_coef(zd gamma, zd s, double mur, zd kappa, zd ref_l, zd ref_t) {
    // src/electrode.c:317-318 and :397-398
    zd cL = s * mur * TAGS_MU0 / TAGS_FOUR_PI;
    zd cT = 1.0 / (TAGS_FOUR_PI * kappa);
    zd cLi = ref_l * s * mur * TAGS_MU0 / TAGS_FOUR_PI;
    zd cTi = ref_t / (TAGS_FOUR_PI * kappa);
    SampleCoef c;
    c.gamma = make_double2(gamma.real(), gamma.imag());
    c.cL = make_double2(cL.real(), cL.imag());
    c.cT = make_double2(cT.real(), cT.imag());
    c.cLi = make_double2(cLi.real(), cLi.imag());
    c.cTi = make_double2(cTi.real(), cTi.imag());
    return c;
}

static inline zd Z(tags_cdouble v) { return zd(v.re, v.im); }

// ---- drop-in: impedance fill ---------------------------------------------------

// Computes the lower triangle of the direct (mode DIRECT) or image (mode
// IMAGE) contributions into host arrays hl, ht (m*m, column-major).
static int fill_to_host(const Electrode* elec, const Electrode* img, size_t m, const SampleCoef& coef, int mode,
                        int itype, std::vector<zd>& hl, std::vector<zd>& ht) {
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    const size_t mm = m * m;
    double* d_elec = (double*)c->scratch(0, sizeof(Electrode) * m * 2);
    double2* d_z = (double2*)c->scratch(1, sizeof(double2) * mm * 2);
    SampleCoef* d_coef = (SampleCoef*)c->scratch(2, sizeof(SampleCoef));
    if (!d_elec || !d_z || !d_coef) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    double* d_img = d_elec + 11 * m;
    cudaStream_t st = c->stream;
    TAGS_CUDA_OK(cudaMemcpyAsync(d_elec, elec, sizeof(Electrode) * m, cudaMemcpyHostToDevice, st));
    if (img) TAGS_CUDA_OK(cudaMemcpyAsync(d_img, img, sizeof(Electrode) * m, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_coef, &coef, sizeof(SampleCoef), cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemsetAsync(c->status, 0, sizeof(int), st));
    FillOut out{};
    out.zl = d_z;
    out.zt = d_z + mm;
    out.ld = (long long)m;
    out.batch_stride = 0;
    out.sign = 1.0;
    int err = tags_launch_fill_fp64(d_elec, img ? d_img : d_elec, (int)m, d_coef, 1, out, mode, itype, 1, c->status, st);
    if (err) return err;
    hl.resize(mm);
    ht.resize(mm);
    int status = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(hl.data(), d_z, sizeof(double2) * mm, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(ht.data(), d_z + mm, sizeof(double2) * mm, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (status & TAGS_ST_DEGENERATE_PAIR)
        return tags_fail(TAGS_E_GEOMETRY, "coincident or overlapping segments: the pair integral diverges");
    return 0;
}

extern "C" int calculate_impedances(tags_cdouble* zl, tags_cdouble* zt, const Electrode* electrodes,
                                    size_t num_electrodes, tags_cdouble gamma, tags_cdouble s, double mur,
                                    tags_cdouble kappa, size_t max_eval, double req_abs_error, double req_rel_error,
                                    int integration_type) {
    (void)max_eval; (void)req_abs_error; (void)req_rel_error;
    std::lock_guard<std::mutex> lk(g_mutex);
    const size_t m = num_electrodes;
    if (m == 0) return 0;
    if (!zl || !zt || !electrodes) return tags_fail(TAGS_E_ARG, "null pointer argument");
    const bool known = integration_type >= 1 && integration_type <= 4;
    SampleCoef coef = tags_sample_coef(Z(gamma), Z(s), mur, Z(kappa), 1.0, 1.0);
    if (!known) {
        // The reference writes the first diagonal entry, then its integral()
        // fails with -10 on the first off-diagonal pair (src/electrode.c:346-363).
        const Electrode& e = electrodes[0];
        double k1 = e.radius / e.length, k2 = sqrt(1.0 + k1 * k1);
        double intg = 2.0 * e.length * (log((k2 + 1.0) / k1) - k2 + k1);
        zd l = zd(coef.cL.x, coef.cL.y) * intg, t = zd(coef.cT.x, coef.cT.y) / (e.length * e.length) * intg;
        zl[0] = {l.real(), l.imag()};
        zt[0] = {t.real(), t.imag()};
        if (m > 1) {
            char msg[64];
            snprintf(msg, sizeof(msg), "integration failed with code: %i\n", -10);
            tags_msg(msg);
            return -10;
        }
        return 0;
    }
    std::vector<zd> hl, ht;
    int err = fill_to_host(electrodes, nullptr, m, coef, TAGS_FILL_DIRECT, integration_type, hl, ht);
    if (err) return err;
    // write order of the reference: diagonal zl then zt; off-diagonal zt then zl
    for (size_t i = 0; i < m; ++i) {
        for (size_t k = i; k < m; ++k) {
            size_t idx = i * m + k;
            if (k == i) {
                zl[idx] = {hl[idx].real(), hl[idx].imag()};
                zt[idx] = {ht[idx].real(), ht[idx].imag()};
            } else {
                zt[idx] = {ht[idx].real(), ht[idx].imag()};
                zl[idx] = {hl[idx].real(), hl[idx].imag()};
            }
        }
    }
    return 0;
}

extern "C" int impedances_images(tags_cdouble* zl, tags_cdouble* zt, const Electrode* electrodes,
                                 const Electrode* images, size_t num_electrodes, tags_cdouble gamma, tags_cdouble s,
                                 double mur, tags_cdouble kappa, tags_cdouble ref_l, tags_cdouble ref_t,
                                 size_t max_eval, double req_abs_error, double req_rel_error, int integration_type) {
    (void)max_eval; (void)req_abs_error; (void)req_rel_error;
    std::lock_guard<std::mutex> lk(g_mutex);
    const size_t m = num_electrodes;
    if (m == 0) return 0;
    if (!zl || !zt || !electrodes || !images) return tags_fail(TAGS_E_ARG, "null pointer argument");
    if (!(integration_type >= 1 && integration_type <= 4)) {
        char msg[64];
        snprintf(msg, sizeof(msg), "integration failed with code: %i\n", -10);
        tags_msg(msg);
        return -10;
    }
    SampleCoef coef = tags_sample_coef(Z(gamma), Z(s), mur, Z(kappa), Z(ref_l), Z(ref_t));
    std::vector<zd> hl, ht;
    int err = fill_to_host(electrodes, images, m, coef, TAGS_FILL_IMAGE, integration_type, hl, ht);
    if (err) return err;
    for (size_t i = 0; i < m; ++i) {
        for (size_t k = i; k < m; ++k) {
            size_t idx = i * m + k;
            // zt += first, then zl += (the image ZL term is zero when cos <= eps)
            zd t = Z(zt[idx]) + ht[idx];
            zt[idx] = {t.real(), t.imag()};
            zd l = Z(zl[idx]) + hl[idx];
            zl[idx] = {l.real(), l.imag()};
        }
    }
    return 0;
}

// ---- drop-in: immittance assembly ---------------------------------------------

extern "C" int fill_incidence_imm(tags_cdouble* wg, const Electrode* electrodes, size_t num_electrodes,
                                  const double* nodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(g_mutex);
    const size_t m = num_electrodes, n = num_nodes, ld = 2 * m + n;
    if (n == 0) return 0;
    if (!wg || !electrodes || !nodes) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    double* d_elec = (double*)c->scratch(0, sizeof(Electrode) * (m ? m : 1));
    double* d_nodes = (double*)c->scratch(2, sizeof(double) * 3 * n);
    signed char* d_cond = (signed char*)c->scratch(1, n * m + 1);
    if (!d_elec || !d_nodes || !d_cond) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    cudaStream_t st = c->stream;
    std::vector<signed char> cond(n * m);
    if (m) {
        TAGS_CUDA_OK(cudaMemcpyAsync(d_elec, electrodes, sizeof(Electrode) * m, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_nodes, nodes, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        int err = tags_incidence_codes(d_elec, (int)m, d_nodes, (int)n, d_cond, st);
        if (err) return err;
        TAGS_CUDA_OK(cudaMemcpyAsync(cond.data(), d_cond, n * m, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    // write in the reference's order, stopping after the first node without
    // incidence (src/linalg.c:29-76)
    long long suma = 0;
    double sumb = 0.0;
    for (size_t nd = 0; nd < n; ++nd) {
        bool none = true;
        for (size_t e = 0; e < m; ++e) {
            int cd = cond[nd * m + e];
            double av = cd == 1 ? 1.0 : (cd == 2 ? -1.0 : 0.0), bv = cd ? 0.5 : 0.0;
            wg[(e + n) + ld * nd] = {av, 0.0};
            wg[(e + n + m) + ld * nd] = {bv, 0.0};
            wg[nd + ld * (e + n)] = {av, 0.0};
            wg[nd + ld * (e + n + m)] = {bv, 0.0};
            suma += (long long)av;
            sumb += bv;
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

extern "C" int fill_impedance_imm(tags_cdouble* wg, const tags_cdouble* zl, const tags_cdouble* zt,
                                  size_t num_electrodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(g_mutex);
    const size_t m = num_electrodes, n = num_nodes, N = n + 2 * m;
    if (N == 0) return 0;
    if (!wg || (m && (!zl || !zt))) return tags_fail(TAGS_E_ARG, "null pointer argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    // Device image of the written region: rows/cols [0,n) (Y_E) and [n,N)
    // (impedance blocks), laid out with leading dimension N like W_G.
    double2* d_z = (double2*)c->scratch(1, sizeof(double2) * (2 * m * m + 1));
    double2* d_W = (double2*)c->scratch(3, sizeof(double2) * N * N);
    if (!d_z || !d_W) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    if (m) {
        TAGS_CUDA_OK(cudaMemcpyAsync(d_z, zl, sizeof(double2) * m * m, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_z + m * m, zt, sizeof(double2) * m * m, cudaMemcpyHostToDevice, st));
    }
    int err = tags_wg_impedance(d_W, (long long)N, d_z, d_z + m * m, (int)m, (int)n, st);
    if (err) return err;
    const size_t pitch = sizeof(double2) * N;
    // Y_E block: rows 0..n, cols 0..n
    if (n)
        TAGS_CUDA_OK(cudaMemcpy2DAsync(wg, pitch, d_W, pitch, sizeof(double2) * n, n, cudaMemcpyDeviceToHost, st));
    // impedance blocks: rows n..N, cols n..N
    if (m)
        TAGS_CUDA_OK(cudaMemcpy2DAsync(wg + n + N * n, pitch, d_W + n + N * n, pitch, sizeof(double2) * 2 * m, 2 * m,
                                       cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

// ---- drop-in: solve -------------------------------------------------------------

extern "C" int solve_immittance(tags_cdouble* wg, tags_cdouble* ie, size_t num_electrodes, size_t num_nodes) {
    std::lock_guard<std::mutex> lk(g_mutex);
    const size_t N = 2 * num_electrodes + num_nodes;
    if (N == 0) return 0;
    if (!wg || !ie) return tags_fail(TAGS_E_ARG, "null pointer argument");
    if (N > 200000) return tags_fail(TAGS_E_ARG, "system too large");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    double2* d_W = (double2*)c->scratch(3, sizeof(double2) * N * N);
    double2* d_x = (double2*)c->scratch(4, sizeof(double2) * N);
    int* d_ipiv = (int*)c->scratch(5, sizeof(int) * (N + 1));
    if (!d_W || !d_x || !d_ipiv) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    TAGS_CUDA_OK(cudaMemcpyAsync(d_W, wg, sizeof(double2) * N * N, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_x, ie, sizeof(double2) * N, cudaMemcpyHostToDevice, st));
    int err = tags_symmetrize_lower(d_W, (int)N, (long long)N, 0, 1, st);
    if (err) return err;
    err = tags_lu_z(d_W, (int)N, (long long)N, 0, 1, 1, d_ipiv, d_ipiv + N, st);
    if (err) return err;
    int info = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(&info, d_ipiv + N, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    if (info > 0) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "The diagonal element of the triangular factor of YN,\nU(%i,%i) is zero, so that YN is singular;\n"
                 "the solution could not be computed.\n",
                 info, info);
        tags_msg(msg);
        return info;
    }
    err = tags_lu_solve_z(d_W, (int)N, (long long)N, 0, 1, d_ipiv, d_x, 1, (long long)N, 0, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaMemcpyAsync(ie, d_x, sizeof(double2) * N, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

// ---- drop-in: numerical Laplace transform pair -----------------------------------

extern "C" int laplace_trans(double* f, tags_cdouble* g, tags_cdouble* s, double tmax, size_t nt) {
    std::lock_guard<std::mutex> lk(g_mutex);
    if (nt < 2 || !f || !g || !s) return tags_fail(TAGS_E_ARG, "invalid argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    const size_t ns = nt / 2 + 1;
    double2* d_tw = (double2*)c->scratch(6, sizeof(double2) * nt);
    double* d_f = (double*)c->scratch(7, sizeof(double) * nt);
    double2* d_g = (double2*)c->scratch(8, sizeof(double2) * ns);
    if (!d_tw || !d_f || !d_g) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    // s_k = c + j k dw (src/auxiliary.c:247-252)
    double cc = log(pow((double)nt, 2.0)) / tmax, dw = TAGS_TWO_PI / tmax;
    for (size_t k = 0; k < ns; ++k) s[k] = {cc, dw * (double)k};
    TAGS_CUDA_OK(cudaMemcpyAsync(d_f, f, sizeof(double) * nt, cudaMemcpyHostToDevice, st));
    int err = tags_twiddles(d_tw, (long long)nt, st);
    if (!err) err = tags_launch_nlt(d_f, 0, (long long)nt, d_tw, tmax, d_g, 0, 1, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaMemcpyAsync(g, d_g, sizeof(double2) * ns, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int inv_laplace_trans(double* f, tags_cdouble* g, tags_cdouble* s, double tmax, size_t nt, int filter) {
    std::lock_guard<std::mutex> lk(g_mutex);
    if (nt < 2 || !f || !g || !s) return tags_fail(TAGS_E_ARG, "invalid argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    const size_t ns = nt / 2 + 1;
    double2* d_tw = (double2*)c->scratch(6, sizeof(double2) * nt);
    double* d_f = (double*)c->scratch(7, sizeof(double) * nt);
    double2* d_g = (double2*)c->scratch(8, sizeof(double2) * ns * 2);
    if (!d_tw || !d_f || !d_g) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    TAGS_CUDA_OK(cudaMemcpyAsync(d_g, g, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_g + ns, s, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
    int err = tags_twiddles(d_tw, (long long)nt, st);
    if (!err)
        err = tags_launch_inlt(d_g, 0, (long long)ns, d_g + ns, d_tw, (long long)nt, tmax,
                               (filter >= 1 && filter <= 4) ? filter : 0, d_f, 0, 1, st);
    if (err) return err;
    TAGS_CUDA_OK(cudaMemcpyAsync(f, d_f, sizeof(double) * nt, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

// Batched inverse over many series in the examples' layout (no counterpart
// function in the reference; it replaces the examples' fftw_plan_many_dft_c2r
// and the scaling loop, examples/three_grids.c:229-242 and :447-465).
extern "C" int tags_inv_laplace_batch(double* f, const tags_cdouble* g, const tags_cdouble* s, double tmax, size_t nt,
                                      size_t nseries, int filter, int flags) {
    std::lock_guard<std::mutex> lk(g_mutex);
    TagsRange range("tags INLT");
    if (nt < 2 || nseries == 0 || !f || !g || !s) return tags_fail(TAGS_E_ARG, "invalid argument");
    if (nt > (size_t)1 << 26 || nseries > (size_t)1 << 26) return tags_fail(TAGS_E_ARG, "transform too large");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    const bool dev = (flags & TAGS_RUN_DEVICE_PTRS) != 0;
    const size_t ns = nt / 2 + 1;
    double2* d_tw = (double2*)c->scratch(6, sizeof(double2) * (nt + ns));
    if (!d_tw) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    double2* d_s = d_tw + nt;
    const double2* d_g = reinterpret_cast<const double2*>(g);
    double* d_f = f;
    if (!dev) {
        double2* dg = (double2*)c->scratch(8, sizeof(double2) * ns * nseries);
        d_f = (double*)c->scratch(7, sizeof(double) * nt * nseries);
        if (!dg || !d_f) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
        TAGS_CUDA_OK(cudaMemcpyAsync(dg, g, sizeof(double2) * ns * nseries, cudaMemcpyHostToDevice, st));
        d_g = dg;
    }
    TAGS_CUDA_OK(cudaMemcpyAsync(d_s, s, sizeof(double2) * ns, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                 st));
    int err = tags_twiddles(d_tw, (long long)nt, st);
    if (!err)
        err = tags_launch_inlt_rows(d_g, (long long)ns, d_s, d_tw, (long long)nt, tmax,
                                    (filter >= 1 && filter <= 4) ? filter : 0, d_f, (long long)nseries, st);
    if (err) return err;
    if (!dev) TAGS_CUDA_OK(cudaMemcpyAsync(f, d_f, sizeof(double) * nt * nseries, cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return 0;
}

// ---- library info ------------------------------------------------------------------

extern "C" long long tags_gpu_launch_count(void) { return g_launches.load(); }
extern "C" const char* tags_gpu_last_error(void) { return g_last_error.c_str(); }
extern "C" void tags_gpu_set_quiet(int q) { g_quiet.store(q ? 1 : 0); }

namespace {
std::atomic<unsigned long long> g_mem_budget{0};     // 0: no cap
}

extern "C" int tags_gpu_set_memory_budget(unsigned long long bytes) {
    g_mem_budget.store(bytes);
    return 0;
}

bool tags_all_finite(const void* v, size_t n) {
    if (!v) return true;
    const double* d = static_cast<const double*>(v);
    for (size_t i = 0; i < 2 * n; ++i)
        if (!std::isfinite(d[i])) return false;
    return true;
}

// Free device memory as the plans and grid batches size themselves against:
// cudaMemGetInfo's figure, capped by tags_gpu_set_memory_budget.
cudaError_t tags_free_memory(size_t* freeb) {
    size_t tot = 0;
    const cudaError_t e = cudaMemGetInfo(freeb, &tot);
    const unsigned long long cap = g_mem_budget.load();
    if (e == cudaSuccess && cap && *freeb > cap) *freeb = (size_t)cap;
    return e;
}
