// Tensor-core LDL^T factorisation of the mixed form's working matrix.
//
// The reordered, scaled immittance matrix W'' (complex, symmetric,
// non-Hermitian) is factorised without pivoting as W'' = L D L^T in 128-column
// panels (right-looking, lower triangle only):
//   1. k_ldl_diag    : 128 x 128 diagonal block -> L11 (unit lower), D1, and
//                      the explicit inverse L11^{-1} (one CTA per sample, in
//                      shared memory, complex FP32);
//   2. k_panel_planes: the block column A21 below it -> bf16 split planes;
//   3. k_gemm_tc     : W21 = A21 L11^{-T} (the triangular solve as a GEMM),
//                      L21 = W21 D1^{-1}, both written as split planes;
//   4. k_gemm_tc     : A22 -= L21 W21^T on the lower 128 x 128 tiles.
// The GEMMs run on the 5th-generation tensor cores: operands are staged in
// shared memory by TMA (128-byte swizzle), tcgen05.mma (kind::f16, bf16 in,
// FP32 accumulate) is issued by one thread, the two accumulators (real and
// imaginary part, 128 x 128 FP32 each) live in tensor memory and are read
// back with tcgen05.ld. A complex product is four real products; each real
// operand is split into bf16 hi + lo, and hi*hi + hi*lo + lo*hi keeps about
// 16 significant bits, so twelve tcgen05.mma per K step.
// Every mbarrier wait has an iteration limit; on expiry the kernel raises an
// error flag, lets its copies in flight land, frees its tensor memory and
// returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

namespace {

constexpr int TB = 128;                 // panel width and tile edge
constexpr int PLANE_BYTES = TB * TB * 2;        // one bf16 plane of a 128 x 128 tile: 32 KiB
constexpr int KBLK_BYTES = TB * 64 * 2;         // 64-wide K block of a plane: 16 KiB
constexpr int GEMM_SMEM = 6 * PLANE_BYTES + 1024 + 256;   // 4 A planes + 2 B slots + align + barriers
constexpr uint64_t WAIT_NS = 50ull * 1000 * 1000;   // 50 ms per wait

// ---- PTX wrappers ----------------------------------------------------------------

TAGS_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

TAGS_D void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
TAGS_D void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
TAGS_D uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase with parity `parity` of the mbarrier at `bar`, bounded by
// WAIT_NS of wall time; gives up early once any CTA raised `err`. Returns
// false (and raises `err`) when the bound ran out.
TAGS_D bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
    const uint64_t t0 = globaltimer_ns();
    for (unsigned it = 0;; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & 255) == 255) {
            if (*(volatile int*)err != 0) return false;
            if (globaltimer_ns() - t0 > WAIT_NS) {
                atomicOr(err, 8);
                return false;
            }
        }
    }
}
TAGS_D void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
TAGS_D void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
TAGS_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
TAGS_D void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
TAGS_D void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
TAGS_D void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
TAGS_D void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
TAGS_D void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
TAGS_D uint64_t sdesc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
    d |= (uint64_t)1 << 46;                    // version
    d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
    return d;
}
// Instruction descriptor: kind::f16, bf16 x bf16 -> f32, M = N = 128, K-major.
TAGS_D uint32_t idesc_bf16(bool negate_a) {
    uint32_t d = 0;
    d |= 1u << 4;                   // D format f32
    d |= 1u << 7;                   // A bf16
    d |= 1u << 10;                  // B bf16
    d |= (negate_a ? 1u : 0u) << 13;
    d |= (uint32_t)(TB >> 3) << 17; // N
    d |= (uint32_t)(TB >> 4) << 24; // M
    return d;
}

TAGS_D void split_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& lo) {
    hi = __float2bfloat16_rn(x);
    lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}

}  // namespace

// ---- GEMM on the tensor cores ------------------------------------------------------

struct GemmArgs {
    int M, Nn;                 // valid rows / columns of the output
    int mode;                  // 0: C -= A B^T into the FP32 matrix; 1: panel output (L21, planes)
    int tri;                   // tiles enumerate the lower triangle (I >= J)
    float2* Amat;              // FP32 working matrices
    long long ld, mstride;
    int row0, col0;            // matrix coordinates of output element (0, 0)
    const float2* dinv;        // per sample 128 values (mode 1)
    __nv_bfloat16* Lp;         // planes written in mode 1: [sample][4][R][128]
    __nv_bfloat16* Wp;
    long long pstride;         // elements per sample of a plane buffer
    int R;                     // rows of a plane buffer
    int* err;
    int zlo, zhi;              // output rows/cols in [zlo, zhi) are structurally zero (skip tiles inside)
};

__global__ void __launch_bounds__(128, 1) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t base_u32 = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* base = smem_raw + (base_u32 - smem_u32(smem_raw));
    const uint32_t sA = base_u32;                         // 4 planes: r_hi, r_lo, i_hi, i_lo
    const uint32_t sB = base_u32 + 4 * PLANE_BYTES;       // 2 slots: real, imaginary
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + 6 * PLANE_BYTES);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(base + 6 * PLANE_BYTES + 64);
    const uint32_t barA = smem_u32(&bars[0]), barB = smem_u32(&bars[1]), barM1 = smem_u32(&bars[2]);
    const uint32_t barB2 = smem_u32(&bars[3]), barAcc = smem_u32(&bars[4]);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int smp = blockIdx.y;
    int I, J;
    if (g.tri) {
        int t = blockIdx.x;
        I = (int)((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
        while ((I + 1) * (I + 2) / 2 <= t) ++I;
        while (I * (I + 1) / 2 > t) --I;
        J = t - I * (I + 1) / 2;
    } else {
        I = blockIdx.x;
        J = 0;
    }
    // tiles that lie entirely in the structurally zero band have nothing to do
    if (g.zhi > g.zlo) {
        const bool row_zero = TB * I >= g.zlo && TB * I + TB <= g.zhi;
        const bool col_zero = g.mode == 0 && TB * J >= g.zlo && TB * J + TB <= g.zhi;
        if (row_zero || col_zero) return;
    }
    if (tid == 0) {
        for (int q = 0; q < 5; ++q) mbar_init(smem_u32(&bars[q]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), 256);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    bool ok = true;

    const int rowA = TB * I, rowB = TB * J;
    if (tid == 0) {
        mbar_expect_tx(barA, 4 * PLANE_BYTES);
        for (int p = 0; p < 4; ++p)
            for (int kb = 0; kb < 2; ++kb)
                tma_load_4d(sA + p * PLANE_BYTES + kb * KBLK_BYTES, &tmA, kb * 64, rowA, p, smp, barA);
        mbar_expect_tx(barB, 2 * PLANE_BYTES);
        for (int s = 0; s < 2; ++s)            // hi planes of B: real (0) and imaginary (2)
            for (int kb = 0; kb < 2; ++kb)
                tma_load_4d(sB + s * PLANE_BYTES + kb * KBLK_BYTES, &tmB, kb * 64, rowB, 2 * s, smp, barB);
    }
    const uint32_t accR = tmem, accI = tmem + 128;
    const uint32_t idp = idesc_bf16(false), idn = idesc_bf16(true);
    // one product over K = 128 (8 steps of 16): acc += sign * A_plane(pa) * B_slot(sb)^T
    auto product = [&](uint32_t acc, int pa, int sb, bool neg, bool first) {
        for (int kk = 0; kk < 8; ++kk) {
            uint32_t off = (kk >> 2) * KBLK_BYTES + (kk & 3) * 32;
            mma_bf16(acc, sdesc(sA + pa * PLANE_BYTES + off), sdesc(sB + sb * PLANE_BYTES + off), neg ? idn : idp,
                     (first && kk == 0) ? 0u : 1u);
        }
    };
    if (tid == 32) {
        ok = mbar_wait(barA, 0, g.err) && mbar_wait(barB, 0, g.err);
        if (ok) {
            tc_fence_after();
            // B slots hold the hi planes: slot 0 = Br_hi, slot 1 = Bi_hi
            product(accR, 0, 0, false, true);   // Ar_hi Br_hi
            product(accR, 1, 0, false, false);  // Ar_lo Br_hi
            product(accR, 2, 1, true, false);   // -Ai_hi Bi_hi
            product(accR, 3, 1, true, false);   // -Ai_lo Bi_hi
            product(accI, 0, 1, false, true);   // Ar_hi Bi_hi
            product(accI, 1, 1, false, false);  // Ar_lo Bi_hi
            product(accI, 2, 0, false, false);  // Ai_hi Br_hi
            product(accI, 3, 0, false, false);  // Ai_lo Br_hi
        }
        mma_commit(barM1);
    }
    if (tid == 0) {
        // the lo planes of B replace the hi planes once the first products are done
        if (mbar_wait(barM1, 0, g.err)) {
            mbar_expect_tx(barB2, 2 * PLANE_BYTES);
            for (int s = 0; s < 2; ++s)
                for (int kb = 0; kb < 2; ++kb)
                    tma_load_4d(sB + s * PLANE_BYTES + kb * KBLK_BYTES, &tmB, kb * 64, rowB, 2 * s + 1, smp, barB2);
        } else {
            ok = false;
            atomicOr(g.err, 1);
            mbar_expect_tx(barB2, 0);   // release the waiter below
        }
    }
    if (tid == 32) {
        bool ok2 = ok && mbar_wait(barB2, 0, g.err);
        if (ok2) {
            tc_fence_after();
            product(accR, 0, 0, false, false);  // Ar_hi Br_lo
            product(accR, 2, 1, true, false);   // -Ai_hi Bi_lo
            product(accI, 0, 1, false, false);  // Ar_hi Bi_lo
            product(accI, 2, 0, false, false);  // Ai_hi Br_lo
        } else {
            ok = false;
            atomicOr(g.err, 2);
        }
        mma_commit(barAcc);
    }
    // ---- epilogue: all four warps, warp w owns tensor-memory lanes 32w..32w+31
    bool acc_ok = mbar_wait(barAcc, 0, g.err);
    if (!acc_ok) {
        atomicOr(g.err, 4);
        // let the copies and products already issued land before tensor
        // memory and shared memory are released
        if (tid == 0) {
            const uint64_t t0 = globaltimer_ns();
            for (int q = 0; q < 5; ++q) {
                uint32_t okq = 0;
                while (!okq && globaltimer_ns() - t0 < WAIT_NS) {
                    asm volatile(
                        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                        : "=r"(okq)
                        : "r"(smem_u32(&bars[q])), "r"(0u)
                        : "memory");
                }
            }
        }
    }
    tc_fence_after();
    if (acc_ok) {
        const int r = 32 * warp + lane;          // row within the tile
        const int gr = TB * I + r;               // row within the output
        const uint32_t lane_off = (uint32_t)(32 * warp) << 16;
        for (int cc = 0; cc < TB / 16; ++cc) {
            float vr[16], vi[16];
            tmem_ld16(accR + lane_off + cc * 16, vr);
            tmem_ld16(accI + lane_off + cc * 16, vi);
            if (gr >= g.M) continue;
            if (g.mode == 0) {
                float2* Cb = g.Amat + g.mstride * smp;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int gc = TB * J + cc * 16 + j;
                    if (gc < g.Nn) {
                        float2* p = Cb + (long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + gc);
                        float2 v = *p;
                        v.x -= vr[j];
                        v.y -= vi[j];
                        *p = v;
                    }
                }
            } else {
                float2* Cb = g.Amat + g.mstride * smp;
                const float2* dv = g.dinv + (long long)TB * smp;
                __align__(16) __nv_bfloat16 lp[4][16], wp[4][16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int c = cc * 16 + j;
                    float2 w = make_float2(vr[j], vi[j]);
                    float2 d = dv[c];
                    float2 l = fmulc(w, d);
                    if (c < g.Nn) Cb[(long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + c)] = l;
                    split_bf16(l.x, lp[0][j], lp[1][j]);
                    split_bf16(l.y, lp[2][j], lp[3][j]);
                    split_bf16(w.x, wp[0][j], wp[1][j]);
                    split_bf16(w.y, wp[2][j], wp[3][j]);
                }
                const long long rowoff = (long long)gr * TB + cc * 16;
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    uint4* dl = reinterpret_cast<uint4*>(g.Lp + g.pstride * smp + (long long)p * g.R * TB + rowoff);
                    uint4* dw = reinterpret_cast<uint4*>(g.Wp + g.pstride * smp + (long long)p * g.R * TB + rowoff);
                    dl[0] = reinterpret_cast<const uint4*>(lp[p])[0];
                    dl[1] = reinterpret_cast<const uint4*>(lp[p])[1];
                    dw[0] = reinterpret_cast<const uint4*>(wp[p])[0];
                    dw[1] = reinterpret_cast<const uint4*>(wp[p])[1];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 256);
}

// ---- diagonal block: LDL^T, L11^{-1} -------------------------------------------------

// One CTA per sample. S (column-major 128 x 128 complex FP32) in shared memory.
__global__ void __launch_bounds__(512) k_ldl_diag(float2* __restrict__ A0, long long ld, long long mstride, int j0,
                                                  int jb, __nv_bfloat16* __restrict__ linv_planes,
                                                  float2* __restrict__ dinv, int* __restrict__ info,
                                                  float2* __restrict__ linv32, long long lstride) {
    extern __shared__ __align__(16) float2 S[];        // S[c * TB + r]
    __shared__ float2 colv[TB];
    const int smp = blockIdx.x, tid = threadIdx.x;
    float2* A = A0 + mstride * smp;
    for (int t = tid; t < TB * TB; t += blockDim.x) {
        int r = t % TB, c = t / TB;
        float2 v;
        if (r < jb && c < jb) {
            int rr = r >= c ? r : c, cc2 = r >= c ? c : r;     // lower triangle, mirrored
            v = A[(long long)(j0 + rr) + ld * (j0 + cc2)];
        } else {
            v = make_float2(r == c ? 1.f : 0.f, 0.f);
        }
        S[c * TB + r] = v;
    }
    __syncthreads();
    // right-looking LDL^T without pivoting on the lower triangle
    for (int k = 0; k < TB; ++k) {
        const float2 d = S[k * TB + k];
        if (tid == 0 && k < jb && !(d.x != 0.f || d.y != 0.f) && *(info + smp) == 0) info[smp] = j0 + k + 1;
        double2 dd = cdiv(make_double2(1.0, 0.0), make_double2(d.x, d.y));
        const float2 di = make_float2((float)dd.x, (float)dd.y);
        // column below the pivot: keep W = old values, L = W / d
        for (int i = k + 1 + tid; i < TB; i += blockDim.x) colv[i] = S[k * TB + i];
        __syncthreads();
        const int n = TB - k - 1;
        for (int t = tid; t < n * n; t += blockDim.x) {
            int i = k + 1 + t % n, j = k + 1 + t / n;
            if (i >= j) {
                // S_ij -= W_i W_j / d
                float2 li = fmulc(colv[i], di);
                S[j * TB + i] = fsub(S[j * TB + i], fmulc(li, colv[j]));
            }
        }
        for (int i = k + 1 + tid; i < TB; i += blockDim.x) S[k * TB + i] = fmulc(colv[i], di);
        __syncthreads();
    }
    // write L11 (unit lower) and D back; D^{-1} for the panel epilogue
    for (int t = tid; t < jb * jb; t += blockDim.x) {
        int r = t % jb, c = t / jb;
        if (r >= c) A[(long long)(j0 + r) + ld * (j0 + c)] = S[c * TB + r];
    }
    for (int c = tid; c < TB; c += blockDim.x) {
        float2 v = make_float2(0.f, 0.f);
        if (c < jb) {
            float2 d = S[c * TB + c];
            double2 dd = cdiv(make_double2(1.0, 0.0), make_double2(d.x, d.y));
            v = make_float2((float)dd.x, (float)dd.y);
        }
        dinv[(long long)TB * smp + c] = v;
    }
    __syncthreads();
    // in-place inverse of the unit lower L11: for j = 127..0,
    // X[j+1:, j] = -X[j+1:, j+1:] L[j+1:, j]
    for (int j = TB - 1; j >= 0; --j) {
        for (int i = j + 1 + tid; i < TB; i += blockDim.x) colv[i] = S[j * TB + i];
        __syncthreads();
        for (int i = j + 1 + tid; i < TB; i += blockDim.x) {
            float2 acc = colv[i];                       // X[i][i] = 1
            for (int k = j + 1; k < i; ++k) acc = ffmac(S[k * TB + i], colv[k], acc);
            S[j * TB + i] = make_float2(-acc.x, -acc.y);
        }
        __syncthreads();
    }
    // L11^{-1} kept in FP32 (row-major, zero outside jb) for the triangular solves
    float2* X32 = linv32 + lstride * smp + (long long)(j0 / TB) * TB * TB;
    for (int t = tid; t < TB * TB; t += blockDim.x) {
        int nrow = t / TB, k = t % TB;
        float2 v = make_float2(0.f, 0.f);
        if (nrow < jb && k < jb) {
            if (k == nrow) v = make_float2(1.f, 0.f);
            else if (k < nrow) v = S[k * TB + nrow];
        }
        X32[t] = v;
    }
    // L11^{-1} as split planes, row-major: B[n][k] = X[n][k] (k <= n), rows/cols >= jb zero
    __nv_bfloat16* P = linv_planes + (long long)smp * 4 * TB * TB;
    for (int t = tid; t < TB * TB; t += blockDim.x) {
        int nrow = t / TB, k = t % TB;
        float2 v = make_float2(0.f, 0.f);
        if (nrow < jb && k < jb) {
            if (k == nrow) v = make_float2(1.f, 0.f);
            else if (k < nrow) v = S[k * TB + nrow];
        }
        __nv_bfloat16 h, l;
        split_bf16(v.x, h, l);
        P[0 * TB * TB + t] = h;
        P[1 * TB * TB + t] = l;
        split_bf16(v.y, h, l);
        P[2 * TB * TB + t] = h;
        P[3 * TB * TB + t] = l;
    }
}

// A21 (rows j0+jb .. j0+jb+M, columns j0 .. j0+jb) -> split planes, row-major
// [sample][4][R][128], columns >= jb zero. Tile: 32 rows x 128 columns.
__global__ void __launch_bounds__(256) k_panel_planes(const float2* __restrict__ A0, long long ld, long long mstride,
                                                      int j0, int jb, int M, __nv_bfloat16* __restrict__ planes,
                                                      long long pstride, int R) {
    __shared__ float2 t[TB][33];
    const int smp = blockIdx.y, r0 = blockIdx.x * 32;
    const float2* A = A0 + mstride * smp;
    for (int q = threadIdx.x; q < 32 * TB; q += blockDim.x) {
        int rr = q % 32, c = q / 32;
        float2 v = make_float2(0.f, 0.f);
        if (r0 + rr < M && c < jb) v = A[(long long)(j0 + jb + r0 + rr) + ld * (j0 + c)];
        t[c][rr] = v;
    }
    __syncthreads();
    __nv_bfloat16* P = planes + pstride * smp;
    for (int q = threadIdx.x; q < 32 * TB; q += blockDim.x) {
        int c = q % TB, rr = q / TB;
        if (r0 + rr >= M) continue;
        float2 v = t[c][rr];
        __nv_bfloat16 h, l;
        long long o = (long long)(r0 + rr) * TB + c;
        split_bf16(v.x, h, l);
        P[o] = h;
        P[(long long)R * TB + o] = l;
        split_bf16(v.y, h, l);
        P[2LL * R * TB + o] = h;
        P[3LL * R * TB + o] = l;
    }
}

// ---- solves with the factors: L D L^T x = b (one right-hand side per sample) ----------

// z_b = Linv_b * r_b for block b (128 rows); one CTA of 128 threads per sample.
// transpose = 1 applies Linv_b^T instead.
__global__ void __launch_bounds__(128) k_blk_inv_apply(const float2* __restrict__ linv32, long long lstride, int blk,
                                                       int jb, float2* __restrict__ x0, long long xstride,
                                                       int transpose) {
    __shared__ float2 v[TB];
    const int smp = blockIdx.x, r = threadIdx.x;
    float2* x = x0 + xstride * smp + (long long)blk * TB;
    const float2* Li = linv32 + lstride * smp + (long long)blk * TB * TB;
    v[r] = r < jb ? x[r] : make_float2(0.f, 0.f);
    __syncthreads();
    float2 acc = make_float2(0.f, 0.f);
    if (!transpose) {
        for (int k = 0; k <= r; ++k) acc = ffmac(Li[r * TB + k], v[k], acc);
    } else {
        for (int k = r; k < TB; ++k) acc = ffmac(Li[k * TB + r], v[k], acc);
    }
    if (r < jb) x[r] = acc;
}

// forward: x[i] -= sum_{k in block} L[i][k] x[k] for rows i below the block
__global__ void k_blk_fwd_update(const float2* __restrict__ A0, long long ld, long long mstride, int N, int j0, int jb,
                                 float2* __restrict__ x0, long long xstride, int zl_m) {
    const int smp = blockIdx.y;
    const int i = j0 + jb + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (j0 + jb <= zl_m && i >= zl_m && i < 2 * zl_m) return;      // L[ZT rows, ZL cols] = 0
    const float2* A = A0 + mstride * smp;
    float2* x = x0 + xstride * smp;
    float2 acc = make_float2(0.f, 0.f);
    for (int k = 0; k < jb; ++k) acc = ffmac(A[i + ld * (long long)(j0 + k)], x[j0 + k], acc);
    x[i] = fsub(x[i], acc);
}

// backward (L^T): x[r] -= sum_{c in block} L[c][r] x[c] for rows r above the block
__global__ void k_blk_bwd_update(const float2* __restrict__ A0, long long ld, long long mstride, int j0, int jb,
                                 float2* __restrict__ x0, long long xstride, int zl_m) {
    const int smp = blockIdx.y;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= j0) return;
    if (j0 >= zl_m && j0 + jb <= 2 * zl_m && r < zl_m) return;       // L[ZT rows, ZL cols] = 0
    const float2* A = A0 + mstride * smp;
    float2* x = x0 + xstride * smp;
    float2 acc = make_float2(0.f, 0.f);
    const float2* col = A + ld * (long long)r;
    for (int c = 0; c < jb; ++c) acc = ffmac(col[j0 + c], x[j0 + c], acc);
    x[r] = fsub(x[r], acc);
}

// x[i] /= D[i] (D on the diagonal of the factored matrix)
__global__ void k_diag_scale(const float2* __restrict__ A0, long long ld, long long mstride, int N,
                             float2* __restrict__ x0, long long xstride) {
    const int smp = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    float2 d = A0[mstride * smp + i + ld * (long long)i];
    double2 q = cdiv(make_double2(x0[xstride * smp + i].x, x0[xstride * smp + i].y), make_double2(d.x, d.y));
    x0[xstride * smp + i] = make_float2((float)q.x, (float)q.y);
}

// ---- host side ---------------------------------------------------------------------

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 4-D map over planes [sample][4][rows][128] bf16, box {64, 128, 1, 1}.
int make_plane_map(CUtensorMap* map, void* base, int rows, int samples) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return tags_fail(TAGS_E_CUDA, "cuTensorMapEncodeTiled is not available");
    cuuint64_t dims[4] = {(cuuint64_t)TB, (cuuint64_t)rows, 4, (cuuint64_t)samples};
    cuuint64_t strides[3] = {(cuuint64_t)TB * 2, (cuuint64_t)TB * 2 * rows, (cuuint64_t)TB * 2 * rows * 4};
    cuuint32_t box[4] = {64, (cuuint32_t)TB, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char msg[96];
        snprintf(msg, sizeof(msg), "cuTensorMapEncodeTiled failed (%d)", (int)r);
        return tags_fail(TAGS_E_CUDA, msg);
    }
    return 0;
}

}  // namespace

static long long linv32_stride(int N) { return (long long)((N + TB - 1) / TB) * TB * TB; }

size_t tags_ldl_tc_workspace(int N, int batch) {
    // A21 planes, L planes, W planes (R = N rows each), L11^{-1} planes, D^{-1},
    // FP32 inverses of all diagonal blocks
    size_t plane = (size_t)4 * N * TB * 2;
    return (size_t)batch * (3 * plane + (size_t)4 * TB * TB * 2 + TB * sizeof(float2) +
                            (size_t)linv32_stride(N) * sizeof(float2)) + 1024;
}

static float2* linv32_of(void* ws, int N, int batch_cap) {
    const long long pstride = (long long)4 * N * TB;
    __nv_bfloat16* Lin = reinterpret_cast<__nv_bfloat16*>(ws) + 3 * pstride * batch_cap;
    float2* dinv = reinterpret_cast<float2*>(Lin + (long long)4 * TB * TB * batch_cap);
    return dinv + (long long)TB * batch_cap;
}

int tags_ldl_solve_c(const float2* A, int N, long long ld, long long mstride, int nb, int batch_cap, void* ws,
                     float2* x, long long xstride, int zl_m, cudaStream_t st) {
    const float2* L32 = linv32_of(ws, N, batch_cap);
    const long long ls = linv32_stride(N);
    const int nblk = (N + TB - 1) / TB;
    int pf = tags_prof_begin(TAGS_PROF_LDL_SOLVE, st);
    for (int b = 0; b < nblk; ++b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        k_blk_inv_apply<<<nb, TB, 0, st>>>(L32, ls, b, jb, x, xstride, 0);
        const int rest = N - j0 - jb;
        if (rest > 0) k_blk_fwd_update<<<dim3((rest + 127) / 128, nb), 128, 0, st>>>(A, ld, mstride, N, j0, jb, x, xstride, zl_m);
        tags_note_launch(rest > 0 ? 2 : 1);
    }
    k_diag_scale<<<dim3((N + 255) / 256, nb), 256, 0, st>>>(A, ld, mstride, N, x, xstride);
    tags_note_launch();
    for (int b = nblk - 1; b >= 0; --b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        k_blk_inv_apply<<<nb, TB, 0, st>>>(L32, ls, b, jb, x, xstride, 1);
        if (j0 > 0) k_blk_bwd_update<<<dim3((j0 + 127) / 128, nb), 128, 0, st>>>(A, ld, mstride, j0, jb, x, xstride, zl_m);
        tags_note_launch(j0 > 0 ? 2 : 1);
    }
    // two triangular sweeps over the factor: 8 N^2 real flops, 8 N^2 bytes read
    tags_prof_end(TAGS_PROF_LDL_SOLVE, pf, st, 8.0 * N * (double)N * nb, 8.0 * N * (double)N * nb);
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// LDL^T of `nb` matrices A (N x N complex FP32, column-major, lower triangle
// used) in place: L strictly below the diagonal, D on it.
int tags_ldl_tc(float2* A, int N, long long ld, long long mstride, int nb, int batch_cap, void* ws, int* info,
                int* err, int zl_m, cudaStream_t st) {
    static bool attr_done = false;
    if (!attr_done) {
        TAGS_CUDA_OK(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
        TAGS_CUDA_OK(cudaFuncSetAttribute(k_ldl_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)(TB * TB * sizeof(float2))));
        attr_done = true;
    }
    const long long pstride = (long long)4 * N * TB;
    __nv_bfloat16* A21p = reinterpret_cast<__nv_bfloat16*>(ws);
    __nv_bfloat16* Lp = A21p + pstride * batch_cap;
    __nv_bfloat16* Wp = Lp + pstride * batch_cap;
    __nv_bfloat16* Lin = Wp + pstride * batch_cap;
    float2* dinv = reinterpret_cast<float2*>(Lin + (long long)4 * TB * TB * batch_cap);
    float2* L32 = linv32_of(ws, N, batch_cap);
    const long long ls = linv32_stride(N);
    CUtensorMap mA21, mL, mW, mLin;
    int e = make_plane_map(&mA21, A21p, N, batch_cap);
    if (!e) e = make_plane_map(&mL, Lp, N, batch_cap);
    if (!e) e = make_plane_map(&mW, Wp, N, batch_cap);
    if (!e) e = make_plane_map(&mLin, Lin, TB, batch_cap);
    if (e) return e;
    TAGS_CUDA_OK(cudaMemsetAsync(info, 0, sizeof(int) * nb, st));
    for (int j0 = 0; j0 < N; j0 += TB) {
        const int jb = N - j0 < TB ? N - j0 : TB;
        const int rest = N - j0 - jb;
        int pf = tags_prof_begin(TAGS_PROF_LDL_DIAG, st);
        k_ldl_diag<<<nb, 512, TB * TB * sizeof(float2), st>>>(A, ld, mstride, j0, jb, Lin, dinv, info, L32, ls);
        tags_prof_end(TAGS_PROF_LDL_DIAG, pf, st, 4.0 / 3.0 * jb * (double)jb * jb * nb, 16.0 * jb * jb * nb);
        tags_note_launch();
        if (rest <= 0) break;
        k_panel_planes<<<dim3((rest + 31) / 32, nb), 256, 0, st>>>(A, ld, mstride, j0, jb, rest, A21p, pstride, N);
        tags_note_launch();
        const int T = (rest + TB - 1) / TB;
        GemmArgs g{};
        // While the first zl_m columns (the ZL block of the ordering ZL, ZT,
        // nodes) are eliminated, the rows/columns zl_m .. 2 zl_m (ZT) of the
        // block column and of the trailing matrix stay exactly zero.
        if (zl_m > 0 && j0 + jb <= zl_m) {
            g.zlo = zl_m - (j0 + jb);
            g.zhi = 2 * zl_m - (j0 + jb);
        }
        g.M = rest;
        g.Nn = jb;
        g.mode = 1;
        g.tri = 0;
        g.Amat = A;
        g.ld = ld;
        g.mstride = mstride;
        g.row0 = j0 + jb;
        g.col0 = j0;
        g.dinv = dinv;
        g.Lp = Lp;
        g.Wp = Wp;
        g.pstride = pstride;
        g.R = N;
        g.err = err;
        pf = tags_prof_begin(TAGS_PROF_LDL_PANEL, st);
        k_gemm_tc<<<dim3(T, nb), 128, GEMM_SMEM, st>>>(mA21, mLin, g);
        // triangular solve: rest x jb unknowns against jb x jb, 4 rest jb^2 real flops
        tags_prof_end(TAGS_PROF_LDL_PANEL, pf, st, 4.0 * rest * (double)jb * jb * nb,
                      (8.0 * rest * jb + 16.0 * rest * 128 * 2) * nb);
        tags_note_launch();
        g.mode = 0;
        g.tri = 1;
        g.Nn = rest;
        g.row0 = j0 + jb;
        g.col0 = j0 + jb;
        pf = tags_prof_begin(TAGS_PROF_LDL_TRAIL, st);
        k_gemm_tc<<<dim3(T * (T + 1) / 2, nb), 128, GEMM_SMEM, st>>>(mL, mW, g);
        // symmetric rank-jb update of the lower triangle: 8 jb rest(rest+1)/2 real flops;
        // bytes: read + write of that triangle in complex FP32, two panels of split planes
        tags_prof_end(TAGS_PROF_LDL_TRAIL, pf, st, 8.0 * jb * (0.5 * rest * (rest + 1.0)) * nb,
                      (16.0 * 0.5 * rest * (rest + 1.0) + 2.0 * rest * 128 * 8) * nb);
        tags_note_launch();
    }
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// ---- diagnostic entry point (declared in include/tags_gpu.h) ------------------------

extern "C" int tags_debug_ldl(tags_cdouble* a, int N, int nb) {
    if (!a || N <= 0 || nb <= 0) return tags_fail(TAGS_E_ARG, "tags_debug_ldl: invalid argument");
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    const long long NN = (long long)N * N;
    float2* A = nullptr;
    double2* Ad = nullptr;
    void* ws = nullptr;
    int *info = nullptr, *err = nullptr;
    int rc = 0;
    const size_t wsb = tags_ldl_tc_workspace(N, nb);
    if (cudaMalloc(&A, sizeof(float2) * NN * nb) != cudaSuccess || cudaMalloc(&Ad, sizeof(double2) * NN * nb) != cudaSuccess ||
        cudaMalloc(&ws, wsb) != cudaSuccess || cudaMalloc(&info, sizeof(int) * nb) != cudaSuccess ||
        cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
        rc = tags_fail(TAGS_E_NOMEM, "device allocation failed");
    }
    std::vector<float2> hf(NN * nb);
    if (!rc) {
        for (long long q = 0; q < NN * nb; ++q) hf[q] = make_float2((float)a[q].re, (float)a[q].im);
        cudaMemcpyAsync(A, hf.data(), sizeof(float2) * NN * nb, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(ws, 0, wsb, st);
        cudaMemsetAsync(err, 0, sizeof(int), st);
        rc = tags_ldl_tc(A, N, N, NN, nb, nb, ws, info, err, 0, st);
    }
    int herr = 0;
    std::vector<int> hinfo(nb, 0);
    if (!rc) {
        cudaMemcpyAsync(hf.data(), A, sizeof(float2) * NN * nb, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = tags_fail(TAGS_E_CUDA, "tags_debug_ldl: stream failed");
    }
    if (!rc) {
        for (long long q = 0; q < NN * nb; ++q) a[q] = {hf[q].x, hf[q].y};
        if (herr) rc = tags_fail(TAGS_E_CUDA, "tags_debug_ldl: tensor-core wait ran out");
        for (int q = 0; q < nb && !rc; ++q)
            if (hinfo[q]) rc = hinfo[q];
    }
    cudaFree(A);
    cudaFree(Ad);
    cudaFree(ws);
    cudaFree(info);
    cudaFree(err);
    return rc;
}
