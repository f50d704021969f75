// Tensor-core LDL^T factorisation of the mixed form's working matrix, and the
// triangular solves with its factors.
//
// The reordered, scaled immittance matrix W'' (complex, symmetric,
// non-Hermitian) is factorised without pivoting as W'' = L D L^T in 128-column
// panels (right-looking, lower triangle only), in groups of up to six panels:
//   1. k_gemm_tc (mode 0, narrow): panel p's block column takes the update
//      from panels 0 .. p-1 of its group (K = 128 p) and is written on as
//      split planes;
//   2. k_ldl_diag: the 128 x 128 diagonal block -> L11 (unit lower), D1 and
//      the explicit inverse L11^{-1}, both in one elimination sweep (one CTA
//      per sample, the block in registers, complex FP32);
//   3. k_gemm_tc (mode 1): W21 = A21 L11^{-T} (the triangular solve as a
//      GEMM), L21 = W21 D1^{-1} in FP32 (for the solves) and V21 = W21
//      D1^{-1/2} = L21 D1^{1/2} as split planes into the group's buffer;
//   4. k_gemm_tc (mode 0, after each group): A22 -= V V^T (= L D L^T) over the
//      group's panels (K = 128 x panels) on the lower 128 x 128 tiles; one
//      plane set feeds both operands. The zero ZL/ZT band is skipped.
// The GEMMs run on the 5th-generation tensor cores: operands are staged in
// shared memory by TMA (64-byte swizzle, K-block-major planes), tcgen05.mma
// (kind::f16, FP32 accumulate) is issued by one thread, the two accumulators
// (real and imaginary part, 128 x 128 FP32 each) live in tensor memory,
// double-buffered, and are read back with tcgen05.ld by eight epilogue warps.
// A complex product is four real products; each real operand is split into
// two fp16 pieces of 2^8 x (about 22 significant bits; three bf16 pieces when
// a value leaves the fp16 range), and hi*hi + hi*lo + lo*hi per real product
// makes twelve tcgen05.mma per K step of 16. k_gemm_tc2 runs the same updates
// on clusters of two SMs (tcgen05.mma.cta_group::2; a plan option, slower
// here).
// The solves L D L^T x = r of the refinement run as one CTA per sample with x
// in shared memory (k_ldl_solve_cta), on clusters of CTAs per sample for small
// passes and for refinement steps with few samples left (k_ldl_solve_cl), or
// block by block where x does not fit in shared memory (k_blk_*).
// Every mbarrier wait is bounded in time (%globaltimer); on expiry the kernel
// raises an error flag, lets its copies in flight land, frees its tensor
// memory and returns, and the pass is re-solved in FP64.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <algorithm>
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
constexpr int GMAX = 6;                 // most panels per trailing update (K up to 768)
constexpr int KG = TB * GMAX;           // K extent of a group's plane buffers

// Split planes are K-block-major: plane p of a buffer with R rows and K
// columns holds blocks of 32 columns, each R rows x 32 (64-byte rows), so a
// TMA box of 32 columns x 128 rows is one contiguous 8 KiB piece.
TAGS_HD long long plane_elem(int p, int R, int K, int row, int col) {
    return (long long)p * R * K + (long long)(col >> 5) * R * 32 + (long long)row * 32 + (col & 31);
}
constexpr int SMAX = 3;                 // most bf16 pieces per real value (split products)
constexpr uint64_t WAIT_NS = 50ull * 1000 * 1000;   // 50 ms per wait
// Limit of the waits in the main loops of the tensor-core kernels (WAIT_NS
// unless a test lowered it through tags_debug_tc_wait_limit). The waits that
// let issued work finish after a failure always use WAIT_NS.
__device__ unsigned long long g_tc_wait_ns = WAIT_NS;

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
    const uint64_t lim = g_tc_wait_ns;
    const unsigned mask = lim < WAIT_NS ? 0u : 255u;     // a lowered limit is checked at every try
    const uint64_t t0 = globaltimer_ns();
    for (unsigned it = 0;; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if ((it & mask) == mask) {
            if (*(volatile int*)err != 0) return false;
            if (globaltimer_ns() - t0 > lim) {
                atomicOr(err, 8);
                return false;
            }
        }
    }
}
// Wait for the phase with parity `parity` of `bar` regardless of `err` (used
// after a wait ran out, to let work already issued finish before the CTA
// releases its resources), bounded by WAIT_NS; raises `err` if even that
// bound runs out.
TAGS_D bool mbar_wait_drain(uint32_t bar, uint32_t parity, int* err) {
    const uint64_t t0 = globaltimer_ns();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
        if (globaltimer_ns() - t0 > WAIT_NS) {
            atomicOr(err, 8);
            return false;
        }
    }
}
TAGS_D void tma_load_5d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                        uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
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

// Instruction descriptor: kind::f16, bf16 x bf16 or fp16 x fp16 -> f32,
// M = N = 128, both operands K-major.
TAGS_D uint32_t idesc_mma(bool negate_a, bool f16) {
    uint32_t d = 0;
    d |= 1u << 4;                            // D format f32
    d |= (f16 ? 0u : 1u) << 7;               // A format: 0 f16, 1 bf16
    d |= (f16 ? 0u : 1u) << 10;              // B format: same type as A
    d |= (negate_a ? 1u : 0u) << 13;
    d |= (uint32_t)(TB >> 3) << 17;          // N
    d |= (uint32_t)(TB >> 4) << 24;          // M
    return d;
}

// 1 / d for complex FP32 d, scaled against overflow
TAGS_D float2 crecip_f(float2 d) {
    const float sc = fmaxf(fabsf(d.x), fabsf(d.y));
    const float a = d.x / sc, b = d.y / sc;
    const float den = sc * fmaf(a, a, b * b);
    return make_float2(a / den, -b / den);
}

// Principal square root of complex FP32 z, in the cancellation-free form:
// with r = |z|, t = sqrt((r + |Re z|) / 2) is the larger part and the other is
// |Im z| / (2 t). sqrt(0) = 0. Any fixed branch serves: only s * s = z is used.
TAGS_D float2 csqrt_f(float2 z) {
    const float r = hypotf(z.x, z.y);
    if (r == 0.f) return make_float2(0.f, 0.f);
    const float t = sqrtf(0.5f * (r + fabsf(z.x)));
    const float u = 0.5f * fabsf(z.y) / t;
    return z.x >= 0.f ? make_float2(t, copysignf(u, z.y)) : make_float2(u, copysignf(t, z.y));
}

// Split forms of an FP32 value, as 16-bit patterns (each piece the rounded
// remainder of the previous ones):
//   bf16: x = p[0] + ... + p[S-1], S = 2 or 3 (3 pieces keep FP32 precision);
//   fp16: 2^8 x = p[0] + p[1] (22 significant bits; the 2^8 keeps values of
//         the scaled working matrix, |x| <= 255, inside fp16's range and its
//         small ones off the subnormals; a value outside raises `ovf`).
constexpr float kF16Scale = 256.f;
constexpr float kF16Unscale = 1.f / 65536.f;     // a product of two scaled operands
constexpr int kErrRange = 1;                      // err[1]: an fp16 piece out of range

TAGS_D void split_n(float x, uint16_t* p, int S, bool f16, int& ovf) {
    if (f16) {
        const float y = x * kF16Scale;
        if (!(fabsf(y) <= 65504.f)) ovf = 1;
        const __half h = __float2half_rn(y);
        p[0] = __half_as_ushort(h);
        p[1] = __half_as_ushort(__float2half_rn(y - __half2float(h)));
        return;
    }
    float r = x;
    for (int q = 0; q < S; ++q) {
        const __nv_bfloat16 b = __float2bfloat16_rn(r);
        p[q] = __bfloat16_as_ushort(b);
        r -= __bfloat162float(b);
    }
}

}  // namespace

// ---- GEMM on the tensor cores ------------------------------------------------------
//
// C (128 x 128 tiles) op= A B^T for complex A, B given as split planes
// [sample][2S][rows][128] bf16 (real pieces, then imaginary pieces). Persistent:
// one CTA per SM walks the tile list. Warp 0 streams K blocks of 32 (64-byte
// rows, 64-byte swizzle) of all planes of A and B through a ring of shared
// stages with TMA; one thread of warp 1 issues the tcgen05.mma products into
// one of two tensor-memory accumulator pairs (real, imaginary; 2 x 256
// columns); warps 2..5 read the other pair back and do the epilogue, so the
// memory-bound read-modify-write of C overlaps the products of the next tile.

constexpr int BK = 32;                               // K elements per stage
constexpr int KBLKS = TB / BK;                       // 4 stages per tile
constexpr int PST = TB * BK * 2;                     // one plane in one stage: 8 KiB

template <int S> struct GemmCfg {
    static constexpr int NPL = 2 * S;                // planes per operand
    static constexpr int STAGE = 2 * NPL * PST;      // A and B planes of one K block
    static constexpr int STAGES = S == 2 ? 3 : 2;
    static constexpr int BARS = 512;                  // mbarriers and the TMEM slot
    static constexpr int DINV = 2 * 8 * 64 * 8;       // mode 1: 64 values of D^{-1} and of D^{-1/2} per epilogue warp
    static constexpr int SMEM = STAGES * STAGE + 1024 + BARS + DINV;
};

// Shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups 512
// bytes apart (stride byte offset), descriptor version 1.
TAGS_D uint64_t sdesc64(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;           // stride byte offset
    d |= (uint64_t)1 << 46;                    // version
    d |= (uint64_t)4 << 61;                    // SWIZZLE_64B
    return d;
}

struct GemmArgs {
    int M, Nn;                 // valid rows / columns of the output
    int mode;                  // 0: C -= A B^T into the FP32 matrix; 1: panel output (L21, planes)
    int tri;                   // tiles enumerate the lower triangle (I >= J)
    int tiles;                 // tiles per sample
    int nb;                    // samples
    float2* Amat;              // FP32 working matrices
    long long ld, mstride;
    int row0, col0;            // matrix coordinates of output element (0, 0)
    const float2* dinv;        // per sample 128 values (mode 1)
    const float2* dsq;         // per sample 128 values of D^{-1/2} (mode 1)
    uint16_t* Lp;              // V planes written in mode 1: [sample][2S][R][KG] (a group's buffer)
    int prow0;                 // mode 1: buffer row of output row 0
    int kcol0;                 // mode 1: buffer column of output column 0 (128 x panel index in the group)
    int band_planes;           // mode 1: skipped band tiles still write (zero) planes
    long long pstride;         // elements per sample of the group buffer (Lp)
    long long npstride;        // elements per sample of the block-column buffer (Np), rows of 128
    int R;                     // rows of a plane buffer
    int* err;                  // err[0]: a wait ran out (all CTAs stop); err[1]: fp16 range
    int f16;                   // planes are scaled fp16 pairs (S == 2) instead of bf16 pieces
    int zlo, zhi;              // output rows/cols in [zlo, zhi) are structurally zero (tiles inside skipped)
    uint16_t* Np;              // mode 0: split planes of the next panel's block column (tiles J = 0, I >= 1), or null
    int Mn;                    // rows of the next panel's block column
    int kblocks;               // K blocks of BK (4 per panel of the group)
    int off;                   // row offset of the operand rows (tile row TB * I reads row TB * I + off)
    int neg_planes;            // mode 1, S = 2: also the negated imaginary planes, at slots 4, 5 of the group buffer
    int ba, bb;                // tri, bb > ba: tile rows/columns [ba, bb) lie wholly in the zero band and are left out
                               // of the enumeration (tri_compact_count), but for the J = 0 tiles that write Np planes
    int np_band;               // mode 0 with Np: also write the planes of the band's rows (the next panel's GEMM reads
                               // them only when its columns reach past the ZL block; before that its band rows are zero
                               // and skipped)
};

// Mode 0: a skipped tile whose rows hold the next panel's block column writes
// their planes (the current values), unless its rows lie in the band and the
// next panel's GEMM skips them.
TAGS_D bool skipped_writes_planes(const GemmArgs& g, int I, int J) {
    if (!(g.Np && J == 0 && I >= 1)) return false;
    if (g.np_band) return true;
    return !(g.zhi > g.zlo && TB * I >= g.zlo && TB * I + TB <= g.zhi);
}

// Lower-triangle tiles of an update with the zero band's tile rows/columns
// [ba, bb) taken out, in the order of the full enumeration (row by row):
//   rows I < ba:        J = 0 .. I                      (n1 = ba (ba + 1) / 2)
//   rows ba <= I < bb:  J = 0 only, where the next panel's planes are written
//                       there (Np and np_band; I >= 1), as a skipped tile (n2)
//   rows I >= bb:       the e left columns (J < ba; if ba = 0, J = 0 as a
//                       skipped tile when Np), then J = bb .. I  (n3)
// Every CTA then strides over tiles that do work, so the CTAs stay within a
// sample or two of each other: with the band's empty slots in the list, a CTA
// whose slots fall in the band ran ahead, and the CTAs in flight spread over
// about a dozen samples, whose operand rows no longer fitted in L2.
struct TriCompact {
    int n1, n2, e, r2s;
};
TAGS_HD TriCompact tri_compact(int ba, int bb, bool planes, bool planes_band) {
    TriCompact c;
    c.n1 = ba * (ba + 1) / 2;
    c.r2s = ba >= 1 ? ba : 1;
    c.n2 = planes && planes_band && bb > c.r2s ? bb - c.r2s : 0;
    c.e = ba >= 1 ? ba : (planes ? 1 : 0);
    return c;
}
TAGS_HD int tri_compact_count(int T, int ba, int bb, bool planes, bool planes_band) {
    const TriCompact c = tri_compact(ba, bb, planes, planes_band);
    const int R = T > bb ? T - bb : 0;
    return c.n1 + c.n2 + R * c.e + R * (R + 1) / 2;
}

// Tile l of the compacted list (row I, column J; skip: a tile that only
// writes planes).
TAGS_HD void tri_compact_tile(int l, int ba, int bb, bool planes, bool planes_band, int& I, int& J, bool& skip) {
    const TriCompact c = tri_compact(ba, bb, planes, planes_band);
    skip = false;
    if (l < c.n1) {
        I = (int)((sqrtf(8.0f * l + 1.0f) - 1.0f) * 0.5f);
        while ((I + 1) * (I + 2) / 2 <= l) ++I;
        while (I * (I + 1) / 2 > l) --I;
        J = l - I * (I + 1) / 2;
    } else if (l < c.n1 + c.n2) {
        I = c.r2s + (l - c.n1);
        J = 0;
        skip = true;
    } else {
        const int l3 = l - c.n1 - c.n2;
        const float bq = 2.0f * c.e + 1.0f;
        int r = (int)((sqrtf(bq * bq + 8.0f * l3) - bq) * 0.5f);
        while ((r + 1) * c.e + (r + 1) * (r + 2) / 2 <= l3) ++r;
        while (r > 0 && r * c.e + r * (r + 1) / 2 > l3) --r;
        const int q = l3 - (r * c.e + r * (r + 1) / 2);
        I = bb + r;
        if (q < c.e) {
            J = q;
            skip = ba == 0;                // J = 0 inside the band: planes only
        } else {
            J = bb + (q - c.e);
        }
    }
}

TAGS_D void tile_of(const GemmArgs& g, int t, int& smp, int& I, int& J, bool& skip) {
    smp = t / g.tiles;
    int l = t - smp * g.tiles;
    if (g.tri && g.bb > g.ba) {
        tri_compact_tile(l, g.ba, g.bb, g.Np != nullptr, g.np_band != 0, I, J, skip);
        return;
    }
    if (g.tri) {
        I = (int)((sqrtf(8.0f * l + 1.0f) - 1.0f) * 0.5f);
        while ((I + 1) * (I + 2) / 2 <= l) ++I;
        while (I * (I + 1) / 2 > l) --I;
        J = l - I * (I + 1) / 2;
    } else {
        I = l;
        J = 0;
    }
    skip = false;
    if (g.zhi > g.zlo) {
        bool row_zero = TB * I >= g.zlo && TB * I + TB <= g.zhi;
        bool col_zero = g.mode == 0 && TB * J >= g.zlo && TB * J + TB <= g.zhi;
        skip = row_zero || col_zero;
    }
}

// Row `row`, columns c0 .. c0+15 of a plane buffer [2S][R][128] (real
// pieces, then imaginary pieces): the split of v[0..15], two columns at a
// time with the packed conversions (one instruction per pair of values).
// With neg (S = 2), the imaginary pieces again with their signs flipped (an
// exact negation of both fp16 or bf16 pieces), as planes 4 and 5: the B rows
// [-Im] of the two-SM products in real form (k_gemm_tc2 with EMB).
template <int S>
TAGS_D void store_planes16(uint16_t* P, int R, int ks, int row, int c0, const float2* v, bool f16, int& ovf,
                           bool neg = false) {
    __align__(16) uint32_t pl[2 * S][8];        // 8 packed pairs = 16 columns per plane
    if (S == 2 && f16) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
#pragma unroll
            for (int c = 0; c < 2; ++c) {       // 0: real parts, 1: imaginary parts
                const float a = (c ? v[2 * j].y : v[2 * j].x) * kF16Scale;
                const float b = (c ? v[2 * j + 1].y : v[2 * j + 1].x) * kF16Scale;
                if (!(fmaxf(fabsf(a), fabsf(b)) <= 65504.f)) ovf = 1;
                const __half2 hi = __floats2half2_rn(a, b);
                const float2 hf = __half22float2(hi);
                const __half2 lo = __floats2half2_rn(a - hf.x, b - hf.y);
                pl[2 * c][j] = *reinterpret_cast<const uint32_t*>(&hi);
                pl[2 * c + 1][j] = *reinterpret_cast<const uint32_t*>(&lo);
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                float2 r = c ? make_float2(v[2 * j].y, v[2 * j + 1].y) : make_float2(v[2 * j].x, v[2 * j + 1].x);
#pragma unroll
                for (int q = 0; q < S; ++q) {
                    const __nv_bfloat162 h = __floats2bfloat162_rn(r.x, r.y);
                    const float2 f = __bfloat1622float2(h);
                    r.x -= f.x;
                    r.y -= f.y;
                    pl[c * S + q][j] = *reinterpret_cast<const uint32_t*>(&h);
                }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < 2 * S; ++p) {
        uint4* d = reinterpret_cast<uint4*>(P + plane_elem(p, R, ks, row, c0));
        d[0] = make_uint4(pl[p][0], pl[p][1], pl[p][2], pl[p][3]);
        d[1] = make_uint4(pl[p][4], pl[p][5], pl[p][6], pl[p][7]);
    }
    if (S == 2 && neg) {
        constexpr uint32_t SG = 0x80008000u;    // the sign bits of both 16-bit values
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const uint32_t* q = pl[S + p];
            uint4* d = reinterpret_cast<uint4*>(P + plane_elem(2 * S + p, R, ks, row, c0));
            d[0] = make_uint4(q[0] ^ SG, q[1] ^ SG, q[2] ^ SG, q[3] ^ SG);
            d[1] = make_uint4(q[4] ^ SG, q[5] ^ SG, q[6] ^ SG, q[7] ^ SG);
        }
    }
}

constexpr int EPI_WARPS = 8;               // two warps per tensor-memory lane quarter
constexpr int GEMM_THREADS = 32 * (2 + EPI_WARPS);

template <int S, int MODE>
__global__ void __launch_bounds__(GEMM_THREADS, 1) k_gemm_tc(const __grid_constant__ CUtensorMap tmA,
                                                             const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    using C = GemmCfg<S>;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t base_u32 = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* base = smem_raw + (base_u32 - smem_u32(smem_raw));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + C::STAGES * C::STAGE);
    // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], drain
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * C::STAGES + 5);
    auto full = [&](int s) { return smem_u32(&bars[s]); };
    auto empty = [&](int s) { return smem_u32(&bars[C::STAGES + s]); };
    auto tfull = [&](int a) { return smem_u32(&bars[2 * C::STAGES + a]); };
    auto tempty = [&](int a) { return smem_u32(&bars[2 * C::STAGES + 2 + a]); };
    const uint32_t drain = smem_u32(&bars[2 * C::STAGES + 4]);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int total = g.tiles * g.nb;
    if (tid == 0) {
        for (int q = 0; q < C::STAGES; ++q) {
            mbar_init(full(q), 1);
            mbar_init(empty(q), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), EPI_WARPS);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), 512);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        // ---- producer: TMA loads of A and B planes, one K block per stage
        int stage = 0;
        uint32_t phase = 0;
        bool alive = true;
        int issued[4] = {0, 0, 0, 0};     // stages with a load whose completion nobody waited for yet
        uint32_t ipar[4] = {0, 0, 0, 0};  // parity of the full-barrier phase each such load completes
        for (int t = blockIdx.x; t < total && alive; t += gridDim.x) {
            int smp, I, J;
            bool skip;
            tile_of(g, t, smp, I, J, skip);
            if (skip) continue;
            if (lane == 0) {
                for (int kb = 0; kb < g.kblocks; ++kb) {
                    if (!mbar_wait(empty(stage), phase ^ 1, g.err)) { alive = false; break; }
                    issued[stage] = 0;
                    const uint32_t sb = base_u32 + stage * C::STAGE;
                    mbar_expect_tx(full(stage), C::STAGE);
                    const int ra = TB * I + g.off, rb = TB * J + g.off;
                    for (int p = 0; p < C::NPL; ++p) {
                        tma_load_5d(sb + p * PST, &tmA, 0, ra, kb, p, smp, full(stage));
                        tma_load_5d(sb + (C::NPL + p) * PST, &tmB, 0, rb, kb, p, smp, full(stage));
                    }
                    issued[stage] = 1;
                    ipar[stage] = phase;
                    if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
            }
            alive = __shfl_sync(0xffffffffu, alive ? 1 : 0, 0) != 0;
        }
        if (lane == 0) {
            // let the copies in flight land before the CTA exits (after a wait
            // ran out anywhere in the CTA some may be unconsumed): each waits
            // on the phase its stage was issued under
            for (int q = 0; q < C::STAGES; ++q)
                if (issued[q]) mbar_wait_drain(full(q), ipar[q], g.err);
        }
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            const uint32_t idp = idesc_mma(false, g.f16 != 0), idn = idesc_mma(true, g.f16 != 0);
            int stage = 0, acc = 0;
            uint32_t phase = 0, aphase = 0;
            bool alive = true;
            for (int t = blockIdx.x; t < total && alive; t += gridDim.x) {
                int smp, I, J;
                bool skip;
                tile_of(g, t, smp, I, J, skip);
                if (skip) continue;
                if (!mbar_wait(tempty(acc), aphase ^ 1, g.err)) { alive = false; break; }
                tc_fence_after();
                const uint32_t accR = tmem + acc * 256, accI = accR + 128;
                for (int kb = 0; kb < g.kblocks && alive; ++kb) {
                    if (!mbar_wait(full(stage), phase, g.err)) { alive = false; break; }
                    tc_fence_after();
                    const uint32_t sa = base_u32 + stage * C::STAGE, sbb = sa + C::NPL * PST;
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint32_t off = kk * 32;
                        bool firstR = kb == 0 && kk == 0, firstI = firstR;
                        // terms (i, j) with i + j < S of the split product
                        for (int i = 0; i < S; ++i) {
                            for (int j = 0; i + j < S; ++j) {
                                const uint64_t ar = sdesc64(sa + i * PST + off), ai = sdesc64(sa + (S + i) * PST + off);
                                const uint64_t br = sdesc64(sbb + j * PST + off), bi = sdesc64(sbb + (S + j) * PST + off);
                                mma_bf16(accR, ar, br, idp, firstR ? 0u : 1u);   // + Ar Br
                                firstR = false;
                                mma_bf16(accR, ai, bi, idn, 1u);                 // - Ai Bi
                                mma_bf16(accI, ar, bi, idp, firstI ? 0u : 1u);   // + Ar Bi
                                firstI = false;
                                mma_bf16(accI, ai, br, idp, 1u);                 // + Ai Br
                            }
                        }
                    }
                    mma_commit(empty(stage));          // stage reusable once these products are done
                    if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
                if (!alive) break;
                mma_commit(tfull(acc));                // accumulator pair ready for the epilogue
                if (++acc == 2) { acc = 0; aphase ^= 1; }
            }
            // every product issued is complete before tensor memory is released
            mma_commit(drain);
            mbar_wait_drain(drain, 0u, g.err);
        }
    } else {
        // ---- epilogue warps 2..9: warp w reads tensor-memory lanes 32 (w % 4) ...
        // and one half of the columns
        const int quarter = warp & 3, half = (warp - 2) >> 2;
        const int r = 32 * quarter + lane;
        float2* dinv_w = reinterpret_cast<float2*>(base + C::STAGES * C::STAGE + C::BARS) + (warp - 2) * 64;
        const uint32_t lane_off = (uint32_t)(32 * quarter) << 16;
        const bool f16 = S == 2 && g.f16 != 0;
        const float unscale = f16 ? kF16Unscale : 1.f;
        int ovf = 0;
        int acc = 0;
        uint32_t aphase = 0;
        for (int t = blockIdx.x; t < total; t += gridDim.x) {
            int smp, I, J;
            bool skip;
            tile_of(g, t, smp, I, J, skip);
            if (skip) {
                const int gr = TB * I + r;
                if (MODE == 1 && g.band_planes && gr < g.M) {
                    // rows of the zero band: L21 = V21 = 0 there; their planes are
                    // written (as zeros) so that a later update that no longer
                    // skips the band reads zeros, not another panel's values
                    float2 zv[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j) zv[j] = make_float2(0.f, 0.f);
                    for (int cc = half * 4; cc < half * 4 + 4; ++cc) {
                        store_planes16<S>(g.Lp + g.pstride * smp, g.R, KG, g.prow0 + gr, g.kcol0 + cc * 16, zv, f16, ovf,
                                          g.neg_planes != 0);
                    }
                }
                // no update of this tile; if it holds rows of the next panel's
                // block column, their planes are the current values
                if (MODE == 0 && skipped_writes_planes(g, I, J) && gr < g.M && gr - TB < g.Mn) {
                    const float2* Cb = g.Amat + g.mstride * smp;
                    for (int cc = half * 4; cc < half * 4 + 4; ++cc) {
                        const float2* base_p = Cb + (long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + cc * 16);
                        float2 cv[16];
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            cv[j] = cc * 16 + j < g.Nn ? base_p[g.ld * j] : make_float2(0.f, 0.f);
                        store_planes16<S>(g.Np + g.npstride * smp, g.R, TB, gr - TB, cc * 16, cv, f16, ovf);
                    }
                }
                continue;
            }
            if (MODE == 1) {
                // this warp's 64 columns of D^{-1} and D^{-1/2}, staged before the wait
                __syncwarp();
                dinv_w[lane] = g.dinv[(long long)TB * smp + half * 64 + lane];
                dinv_w[32 + lane] = g.dinv[(long long)TB * smp + half * 64 + 32 + lane];
                dinv_w[8 * 64 + lane] = g.dsq[(long long)TB * smp + half * 64 + lane];
                dinv_w[8 * 64 + 32 + lane] = g.dsq[(long long)TB * smp + half * 64 + 32 + lane];
                __syncwarp();
            }
            if (!mbar_wait(tfull(acc), aphase, g.err)) break;
            tc_fence_after();
            const uint32_t accR = tmem + acc * 256, accI = accR + 128;
            const int gr = TB * I + r;
            float2* Cb = g.Amat + g.mstride * smp;
            for (int cc = half * 4; cc < half * 4 + 4; ++cc) {
                float vr[16], vi[16];
                tmem_ld16(accR + lane_off + cc * 16, vr);
                tmem_ld16(accI + lane_off + cc * 16, vi);
                if (gr >= g.M) continue;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    vr[j] *= unscale;
                    vi[j] *= unscale;
                }
                if (MODE == 0) {
                    // rows of the next panel's block column below its diagonal
                    // block go on as split planes only: the panel GEMM reads them
                    // from the planes and then writes L21 over them in FP32, so
                    // their FP32 store would be dead
                    const bool planes_only = g.Np && J == 0 && I >= 1 && gr - TB < g.Mn;
                    // in a diagonal tile (the updates' rows and columns share
                    // their origin) only the lower triangle is live: the
                    // diagonal-block kernel reads nothing above it
                    const int cend = I == J ? min(g.Nn, gr + 1) : g.Nn;
                    // all loads of the chunk first, then the stores
                    float2* base_p = Cb + (long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + TB * J + cc * 16);
                    float2 cv[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (TB * J + cc * 16 + j < cend) cv[j] = base_p[g.ld * j];
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        cv[j] = make_float2(cv[j].x - vr[j], cv[j].y - vi[j]);
                        if (!planes_only && TB * J + cc * 16 + j < cend) base_p[g.ld * j] = cv[j];
                    }
                    if (planes_only) {
                        // the next panel's block column, as split planes
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (cc * 16 + j >= g.Nn) cv[j] = make_float2(0.f, 0.f);
                        store_planes16<S>(g.Np + g.npstride * smp, g.R, TB, gr - TB, cc * 16, cv, f16, ovf);
                    }
                } else {
                    const float2* dv = dinv_w - half * 64;      // indexed by the tile column
                    const float2* sq = dv + 8 * 64;
                    float2 vv[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const int c = cc * 16 + j;
                        const float2 wv = make_float2(vr[j], vi[j]);
                        vv[j] = fmulc(wv, sq[c]);
                        if (c < g.Nn) Cb[(long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + c)] = fmulc(wv, dv[c]);
                    }
                    store_planes16<S>(g.Lp + g.pstride * smp, g.R, KG, g.prow0 + gr, g.kcol0 + cc * 16, vv, f16, ovf,
                                      g.neg_planes != 0);
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tempty(acc)) : "memory");
            if (++acc == 2) { acc = 0; aphase ^= 1; }
        }
        if (ovf) atomicOr(g.err + kErrRange, 1);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// ---- two-SM GEMM (tcgen05 cta_group::2) for the mode-0 updates -----------------------
//
// A cluster of two CTAs on two SMs computes a pair of vertically adjacent
// tiles, rows (I0, I0 + 1) x column J, as tcgen05.mma.cta_group::2 products
// with M = 256, N = 128. Each CTA stages its own 128 rows of A and one half
// (64 rows) of B in its shared memory; the products, issued by one thread of
// the even CTA, read A from each CTA's own shared memory and B from both, so
// each SM streams 4 KiB of A and 2 KiB of B per 64-clock product instead of
// 4 + 4 KiB (the single-CTA kernel's shared-memory bound). Each CTA's tensor
// memory holds the accumulators of its own 128 rows; its epilogue warps do
// the read-modify-write of its own tile exactly as in k_gemm_tc (mode 0).
// Barriers: the even CTA's full[s] takes two arrivals (one per CTA, each with
// its own byte count) and both CTAs' copies complete on it; the products'
// commits are multicast to both CTAs' empty[s] (stage free) and tfull[a]
// (accumulators ready); the epilogue warps of both CTAs arrive on the even
// CTA's tempty[a]. Every wait is bounded as in k_gemm_tc; at the end the even
// CTA waits for its products and copies, then both CTAs meet at a cluster
// barrier before the tensor memory is released.

constexpr int PSTB = (TB / 2) * BK * 2;              // one plane of a B half in one stage: 4 KiB

// EMB = 1 (S = 2 only): the complex update as one real product per split
// pair with N = 256, [Re | Im] = [Ar Ai] [[Br, -Bi], [Bi, Br]]^T: the even CTA
// stages B rows Br (planes 0, 1) and -Bi (planes 4, 5), the odd CTA Bi
// (planes 2, 3) and Br, each 128 rows, so an SM reads 4 KiB of A and 4 KiB of
// its own B per 128-cycle product (64 B per cycle, half of the single-SM
// kernel's) and the products per K step fall from 12 to 6.
template <int S, int EMB = 0> struct Gemm2Cfg {
    static constexpr int NPL = 2 * S;
    static constexpr int ABYTES = NPL * PST;          // A planes of one stage
    static constexpr int STAGE = EMB ? 2 * NPL * PST : NPL * (PST + PSTB);   // A planes, then the B planes
    static constexpr int STAGES = EMB ? 3 : (S == 2 ? 4 : 3);
    static constexpr int BARS = 512;
    static constexpr int SMEM = STAGES * STAGE + 1024 + BARS;
};

TAGS_D uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
TAGS_D uint32_t cluster_idx() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
TAGS_D uint32_t cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
// Address in the shared::cluster window of the same variable in CTA `rank`.
TAGS_D uint32_t mapa_cta(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
TAGS_D void mbar_arrive_expect_tx_cluster(uint32_t cbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cluster.shared::cluster.b64 _, [%0], %1;" ::"r"(cbar), "r"(bytes)
                 : "memory");
}
TAGS_D void mbar_arrive_cluster(uint32_t cbar) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cbar) : "memory");
}
TAGS_D void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire;" ::: "memory");
}
// Copy into this CTA's shared memory; completion is signalled on the mbarrier
// at cluster address `cbar` (the even CTA's).
TAGS_D void tma_load_5d_pair(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3, int c4,
                             uint32_t cbar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.cta_group::2 [%0], [%1, {%2, "
        "%3, %4, %5, %6}], [%7];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(cbar)
        : "memory");
}
TAGS_D void tmem_alloc_pair(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
TAGS_D void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
TAGS_D void mma_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// Arrive on the mbarrier at this shared offset in both CTAs of the pair once
// the products issued so far are complete.
TAGS_D void mma_pair_commit_both(uint32_t bar) {
    const uint16_t mask = 3;
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
        "h"(mask)
        : "memory");
}
TAGS_D void mma_pair_commit_local(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// Instruction descriptor of the pair products: M = 256, N = 128 (or N = 256).
TAGS_D uint32_t idesc_mma_pair(bool negate_a, bool f16, bool n256 = false) {
    uint32_t d = idesc_mma(negate_a, f16);
    d &= ~(31u << 24);
    d |= (uint32_t)(2 * TB >> 4) << 24;                 // M = 256
    if (n256) {
        d &= ~(63u << 17);
        d |= (uint32_t)(2 * TB >> 3) << 17;             // N = 256
    }
    return d;
}

TAGS_D bool tile_in_band(const GemmArgs& g, int I, int J) {
    if (g.zhi <= g.zlo) return false;
    const bool row_zero = TB * I >= g.zlo && TB * I + TB <= g.zhi;
    const bool col_zero = TB * J >= g.zlo && TB * J + TB <= g.zhi;
    return row_zero || col_zero;
}
// Tile rows of the update, and pair tiles per sample: tile rows I0, I0 + 1 of
// column J (lower triangle: I0 = J, J + 2, ...; block column: J = 0).
TAGS_HD int pair_rows(const GemmArgs& g) { return g.tri ? (g.M + TB - 1) / TB : g.tiles; }
TAGS_HD int pair_count(const GemmArgs& g, int T) {
    if (!g.tri) return (T + 1) / 2;
    int c = 0;
    for (int j = 0; j < T; ++j) c += (T - j + 1) / 2;
    return c;
}
TAGS_D void pair_of(const GemmArgs& g, int T, int l, int& I0, int& J) {
    if (!g.tri) {
        J = 0;
        I0 = 2 * l;
        return;
    }
    int j = 0;
    for (; j < T - 1; ++j) {
        const int c = (T - j + 1) / 2;
        if (l < c) break;
        l -= c;
    }
    J = j;
    I0 = j + 2 * l;
}

// Mode 0, a tile outside the products (zero band, or past the last tile
// row): if it holds rows of the next panel's block column, their current
// values become that block column's split planes.
template <int S>
TAGS_D void skipped_tile_planes(const GemmArgs& g, int smp, int I, int J, int r, int half, int& ovf) {
    const int gr = TB * I + r;
    if (!(skipped_writes_planes(g, I, J) && gr < g.M && gr - TB < g.Mn)) return;
    const bool f16 = S == 2 && g.f16 != 0;
    const float2* Cb = g.Amat + g.mstride * smp;
    for (int cc = half * 4; cc < half * 4 + 4; ++cc) {
        const float2* base_p = Cb + (long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + cc * 16);
        float2 cv[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) cv[j] = cc * 16 + j < g.Nn ? base_p[g.ld * j] : make_float2(0.f, 0.f);
        store_planes16<S>(g.Np + g.npstride * smp, g.R, TB, gr - TB, cc * 16, cv, f16, ovf);
    }
}

template <int S, int EMB>
__global__ void __launch_bounds__(GEMM_THREADS, 1) k_gemm_tc2(const __grid_constant__ CUtensorMap tmA,
                                                              const __grid_constant__ CUtensorMap tmB, GemmArgs g) {
    static_assert(!EMB || S == 2, "the real-form products need the negated planes of S = 2");
    using C = Gemm2Cfg<S, EMB>;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t base_u32 = (smem_u32(smem_raw) + 1023u) & ~1023u;
    uint8_t* base = smem_raw + (base_u32 - smem_u32(smem_raw));
    uint64_t* bars = reinterpret_cast<uint64_t*>(base + C::STAGES * C::STAGE);
    // bars: full[STAGES], empty[STAGES], tfull[2], tempty[2], drain
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2 * C::STAGES + 5);
    auto full = [&](int q) { return smem_u32(&bars[q]); };
    auto empty = [&](int q) { return smem_u32(&bars[C::STAGES + q]); };
    auto tfull = [&](int a) { return smem_u32(&bars[2 * C::STAGES + a]); };
    auto tempty = [&](int a) { return smem_u32(&bars[2 * C::STAGES + 2 + a]); };
    const uint32_t drain = smem_u32(&bars[2 * C::STAGES + 4]);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t rank = cluster_rank();
    const int T = pair_rows(g);
    const int P = pair_count(g, T);
    const long long total = (long long)P * g.nb;
    const long long first = cluster_idx(), stride = cluster_count();
    if (tid == 0) {
        for (int q = 0; q < C::STAGES; ++q) {
            mbar_init(full(q), 2);            // one arrival (with its bytes) per CTA of the pair
            mbar_init(empty(q), 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(tfull(a), 1);
            mbar_init(tempty(a), 2 * EPI_WARPS);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // both CTAs' barriers are initialised before either arrives remotely
    cluster_sync_all();
    if (warp == 1) tmem_alloc_pair(smem_u32(tslot), 512);
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        // ---- producer (both CTAs): own A rows, own half of B; completion on the even CTA's full[s]
        int stage = 0;
        uint32_t phase = 0;
        bool alive = true;
        int issued[4] = {0, 0, 0, 0};
        uint32_t ipar[4] = {0, 0, 0, 0};
        for (long long t = first; t < total && alive; t += stride) {
            const int smp = (int)(t / P);
            int I0, J;
            pair_of(g, T, (int)(t - (long long)smp * P), I0, J);
            const bool skip0 = tile_in_band(g, I0, J), skip1 = I0 + 1 >= T || tile_in_band(g, I0 + 1, J);
            if (skip0 && skip1) continue;
            if (lane == 0) {
                const int I = I0 + (int)rank;
                for (int kb = 0; kb < g.kblocks; ++kb) {
                    if (!mbar_wait(empty(stage), phase ^ 1, g.err)) { alive = false; break; }
                    issued[stage] = 0;
                    const uint32_t sa = base_u32 + stage * C::STAGE, sb = sa + C::ABYTES;
                    const uint32_t cfull = mapa_cta(full(stage), 0);
                    mbar_arrive_expect_tx_cluster(cfull, C::STAGE);
                    const int ra = TB * I + g.off;
                    if (EMB) {
                        // 128 B rows per CTA: even Br (0, 1), -Bi (4, 5); odd Bi (2, 3), Br (0, 1)
                        const int rb = TB * J + g.off;
                        for (int p = 0; p < C::NPL; ++p) {
                            const int pb = rank == 0 ? (p < S ? p : 2 * S + p - S) : (p < S ? S + p : p - S);
                            tma_load_5d_pair(sa + p * PST, &tmA, 0, ra, kb, p, smp, cfull);
                            tma_load_5d_pair(sb + p * PST, &tmB, 0, rb, kb, pb, smp, cfull);
                        }
                    } else {
                        const int rb = TB * J + g.off + (TB / 2) * (int)rank;
                        for (int p = 0; p < C::NPL; ++p) {
                            tma_load_5d_pair(sa + p * PST, &tmA, 0, ra, kb, p, smp, cfull);
                            tma_load_5d_pair(sb + p * PSTB, &tmB, 0, rb, kb, p, smp, cfull);
                        }
                    }
                    issued[stage] = 1;
                    ipar[stage] = phase;
                    if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
            }
            alive = __shfl_sync(0xffffffffu, alive ? 1 : 0, 0) != 0;
        }
        if (lane == 0) {
            // let this CTA's copies land before the pair releases its memory: the
            // even CTA on its full barriers (both CTAs' bytes), the odd CTA on the
            // products' release of each stage it filled
            for (int q = 0; q < C::STAGES; ++q)
                if (issued[q]) mbar_wait_drain(rank == 0 ? full(q) : empty(q), ipar[q], g.err);
        }
    } else if (warp == 1) {
        // ---- MMA issuer: one thread of the even CTA
        if (rank == 0 && lane == 0) {
            const uint32_t idp = idesc_mma_pair(false, g.f16 != 0), idn = idesc_mma_pair(true, g.f16 != 0);
            const uint32_t id256 = idesc_mma_pair(false, g.f16 != 0, true);
            int stage = 0, acc = 0;
            uint32_t phase = 0, aphase = 0;
            bool alive = true;
            for (long long t = first; t < total && alive; t += stride) {
                const int smp = (int)(t / P);
                int I0, J;
                pair_of(g, T, (int)(t - (long long)smp * P), I0, J);
                const bool skip0 = tile_in_band(g, I0, J), skip1 = I0 + 1 >= T || tile_in_band(g, I0 + 1, J);
                if (skip0 && skip1) continue;
                if (!mbar_wait(tempty(acc), aphase ^ 1, g.err)) { alive = false; break; }
                tc_fence_after();
                const uint32_t accR = tmem + acc * 256, accI = accR + 128;
                for (int kb = 0; kb < g.kblocks && alive; ++kb) {
                    if (!mbar_wait(full(stage), phase, g.err)) { alive = false; break; }
                    tc_fence_after();
                    const uint32_t sa = base_u32 + stage * C::STAGE, sbb = sa + C::ABYTES;
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint32_t off = kk * 32;
                        bool firstR = kb == 0 && kk == 0, firstI = firstR;
                        for (int i = 0; i < S; ++i) {
                            for (int j = 0; i + j < S; ++j) {
                                const uint64_t ar = sdesc64(sa + i * PST + off), ai = sdesc64(sa + (S + i) * PST + off);
                                if (EMB) {
                                    // [Re | Im] += Ar [Br | Bi]^T, then Ai [-Bi | Br]^T (B rows per CTA)
                                    const uint64_t bx = sdesc64(sbb + j * PST + off),
                                                   by = sdesc64(sbb + (S + j) * PST + off);
                                    mma_pair(accR, ar, bx, id256, firstR ? 0u : 1u);
                                    firstR = false;
                                    mma_pair(accR, ai, by, id256, 1u);
                                } else {
                                    const uint64_t br = sdesc64(sbb + j * PSTB + off),
                                                   bi = sdesc64(sbb + (S + j) * PSTB + off);
                                    mma_pair(accR, ar, br, idp, firstR ? 0u : 1u);   // + Ar Br
                                    firstR = false;
                                    mma_pair(accR, ai, bi, idn, 1u);                 // - Ai Bi
                                    mma_pair(accI, ar, bi, idp, firstI ? 0u : 1u);   // + Ar Bi
                                    firstI = false;
                                    mma_pair(accI, ai, br, idp, 1u);                 // + Ai Br
                                }
                            }
                        }
                    }
                    mma_pair_commit_both(empty(stage));      // stage reusable in both CTAs
                    if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
                if (!alive) break;
                mma_pair_commit_both(tfull(acc));            // both CTAs' accumulators ready
                if (++acc == 2) { acc = 0; aphase ^= 1; }
            }
            // every product issued is complete before tensor memory is released
            mma_pair_commit_local(drain);
            mbar_wait_drain(drain, 0u, g.err);
        }
    } else {
        // ---- epilogue warps 2..9 of both CTAs: this CTA's tile row I0 + rank
        const int quarter = warp & 3, half = (warp - 2) >> 2;
        const int r = 32 * quarter + lane;
        const uint32_t lane_off = (uint32_t)(32 * quarter) << 16;
        const bool f16 = S == 2 && g.f16 != 0;
        const float unscale = f16 ? kF16Unscale : 1.f;
        int ovf = 0;
        int acc = 0;
        uint32_t aphase = 0;
        for (long long t = first; t < total; t += stride) {
            const int smp = (int)(t / P);
            int I0, J;
            pair_of(g, T, (int)(t - (long long)smp * P), I0, J);
            const bool skip0 = tile_in_band(g, I0, J), skip1 = I0 + 1 >= T || tile_in_band(g, I0 + 1, J);
            const int I = I0 + (int)rank;
            const bool mine_valid = I < T;
            const bool mine_skip = rank == 0 ? skip0 : skip1;
            if (skip0 && skip1) {
                if (mine_valid) skipped_tile_planes<S>(g, smp, I, J, r, half, ovf);
                continue;
            }
            if (!mbar_wait(tfull(acc), aphase, g.err)) break;
            tc_fence_after();
            if (mine_skip) {
                if (mine_valid) skipped_tile_planes<S>(g, smp, I, J, r, half, ovf);
            } else {
                const uint32_t accR = tmem + acc * 256, accI = accR + 128;
                const int gr = TB * I + r;
                float2* Cb = g.Amat + g.mstride * smp;
                for (int cc = half * 4; cc < half * 4 + 4; ++cc) {
                    float vr[16], vi[16];
                    tmem_ld16(accR + lane_off + cc * 16, vr);
                    tmem_ld16(accI + lane_off + cc * 16, vi);
                    if (gr >= g.M) continue;
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        vr[j] *= unscale;
                        vi[j] *= unscale;
                    }
                    const bool planes_only = g.Np && J == 0 && I >= 1 && gr - TB < g.Mn;
                    const int cend = I == J ? min(g.Nn, gr + 1) : g.Nn;
                    float2* base_p = Cb + (long long)(g.row0 + gr) + g.ld * (long long)(g.col0 + TB * J + cc * 16);
                    float2 cv[16];
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if (TB * J + cc * 16 + j < cend) cv[j] = base_p[g.ld * j];
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        cv[j] = make_float2(cv[j].x - vr[j], cv[j].y - vi[j]);
                        if (!planes_only && TB * J + cc * 16 + j < cend) base_p[g.ld * j] = cv[j];
                    }
                    if (planes_only) {
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (cc * 16 + j >= g.Nn) cv[j] = make_float2(0.f, 0.f);
                        store_planes16<S>(g.Np + g.npstride * smp, g.R, TB, gr - TB, cc * 16, cv, f16, ovf);
                    }
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive_cluster(mapa_cta(tempty(acc), 0));
            if (++acc == 2) { acc = 0; aphase ^= 1; }
        }
        if (ovf) atomicOr(g.err + kErrRange, 1);
    }
    tc_fence_before();
    __syncthreads();
    // the even CTA arrives here only after its products and copies are done
    cluster_sync_all();
    if (warp == 1) tmem_dealloc_pair(tmem, 512);
}

// ---- diagonal block: LDL^T, L11^{-1} -------------------------------------------------

// One CTA of 512 threads per sample. The block lives in registers: thread
// (lane tx, warp ty) holds the 32 elements (tx + 32 p, ty + 16 q), p < 4,
// q < 8, so column k belongs to warp k % 16 and row k to lane k % 32 of
// every warp. Step k of the right-looking LDL^T: the owner warp of column k
// forms W = A[k+1:, k] and L = W / d into a double-buffered shared pair, one
// barrier, then every thread updates its elements i >= j > k. The inverse
// of the unit lower L11 is the same sweep applied to the identity, with
// the L columns kept in shared memory and the finished row k of L11^{-1}
// broadcast per step. Outside jb the block is padded with the identity.
constexpr int DIAG_LD = TB + 1;        // padded row stride of the output staging

__global__ void __launch_bounds__(512, 1) k_ldl_diag(float2* __restrict__ A0, long long ld, long long mstride, int j0,
                                                     int jb, uint16_t* __restrict__ linv_planes,
                                                     float2* __restrict__ dinv, float2* __restrict__ dsq,
                                                     int* __restrict__ info,
                                                     float2* __restrict__ linv32, long long lstride, int NS, int f16,
                                                     int* __restrict__ err) {
    extern __shared__ __align__(16) float2 S[];        // L columns S[k * TB + i]; later X staged S[i * DIAG_LD + j]
    __shared__ float2 wv[2][TB], lv[2][TB], dsh[TB];
    __shared__ int zero_at;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5, smp = blockIdx.x;
    float2* A = A0 + mstride * smp;
    if (tid == 0) zero_at = 0x7fffffff;
    float2 a[4][8];
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int i = tx + 32 * p, j = ty + 16 * q;
            float2 v = make_float2(i == j ? 1.f : 0.f, 0.f);
            if (i < jb && j < jb && i >= j) v = A[(long long)(j0 + i) + ld * (j0 + j)];
            a[p][q] = v;
        }
    __syncthreads();
    // ---- LDL^T and X = L11^{-1} in one sweep: k = 16 kq + kw (q index kq and p
    // index kq / 2 are compile-time). Step k scales column k (l_i = w_i / d_k)
    // and applies one rank-1 update to the rows i > k: the columns j > k hold
    // the trailing matrix (A[i][j] -= l_i A[j][k]), the finished columns j < k
    // hold X, which takes the same row operation (X[i][j] -= l_i X[k][j]), and
    // column k switches from A to X (X[i][k] = 0 - l_i, X[k][k] = 1). Each X
    // entry sees the operations of the forward substitution in the same order.
    // One barrier per step; the broadcast row is W: X[k][j] for j < k, 1 at k,
    // A[j][k] for j > k.
#pragma unroll
    for (int kq = 0; kq < 8; ++kq) {
        for (int kw = 0; kw < 16; ++kw) {
            const int k = 16 * kq + kw, buf = k & 1;
            if (tx == (k & 31)) {                // row k of X, final since step k - 1
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int j = ty + 16 * q;
                    if (j < k) wv[buf][j] = a[kq >> 1][q];
                }
            }
            if (ty == kw) {
                const int src = k & 31;
                float2 d;
                d.x = __shfl_sync(0xffffffffu, a[kq >> 1][kq].x, src);
                d.y = __shfl_sync(0xffffffffu, a[kq >> 1][kq].y, src);
                if (tx == 0) {
                    dsh[k] = d;
                    wv[buf][k] = make_float2(1.f, 0.f);
                    if (!(d.x != 0.f || d.y != 0.f) && k < jb) atomicMin(&zero_at, k);
                }
                const float2 di = crecip_f(d);
#pragma unroll
                for (int p = 0; p < 4; ++p) {
                    const int i = tx + 32 * p;
                    if (i > k) {
                        const float2 w = a[p][kq], l = fmulc(w, di);
                        wv[buf][i] = w;
                        lv[buf][i] = l;
                        S[k * TB + i] = l;
                        a[p][kq] = make_float2(0.f, 0.f);
                    } else if (i == k) {
                        a[p][kq] = make_float2(1.f, 0.f);
                    }
                }
            }
            __syncthreads();
            float2 nL[4], W[8];
#pragma unroll
            for (int p = kq >> 1; p < 4; ++p) {
                const float2 l = lv[buf][tx + 32 * p];
                nL[p] = make_float2(-l.x, -l.y);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) W[q] = wv[buf][ty + 16 * q];
            // rows i <= k are final: only register row kq / 2 holds some
#pragma unroll
            for (int p = kq >> 1; p < 4; ++p)
#pragma unroll
                for (int q = 0; q < 2 * p + 2; ++q)     // columns j >= 32 p + 32 lie above the diagonal
                    if (p > (kq >> 1) || tx + 32 * p > k) a[p][q] = ffmac(nL[p], W[q], a[p][q]);
        }
    }
    // X is unit lower: clear what the updates left above the diagonal
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (ty + 16 * q > tx + 32 * p) a[p][q] = make_float2(0.f, 0.f);
    __syncthreads();
    // L11 (unit lower, strictly below the diagonal, from S) and D back to A
    for (int t = tid; t < TB * TB; t += blockDim.x) {
        const int i = t % TB, j = t / TB;
        if (i < jb && j < jb && i >= j) A[(long long)(j0 + i) + ld * (j0 + j)] = i == j ? dsh[i] : S[j * TB + i];
    }
    if (tid == 0 && zero_at < jb && info[smp] == 0) info[smp] = j0 + zero_at + 1;
    if (tid < TB) {
        const float2 di = tid < jb ? crecip_f(dsh[tid]) : make_float2(0.f, 0.f);
        dinv[(long long)TB * smp + tid] = di;
        dsq[(long long)TB * smp + tid] = csqrt_f(di);
    }
    __syncthreads();                                    // S (L columns) is dead: stage X row-major, padded
#pragma unroll
    for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 8; ++q) S[(tx + 32 * p) * DIAG_LD + ty + 16 * q] = a[p][q];
    __syncthreads();
    // L11^{-1} kept in FP32 for the triangular solves, row-major, zero outside
    // jb: the inverse itself and its transpose (both read row-wise there)
    float2* X32 = linv32 + lstride * smp + (long long)(j0 / TB) * 2 * TB * TB;
    // L11^{-1} as split planes (NS pieces of the real part, then of the
    // imaginary part), row-major: B[n][k] = X[n][k] (k <= n), zero outside jb
    uint16_t* P = linv_planes + (long long)smp * 2 * SMAX * TB * TB;   // sample stride of the tensor map
    int ovf = 0;
    for (int t = tid; t < TB * TB; t += blockDim.x) {
        const int n = t / TB, k = t % TB;
        float2 v = make_float2(0.f, 0.f), vt = make_float2(0.f, 0.f);
        if (n < jb && k < jb) {
            v = S[n * DIAG_LD + k];
            vt = S[k * DIAG_LD + n];
        }
        X32[t] = v;
        X32[TB * TB + t] = vt;
        uint16_t pc[SMAX];
        split_n(v.x, pc, NS, f16 != 0, ovf);
        for (int q = 0; q < NS; ++q) P[plane_elem(q, TB, TB, n, k)] = pc[q];
        split_n(v.y, pc, NS, f16 != 0, ovf);
        for (int q = 0; q < NS; ++q) P[plane_elem(NS + q, TB, TB, n, k)] = pc[q];
    }
    if (ovf) atomicOr(err + kErrRange, 1);
}

// A21 (rows j0+jb .. j0+jb+M, columns j0 .. j0+jb) -> split planes, row-major
// [sample][2 NS][R][128], columns >= jb zero. Tile: 32 rows x 128 columns.
__global__ void __launch_bounds__(256) k_panel_planes(const float2* __restrict__ A0, long long ld, long long mstride,
                                                      int j0, int jb, int M, uint16_t* __restrict__ planes,
                                                      long long pstride, int R, int NS, int f16,
                                                      int* __restrict__ err) {
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
    uint16_t* P = planes + pstride * smp;
    int ovf = 0;
    for (int q = threadIdx.x; q < 32 * TB; q += blockDim.x) {
        int c = q % TB, rr = q / TB;
        if (r0 + rr >= M) continue;
        float2 v = t[c][rr];
        uint16_t pc[SMAX];
        split_n(v.x, pc, NS, f16 != 0, ovf);
        for (int q = 0; q < NS; ++q) P[plane_elem(q, R, TB, r0 + rr, c)] = pc[q];
        split_n(v.y, pc, NS, f16 != 0, ovf);
        for (int q = 0; q < NS; ++q) P[plane_elem(NS + q, R, TB, r0 + rr, c)] = pc[q];
    }
    if (ovf) atomicOr(err + kErrRange, 1);
}

// ---- solves with the factors: L D L^T x = b (one right-hand side per sample) ----------

// A right-hand side whose first lead_zero rows are zero (the immittance
// system's b = [I_E; 0; 0] in the order ZL, ZT, nodes) stays zero there
// through the forward sweep, so the blocks that end at or before lead_zero
// have nothing to do. Applies while *lead_step is 0 (the refinement's first
// solve, whose right-hand side is b itself); later residuals are dense.
TAGS_D bool lead_skip(const int* lead_step, int lead_zero, int block_end) {
    return lead_step && block_end <= lead_zero && *lead_step == 0;
}

// z_b = Linv_b * r_b for block b (128 rows), or Linv_b^T * r_b with
// transpose = 1, in place; one CTA of 512 threads per sample: four threads
// per output row, each a quarter of the row, reading the stored copy whose
// row index is contiguous across threads (the transpose of the one applied).
__global__ void __launch_bounds__(512) k_blk_inv_apply(const float2* __restrict__ linv32, long long lstride, int blk,
                                                       int jb, float2* __restrict__ x0, long long xstride,
                                                       int transpose, const int* __restrict__ active,
                                                       const int* __restrict__ lead_step, int lead_zero) {
    __shared__ float2 v[TB];
    __shared__ float2 part[4][TB];
    const int smp = blockIdx.x, tid = threadIdx.x, r = tid & (TB - 1), qt = tid >> 7;
    if (active && !active[smp]) return;              // the sample has finished refining
    if (lead_skip(lead_step, lead_zero, blk * TB + jb)) return;
    float2* x = x0 + xstride * smp + (long long)blk * TB;
    // M[r][k] is at Mt[k * TB + r]: Mt = Linv^T (row-major) for z = Linv r, Linv for z = Linv^T r
    const float2* Mt = linv32 + lstride * smp + (long long)blk * 2 * TB * TB + (transpose ? 0 : TB * TB);
    if (tid < TB) v[tid] = tid < jb ? x[tid] : make_float2(0.f, 0.f);
    __syncthreads();
    float2 acc = make_float2(0.f, 0.f);
    const int k0 = 32 * qt;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        float2 w[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) w[q] = Mt[(long long)(k0 + 16 * h + q) * TB + r];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc = ffmac(w[q], v[k0 + 16 * h + q], acc);
    }
    part[qt][r] = acc;
    __syncthreads();
    if (tid < jb) {
        const float2 a = part[0][tid], b = part[1][tid], c = part[2][tid], d = part[3][tid];
        x[tid] = make_float2((a.x + b.x) + (c.x + d.x), (a.y + b.y) + (c.y + d.y));
    }
}

// forward: x[i] -= sum_{k in block} L[i][k] x[k] for rows i below the block;
// a thread per row, 16 loads in flight, the block's x in shared memory
__global__ void __launch_bounds__(128) k_blk_fwd_update(const float2* __restrict__ A0, long long ld, long long mstride,
                                                        int N, int j0, int jb, float2* __restrict__ x0,
                                                        long long xstride, int zl_m, const int* __restrict__ active,
                                                        const int* __restrict__ lead_step, int lead_zero) {
    __shared__ float2 xs[TB];
    const int smp = blockIdx.y;
    if (active && !active[smp]) return;
    if (lead_skip(lead_step, lead_zero, j0 + jb)) return;
    float2* x = x0 + xstride * smp;
    if ((int)threadIdx.x < jb) xs[threadIdx.x] = x[j0 + threadIdx.x];
    __syncthreads();
    const int i = j0 + jb + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    if (j0 + jb <= zl_m && i >= zl_m && i < 2 * zl_m) return;      // L[ZT rows, ZL cols] = 0
    const float2* Ai = A0 + mstride * smp + i + ld * (long long)j0;
    float2 acc = make_float2(0.f, 0.f);
    int k = 0;
    for (; k + 16 <= jb; k += 16) {
        float2 w[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) w[q] = Ai[ld * (long long)(k + q)];
#pragma unroll
        for (int q = 0; q < 16; ++q) acc = ffmac(w[q], xs[k + q], acc);
    }
    for (; k < jb; ++k) acc = ffmac(Ai[ld * (long long)k], xs[k], acc);
    x[i] = fsub(x[i], acc);
}

// backward (L^T): x[r] -= sum_{c in block} L[c][r] x[c] for rows r above the
// block; a warp per 4 consecutive r, lanes over the block's rows of column r
// (coalesced), 16 loads in flight per lane.
__global__ void __launch_bounds__(256) k_blk_bwd_update(const float2* __restrict__ A0, long long ld, long long mstride,
                                                        int j0, int jb, float2* __restrict__ x0, long long xstride,
                                                        int zl_m, const int* __restrict__ active) {
    __shared__ float2 xs[TB];
    const int smp = blockIdx.y, lane = threadIdx.x & 31;
    if (active && !active[smp]) return;
    float2* x = x0 + xstride * smp;
    // zero beyond jb: the products there have zero weights, and 0 * NaN would not vanish
    if ((int)threadIdx.x < TB) xs[threadIdx.x] = (int)threadIdx.x < jb ? x[j0 + threadIdx.x] : make_float2(0.f, 0.f);
    __syncthreads();
    const int r0 = (blockIdx.x * 8 + (threadIdx.x >> 5)) * 4;
    if (r0 >= j0) return;
    const bool zero_cols = j0 >= zl_m && j0 + jb <= 2 * zl_m;         // L[ZT rows, ZL cols] = 0
    const float2* A = A0 + mstride * smp;
    float2 acc[4];
    float2 w[4][4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        acc[q] = make_float2(0.f, 0.f);
        const int r = r0 + q;
        const float2* col = A + ld * (long long)r + j0;
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int c = lane + 32 * t;
            w[q][t] = r < j0 && c < jb && !(zero_cols && r < zl_m) ? col[c] : make_float2(0.f, 0.f);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int t = 0; t < 4; ++t) acc[q] = ffmac(w[q][t], xs[lane + 32 * t], acc[q]);
    // butterfly: every lane ends with all four totals (lane q writes row r0 + q)
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int o = 16; o > 0; o >>= 1) {
            acc[q].x += __shfl_xor_sync(0xffffffffu, acc[q].x, o);
            acc[q].y += __shfl_xor_sync(0xffffffffu, acc[q].y, o);
        }
    if (lane < 4) {
        const int r = r0 + lane;
        float2 a = acc[0];
#pragma unroll
        for (int q = 1; q < 4; ++q)
            if (lane == q) a = acc[q];
        if (r < j0 && !(zero_cols && r < zl_m)) x[r] = fsub(x[r], a);
    }
}

// x[i] /= D[i] (D on the diagonal of the factored matrix)
__global__ void k_diag_scale(const float2* __restrict__ A0, long long ld, long long mstride, int N,
                             float2* __restrict__ x0, long long xstride, const int* __restrict__ active) {
    const int smp = blockIdx.y;
    if (active && !active[smp]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    const float2 d = A0[mstride * smp + i + ld * (long long)i];
    x0[xstride * smp + i] = fmulc(x0[xstride * smp + i], crecip_f(d));
}

// How the triangular solves run (tags_debug_solve_path): 0 the per-block
// kernels; 1 k_ldl_solve_cta (one CTA per sample); 2, 4, 8 k_ldl_solve_cl
// (a cluster of that many CTAs per sample); -1 (default) the larger of the
// cluster sizes 4 and 2 with G x samples <= SMs, else one CTA per sample: with
// the SMs full, one CTA per sample already saturates HBM and clusters only add
// barriers and waves (measured on the 1560-segment grid, 2048 samples in
// passes of 128: solves 104 ms against 113, 134 and 209 ms for G = 2, 4, 8),
// while a pass of few samples gets G SMs per sample (passes of 16: 51 ms with
// one CTA, 35, 24 and 34 ms for G = 2, 4, 8; passes of 32: 39 ms, then 27, 20
// and 41 ms). Paths 1.. need x in shared memory and fall back to the
// per-block kernels where it does not fit.
static int g_solve_path = -1;

// The whole solve of one sample (forward sweep, D, backward sweep) in one CTA
// of SOLVE_THREADS threads, x held in shared memory: one launch per solve, no
// grid-wide step between the blocks, and each SM keeps 16 loads per thread of
// L in flight. Every sum is formed in the same order as in the per-block
// kernels above (k_blk_inv_apply, k_blk_fwd_update, k_diag_scale,
// k_blk_bwd_update), so both paths give identical results. Dynamic shared
// memory: v (TB), part (4 TB), x (N) complex values.
constexpr int SOLVE_THREADS = 1024;
constexpr int SOLVE_SMEM_MAX = 200 * 1024;

__global__ void __launch_bounds__(SOLVE_THREADS, 1) k_ldl_solve_cta(
    const float2* __restrict__ A0, long long ld, long long mstride, int N, const float2* __restrict__ linv32,
    long long lstride, float2* __restrict__ x0, long long xstride, int zl_m, const int* __restrict__ active,
    const int* __restrict__ lead_step, int lead_zero, const int* __restrict__ nact, int few) {
    extern __shared__ float2 solve_sm[];
    float2* v = solve_sm;                          // the current block of x, zero beyond jb
    float2* part = solve_sm + TB;                  // 4 x TB partial sums of the block-inverse products
    float2* xs = solve_sm + 5 * TB;                // x
    const int smp = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (active && !active[smp]) return;            // the sample has finished refining
    if (nact && *nact <= few) return;              // few samples left: the cluster kernel takes them
    const float2* A = A0 + mstride * smp;
    const float2* Lv = linv32 + lstride * smp;
    float2* x = x0 + xstride * smp;
    const int nblk = (N + TB - 1) / TB;
    const int b0 = lead_step && *lead_step == 0 ? lead_zero / TB : 0;
    for (int i = tid; i < N; i += SOLVE_THREADS) xs[i] = x[i];
    __syncthreads();
    // z_b = M x_b for the block inverse M (M[r][k] at Mt[k TB + r]), as k_blk_inv_apply
    auto inv_apply = [&](const float2* Mt, int j0, int jb) {
        if (tid < TB) v[tid] = tid < jb ? xs[j0 + tid] : make_float2(0.f, 0.f);
        __syncthreads();
        if (tid < 4 * TB) {
            const int r = tid & (TB - 1), qt = tid >> 7, k0 = 32 * qt;
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float2 w[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) w[q] = Mt[(long long)(k0 + 16 * h + q) * TB + r];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc = ffmac(w[q], v[k0 + 16 * h + q], acc);
            }
            part[qt * TB + r] = acc;
        }
        __syncthreads();
        if (tid < jb) {
            const float2 a = part[tid], b = part[TB + tid], c = part[2 * TB + tid], d = part[3 * TB + tid];
            xs[j0 + tid] = make_float2((a.x + b.x) + (c.x + d.x), (a.y + b.y) + (c.y + d.y));
        }
        __syncthreads();
    };
    // forward: L y = b
    for (int b = b0; b < nblk; ++b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        inv_apply(Lv + (long long)b * 2 * TB * TB + TB * TB, j0, jb);
        // rows below the block, as k_blk_fwd_update; while the block lies in
        // the ZL columns the ZT rows are skipped (L[ZT rows, ZL cols] = 0)
        const int i_lo = j0 + jb;
        const bool band = i_lo <= zl_m;
        const int nhead = band ? zl_m - i_lo : N - i_lo;               // rows before the band (or all)
        const int nrows = band ? nhead + (N - 2 * zl_m) : N - i_lo;
        for (int t = tid; t < nrows; t += SOLVE_THREADS) {
            const int i = t < nhead ? i_lo + t : 2 * zl_m + (t - nhead);
            const float2* Ai = A + i + ld * (long long)j0;
            float2 acc = make_float2(0.f, 0.f);
            int k = 0;
            for (; k + 16 <= jb; k += 16) {
                float2 w[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) w[q] = Ai[ld * (long long)(k + q)];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc = ffmac(w[q], xs[j0 + k + q], acc);
            }
            for (; k < jb; ++k) acc = ffmac(Ai[ld * (long long)k], xs[j0 + k], acc);
            xs[i] = fsub(xs[i], acc);
        }
        __syncthreads();
    }
    // x /= D, as k_diag_scale
    for (int i = tid; i < N; i += SOLVE_THREADS) xs[i] = fmulc(xs[i], crecip_f(A[i + ld * (long long)i]));
    __syncthreads();
    // backward: L^T x = y
    for (int b = nblk - 1; b >= 0; --b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        inv_apply(Lv + (long long)b * 2 * TB * TB, j0, jb);
        if (j0 == 0) break;
        if (tid < TB) v[tid] = tid < jb ? xs[j0 + tid] : make_float2(0.f, 0.f);
        __syncthreads();
        // rows above the block, as k_blk_bwd_update: a warp per 4 consecutive r
        const bool zero_cols = j0 >= zl_m && j0 + jb <= 2 * zl_m;   // L[ZT rows, ZL cols] = 0
        for (int r0 = 4 * warp; r0 < j0; r0 += 4 * (SOLVE_THREADS / 32)) {
            float2 acc[4];
            float2 w[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = make_float2(0.f, 0.f);
                const int r = r0 + q;
                const float2* col = A + ld * (long long)r + j0;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int c = lane + 32 * t;
                    w[q][t] = r < j0 && c < jb && !(zero_cols && r < zl_m) ? col[c] : make_float2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int t = 0; t < 4; ++t) acc[q] = ffmac(w[q][t], v[lane + 32 * t], acc[q]);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                for (int o = 16; o > 0; o >>= 1) {
                    acc[q].x += __shfl_xor_sync(0xffffffffu, acc[q].x, o);
                    acc[q].y += __shfl_xor_sync(0xffffffffu, acc[q].y, o);
                }
            if (lane < 4) {
                const int r = r0 + lane;
                float2 a = acc[0];
#pragma unroll
                for (int q = 1; q < 4; ++q)
                    if (lane == q) a = acc[q];
                if (r < j0 && !(zero_cols && r < zl_m)) xs[r] = fsub(xs[r], a);
            }
        }
        __syncthreads();
    }
    for (int i = tid; i < N; i += SOLVE_THREADS) x[i] = xs[i];
}

// The solve of one sample on a cluster of G CTAs (G = 2, 4 or 8): CTA g owns
// the rows whose 32-row chunk index is g mod G, so for G = 4 it owns rows
// 32 g .. 32 g + 31 of every 128-row block, and keeps them in its shared
// memory. Per block and sweep: every CTA gathers the block's 128 values from
// their owners (distributed shared memory), applies the block inverse to its
// own rows, and after a cluster barrier gathers the new values and updates its
// own rows outside the block. Each row's sums are formed in the order of the
// per-block kernels (identical results); the tail steps of a refinement, with
// few samples still active, get G SMs per sample instead of one. Shared
// memory: v (TB), part (4 TB), x (N) complex values; the cluster barriers are
// the hardware's (all CTAs of a cluster run the same sequence).
template <int G>
__global__ void __launch_bounds__(SOLVE_THREADS, 1) k_ldl_solve_cl(
    const float2* __restrict__ A0, long long ld, long long mstride, int N, const float2* __restrict__ linv32,
    long long lstride, float2* __restrict__ x0, long long xstride, int zl_m, const int* __restrict__ active,
    const int* __restrict__ lead_step, int lead_zero, const int* __restrict__ nact, int few, int nb) {
    static_assert(G == 2 || G == 4 || G == 8, "cluster of 2, 4 or 8 CTAs");
    extern __shared__ float2 solve_sm[];
    __shared__ int s_smp;
    float2* v = solve_sm;
    float2* part = solve_sm + TB;
    float2* xs = solve_sm + 5 * TB;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = (int)cluster_rank();
    int smp = blockIdx.x / G;
    if (nact) {
        // a step with few samples left: cluster c takes the c-th active one
        // (every CTA of the cluster finds the same)
        const int na = *nact;
        if (na > few || smp >= na) return;         // the whole cluster
        if (warp == 0) {
            int seen = 0, found = -1;
            for (int q0 = 0; q0 < nb && found < 0; q0 += 32) {
                const int q = q0 + lane;
                const unsigned msk = __ballot_sync(0xffffffffu, q < nb && active[q] != 0);
                const int c = __popc(msk);
                if (smp < seen + c) {
                    unsigned mm = msk;
                    for (int k = smp - seen; k > 0; --k) mm &= mm - 1;
                    found = q0 + __ffs(mm) - 1;
                }
                seen += c;
            }
            if (lane == 0) s_smp = found;
        }
        __syncthreads();
        smp = s_smp;
        if (smp < 0) return;                       // the whole cluster
    } else if (active && !active[smp]) {
        return;                                    // the whole cluster: the sample has finished refining
    }
    const float2* A = A0 + mstride * smp;
    const float2* Lv = linv32 + lstride * smp;
    float2* x = x0 + xstride * smp;
    const int nblk = (N + TB - 1) / TB;
    const int b0 = lead_step && *lead_step == 0 ? lead_zero / TB : 0;
    auto own = [&](int i) { return ((i >> 5) & (G - 1)) == g; };
    for (int i = tid; i < N; i += SOLVE_THREADS)
        if (own(i)) xs[i] = x[i];
    __syncthreads();
    // v = the block's values x[j0 ..), zero beyond jb, read from their owners
    auto gather = [&](int j0, int jb) {
        if (tid < TB) {
            float2 val = make_float2(0.f, 0.f);
            if (tid < jb) {
                const int i = j0 + tid;
                const uint32_t a = mapa_cta(smem_u32(xs + i), (uint32_t)((i >> 5) & (G - 1)));
                asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(val.x), "=f"(val.y) : "r"(a) : "memory");
            }
            v[tid] = val;
        }
        __syncthreads();
    };
    // own rows of z_b = M v (M[r][k] at Mt[k TB + r]), as k_blk_inv_apply:
    // four quarter sums of 32 k each per row
    auto inv_apply = [&](const float2* Mt, int j0, int jb) {
        for (int t = tid; t < 4 * TB; t += SOLVE_THREADS) {
            const int r = t & (TB - 1), qt = t >> 7, k0 = 32 * qt;
            if (!own(j0 + r)) continue;
            float2 acc = make_float2(0.f, 0.f);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float2 w[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) w[q] = Mt[(long long)(k0 + 16 * h + q) * TB + r];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc = ffmac(w[q], v[k0 + 16 * h + q], acc);
            }
            part[qt * TB + r] = acc;
        }
        __syncthreads();
        if (tid < jb && own(j0 + tid)) {
            const float2 a = part[tid], b = part[TB + tid], c = part[2 * TB + tid], d = part[3 * TB + tid];
            xs[j0 + tid] = make_float2((a.x + b.x) + (c.x + d.x), (a.y + b.y) + (c.y + d.y));
        }
        __syncthreads();
    };
    // forward: L y = b
    for (int b = b0; b < nblk; ++b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        cluster_sync_all();                        // the block's rows are updated by all earlier blocks
        gather(j0, jb);
        inv_apply(Lv + (long long)b * 2 * TB * TB + TB * TB, j0, jb);
        cluster_sync_all();                        // every owner has applied the block inverse
        gather(j0, jb);
        // own rows below the block, as k_blk_fwd_update (ZT rows skipped while
        // the block lies in the ZL columns)
        const int i_lo = j0 + jb;
        const bool band = i_lo <= zl_m;
        int c0 = i_lo >> 5;
        c0 += (g - (c0 & (G - 1)) + G) & (G - 1);  // first own chunk at or after i_lo's
        for (int c = c0 + G * warp; 32 * c < N; c += G * (SOLVE_THREADS / 32)) {
            const int i = 32 * c + lane;
            if (i >= N || i < i_lo || (band && i >= zl_m && i < 2 * zl_m)) continue;
            const float2* Ai = A + i + ld * (long long)j0;
            float2 acc = make_float2(0.f, 0.f);
            int k = 0;
            for (; k + 16 <= jb; k += 16) {
                float2 w[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) w[q] = Ai[ld * (long long)(k + q)];
#pragma unroll
                for (int q = 0; q < 16; ++q) acc = ffmac(w[q], v[k + q], acc);
            }
            for (; k < jb; ++k) acc = ffmac(Ai[ld * (long long)k], v[k], acc);
            xs[i] = fsub(xs[i], acc);
        }
    }
    __syncthreads();
    // own rows /= D, as k_diag_scale
    for (int i = tid; i < N; i += SOLVE_THREADS)
        if (own(i)) xs[i] = fmulc(xs[i], crecip_f(A[i + ld * (long long)i]));
    __syncthreads();
    // backward: L^T x = y
    for (int b = nblk - 1; b >= 0; --b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        cluster_sync_all();                        // the block's rows are updated by all later blocks
        gather(j0, jb);
        inv_apply(Lv + (long long)b * 2 * TB * TB, j0, jb);
        cluster_sync_all();
        if (j0 == 0) break;
        gather(j0, jb);
        // own rows above the block, as k_blk_bwd_update: a warp per 4
        // consecutive rows, 8 groups per own chunk
        const bool zero_cols = j0 >= zl_m && j0 + jb <= 2 * zl_m;   // L[ZT rows, ZL cols] = 0
        const int ngroups = 8 * ((j0 / 32 - g + G - 1) / G);        // own chunks below j0, 8 groups each
        for (int q_idx = warp; q_idx < ngroups; q_idx += SOLVE_THREADS / 32) {
            const int r0 = 32 * (g + G * (q_idx >> 3)) + 4 * (q_idx & 7);
            float2 acc[4];
            float2 w[4][4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = make_float2(0.f, 0.f);
                const int r = r0 + q;
                const float2* col = A + ld * (long long)r + j0;
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int c = lane + 32 * t;
                    w[q][t] = r < j0 && c < jb && !(zero_cols && r < zl_m) ? col[c] : make_float2(0.f, 0.f);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int t = 0; t < 4; ++t) acc[q] = ffmac(w[q][t], v[lane + 32 * t], acc[q]);
#pragma unroll
            for (int q = 0; q < 4; ++q)
                for (int o = 16; o > 0; o >>= 1) {
                    acc[q].x += __shfl_xor_sync(0xffffffffu, acc[q].x, o);
                    acc[q].y += __shfl_xor_sync(0xffffffffu, acc[q].y, o);
                }
            if (lane < 4) {
                const int r = r0 + lane;
                float2 a = acc[0];
#pragma unroll
                for (int q = 1; q < 4; ++q)
                    if (lane == q) a = acc[q];
                if (r < j0 && !(zero_cols && r < zl_m)) xs[r] = fsub(xs[r], a);
            }
        }
    }
    // the last cluster barrier followed every read of another CTA's x
    for (int i = tid; i < N; i += SOLVE_THREADS)
        if (own(i)) x[i] = xs[i];
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

// 4-D map over planes [sample][nplanes][rows][128] bf16, box {32, 128, 1, 1}
// (64-byte rows, 64-byte swizzle: the K block of one pipeline stage).
// 5-D map over K-block-major planes [sample][plane][K / 32][rows][32] (16-bit),
// box {32, 128, 1, 1, 1}: one K block of 128 rows (64-byte rows, 64-byte swizzle).
int make_plane_map(CUtensorMap* map, void* base, int rows, int nplanes, int samples, int klen = TB,
                   int box_rows = TB) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return tags_fail(TAGS_E_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t kblk = (cuuint64_t)klen / BK;
    cuuint64_t dims[5] = {(cuuint64_t)BK, (cuuint64_t)rows, kblk, (cuuint64_t)nplanes, (cuuint64_t)samples};
    cuuint64_t strides[4] = {(cuuint64_t)BK * 2, (cuuint64_t)BK * 2 * rows, (cuuint64_t)BK * 2 * rows * kblk,
                             (cuuint64_t)BK * 2 * rows * kblk * nplanes};
    cuuint32_t box[5] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1, 1, 1};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 5, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        char msg[96];
        snprintf(msg, sizeof(msg), "cuTensorMapEncodeTiled failed (%d)", (int)r);
        return tags_fail(TAGS_E_CUDA, msg);
    }
    return 0;
}

}  // namespace

static long long linv32_stride(int N) { return (long long)((N + TB - 1) / TB) * 2 * TB * TB; }

// Workspace layout (sized for SMAX pieces): A21 planes, V planes (2 SMAX
// planes of N x 128 each per sample), L11^{-1} planes, D^{-1}, D^{-1/2}, FP32
// inverses of all diagonal blocks (and their transposes).
static long long plane_stride(int N) { return (long long)2 * SMAX * N * TB; }

// Workspace per sample: the block-column planes (rows of 128), the V planes
// of a group of up to GMAX panels (rows of KG), the L11^{-1} planes, D^{-1},
// D^{-1/2}, and the FP32 inverses of all diagonal blocks.
size_t tags_ldl_tc_workspace(int N, int batch) {
    size_t plane = (size_t)plane_stride(N) * 2;
    return (size_t)batch * ((1 + GMAX) * plane + (size_t)2 * SMAX * TB * TB * 2 + 2 * TB * sizeof(float2) +
                            (size_t)linv32_stride(N) * sizeof(float2)) + 1024;
}

static float2* linv32_of(void* ws, int N, int batch_cap) {
    const long long pstride = plane_stride(N);
    uint16_t* Lin = reinterpret_cast<uint16_t*>(ws) + (1 + GMAX) * pstride * batch_cap;
    float2* dinv = reinterpret_cast<float2*>(Lin + (long long)2 * SMAX * TB * TB * batch_cap);
    return dinv + 2LL * TB * batch_cap;
}

static int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 132;
    }
    return n;
}

template <int S, int MODE>
static int set_gemm_attr() {
    TAGS_CUDA_OK(cudaFuncSetAttribute(k_gemm_tc<S, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      GemmCfg<S>::SMEM));
    return 0;
}

// Two-SM GEMM: shared-memory size and the most clusters of two that can be
// resident at once (the persistent grid), per split form and product form.
static int g_pair_clusters[4][2] = {};

template <int S, int EMB>
static int set_gemm2_attr() {
    TAGS_CUDA_OK(cudaFuncSetAttribute(k_gemm_tc2<S, EMB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Gemm2Cfg<S, EMB>::SMEM));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * 76);
    cfg.blockDim = dim3(GEMM_THREADS);
    cfg.dynamicSmemBytes = Gemm2Cfg<S, EMB>::SMEM;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (void*)k_gemm_tc2<S, EMB>, &cfg) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 0;                        // two-SM products unavailable: the single-SM kernel is used
    }
    g_pair_clusters[S][EMB] = n;
    return 0;
}

// Cluster solves: shared-memory size and whether a cluster of G CTAs with the
// largest shared memory fits at all (else the one-CTA solve runs).
static bool g_solve_cl_ok[9] = {};

template <int G>
static int set_solve_cl_attr() {
    TAGS_CUDA_OK(cudaFuncSetAttribute(k_ldl_solve_cl<G>, cudaFuncAttributeMaxDynamicSharedMemorySize, SOLVE_SMEM_MAX));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(G);
    cfg.blockDim = dim3(SOLVE_THREADS);
    cfg.dynamicSmemBytes = SOLVE_SMEM_MAX;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, (void*)k_ldl_solve_cl<G>, &cfg) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 0;
    }
    g_solve_cl_ok[G] = n > 0;
    return 0;
}

// clusters: nb (one per sample), or, with nact, `few` (one per active sample
// of a step with at most `few` of them)
template <int G>
static int launch_solve_cl(const float2* A, long long ld, long long mstride, int N, const float2* L32, long long ls,
                           float2* x, long long xstride, int zl_m, const int* active, const int* lead_step,
                           int lead_zero, int nb, size_t smem, cudaStream_t st, const int* nact = nullptr,
                           int few = 0) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(G * (nact ? few : nb)));
    cfg.blockDim = dim3(SOLVE_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = G;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TAGS_CUDA_OK(cudaLaunchKernelEx(&cfg, k_ldl_solve_cl<G>, A, ld, mstride, N, L32, ls, x, xstride, zl_m, active,
                                    lead_step, lead_zero, nact, few, nb));
    tags_note_launch();
    return 0;
}

// Kernel attributes and the tensor-map encoder, set once per process before
// any launch (and so before any graph capture).
int tags_ldl_tc_prepare() {
    static std::once_flag once;
    static int rc = 0;
    std::call_once(once, [] {
        rc = set_gemm_attr<2, 0>();
        if (!rc) rc = set_gemm_attr<2, 1>();
        if (!rc) rc = set_gemm_attr<3, 0>();
        if (!rc) rc = set_gemm_attr<3, 1>();
        if (!rc) rc = set_gemm2_attr<2, 0>();
        if (!rc) rc = set_gemm2_attr<3, 0>();
        if (!rc) rc = set_gemm2_attr<2, 1>();
        if (!rc && cudaFuncSetAttribute(k_ldl_diag, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(TB * DIAG_LD * sizeof(float2))) != cudaSuccess)
            rc = tags_fail(TAGS_E_CUDA, "cudaFuncSetAttribute(k_ldl_diag) failed");
        if (!rc && cudaFuncSetAttribute(k_ldl_solve_cta, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        SOLVE_SMEM_MAX) != cudaSuccess)
            rc = tags_fail(TAGS_E_CUDA, "cudaFuncSetAttribute(k_ldl_solve_cta) failed");
        if (!rc) rc = set_solve_cl_attr<2>();
        if (!rc) rc = set_solve_cl_attr<4>();
        if (!rc) rc = set_solve_cl_attr<8>();
        if (!rc && !encode_fn()) rc = tags_fail(TAGS_E_CUDA, "cuTensorMapEncodeTiled is not available");
    });
    return rc;
}

template <int S, int MODE>
static int launch_gemm_m(const CUtensorMap& mA, const CUtensorMap& mB, const GemmArgs& g, cudaStream_t st) {
    const int total = g.tiles * g.nb;
    const int grid = total < num_sms() ? total : num_sms();
    if (grid <= 0) return 0;
    k_gemm_tc<S, MODE><<<grid, GEMM_THREADS, GemmCfg<S>::SMEM, st>>>(mA, mB, g);
    tags_note_launch();
    return 0;
}

// Mode-0 update on the two-SM kernel: clusters of two CTAs walk the pair
// tiles (mB: the operand map with 64-row boxes, each CTA's half of B; with
// EMB the 128-row map, each CTA's B rows of the real form).
template <int S, int EMB>
static int launch_gemm2_m(const CUtensorMap& mA, const CUtensorMap& mB, const GemmArgs& g, cudaStream_t st) {
    const int T = pair_rows(g);
    const long long total = (long long)pair_count(g, T) * g.nb;
    if (total <= 0) return 0;
    const int clusters = (int)std::min<long long>(total, g_pair_clusters[S][EMB]);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * clusters);
    cfg.blockDim = dim3(GEMM_THREADS);
    cfg.dynamicSmemBytes = Gemm2Cfg<S, EMB>::SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    TAGS_CUDA_OK(cudaLaunchKernelEx(&cfg, k_gemm_tc2<S, EMB>, mA, mB, g));
    tags_note_launch();
    return 0;
}

static bool pair_ready(int NS, int emb) { return g_pair_clusters[NS == 3 ? 3 : 2][emb ? 1 : 0] > 0; }

static int launch_gemm2(int NS, int emb, const CUtensorMap& mA, const CUtensorMap& mB, const GemmArgs& g,
                        cudaStream_t st) {
    if (emb) return launch_gemm2_m<2, 1>(mA, mB, g, st);
    return NS == 3 ? launch_gemm2_m<3, 0>(mA, mB, g, st) : launch_gemm2_m<2, 0>(mA, mB, g, st);
}

// One GEMM launch: K = 32 g.kblocks from the operand maps (mA, mB).
static int launch_gemm(int NS, const CUtensorMap& mA, const CUtensorMap& mB, const GemmArgs& g, cudaStream_t st) {
    if (NS == 3) return g.mode == 0 ? launch_gemm_m<3, 0>(mA, mB, g, st) : launch_gemm_m<3, 1>(mA, mB, g, st);
    return g.mode == 0 ? launch_gemm_m<2, 0>(mA, mB, g, st) : launch_gemm_m<2, 1>(mA, mB, g, st);
}

int tags_ldl_solve_c(const float2* A, int N, long long ld, long long mstride, int nb, int batch_cap, void* ws,
                     float2* x, long long xstride, int zl_m, cudaStream_t st, const int* active,
                     const int* lead_step, int lead_zero, const int* nact) {
    if (int e0 = tags_ldl_tc_prepare()) return e0;
    const float2* L32 = linv32_of(ws, N, batch_cap);
    const long long ls = linv32_stride(N);
    const int nblk = (N + TB - 1) / TB;
    int pf = tags_prof_begin(TAGS_PROF_LDL_SOLVE, st);
    const size_t smem = sizeof(float2) * (5 * TB + (size_t)N);
    int path = g_solve_path;
    bool split = false;
    if (path < 0) {
        path = 1;
        for (int G = 4; G >= 2; G /= 2)
            if ((long long)nb * G <= num_sms() && g_solve_cl_ok[G]) {
                path = G;
                break;
            }
        // one CTA per sample, except in steps with few samples left (known
        // on the device only): those run on clusters of four per sample
        split = path == 1 && nact && active && g_solve_cl_ok[4];
    }
    if (path >= 1 && smem <= (size_t)SOLVE_SMEM_MAX) {
        int e = 0;
        if (path >= 2 && g_solve_cl_ok[path]) {
            e = path == 2   ? launch_solve_cl<2>(A, ld, mstride, N, L32, ls, x, xstride, zl_m, active, lead_step,
                                                 lead_zero, nb, smem, st)
                : path == 4 ? launch_solve_cl<4>(A, ld, mstride, N, L32, ls, x, xstride, zl_m, active, lead_step,
                                                 lead_zero, nb, smem, st)
                            : launch_solve_cl<8>(A, ld, mstride, N, L32, ls, x, xstride, zl_m, active, lead_step,
                                                 lead_zero, nb, smem, st);
        } else {
            const int few = split ? num_sms() / 4 : 0;
            k_ldl_solve_cta<<<nb, SOLVE_THREADS, smem, st>>>(A, ld, mstride, N, L32, ls, x, xstride, zl_m, active,
                                                             lead_step, lead_zero, split ? nact : nullptr, few);
            tags_note_launch();
            if (split)
                e = launch_solve_cl<4>(A, ld, mstride, N, L32, ls, x, xstride, zl_m, active, lead_step, lead_zero, nb,
                                       smem, st, nact, few);
        }
        if (e) return e;
        tags_prof_end(TAGS_PROF_LDL_SOLVE, pf, st, 8.0 * N * (double)N * nb, 8.0 * N * (double)N * nb);
        TAGS_CUDA_OK(cudaGetLastError());
        return 0;
    }
    for (int b = 0; b < nblk; ++b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        k_blk_inv_apply<<<nb, 512, 0, st>>>(L32, ls, b, jb, x, xstride, 0, active, lead_step, lead_zero);
        const int rest = N - j0 - jb;
        if (rest > 0)
            k_blk_fwd_update<<<dim3((rest + 127) / 128, nb), 128, 0, st>>>(A, ld, mstride, N, j0, jb, x, xstride, zl_m,
                                                                         active, lead_step, lead_zero);
        tags_note_launch(rest > 0 ? 2 : 1);
    }
    k_diag_scale<<<dim3((N + 255) / 256, nb), 256, 0, st>>>(A, ld, mstride, N, x, xstride, active);
    tags_note_launch();
    for (int b = nblk - 1; b >= 0; --b) {
        const int j0 = b * TB, jb = N - j0 < TB ? N - j0 : TB;
        k_blk_inv_apply<<<nb, 512, 0, st>>>(L32, ls, b, jb, x, xstride, 1, active, nullptr, 0);
        if (j0 > 0)
            k_blk_bwd_update<<<dim3((j0 + 31) / 32, nb), 256, 0, st>>>(A, ld, mstride, j0, jb, x, xstride, zl_m,
                                                                     active);
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
                int* err, int zl_m, int pieces, int group_panels, cudaStream_t st, int pairs) {
    if (int e0 = tags_ldl_tc_prepare()) return e0;
    // split forms: 3 = bf16 x 3 pieces (6 products), 2 = bf16 x 2 (3 products),
    // TAGS_SPLIT_F16 = scaled fp16 x 2 (3 products, range-checked)
    const int f16 = pieces == TAGS_SPLIT_F16 ? 1 : 0;
    const int NS = pieces == 3 ? 3 : 2;
    // planes of this run use 2 NS of the 2 SMAX slots of each sample
    const long long pstride = plane_stride(N);           // block-column buffer, rows of 128
    const long long gstride = pstride * GMAX;             // group buffers, rows of KG
    uint16_t* A21p = reinterpret_cast<uint16_t*>(ws);
    uint16_t* Lg = A21p + pstride * batch_cap;            // V planes of the current group of panels
    uint16_t* Lin = Lg + gstride * batch_cap;
    float2* dinv = reinterpret_cast<float2*>(Lin + (long long)2 * SMAX * TB * TB * batch_cap);
    float2* dsq = dinv + (long long)TB * batch_cap;
    float2* L32 = linv32_of(ws, N, batch_cap);
    const long long ls = linv32_stride(N);
    // the maps see a sample stride of 2 SMAX planes: declare that many planes
    CUtensorMap mA21, mLg, mLin, mLg64;
    int e = make_plane_map(&mA21, A21p, N, 2 * SMAX, batch_cap);
    if (!e) e = make_plane_map(&mLg, Lg, N, 2 * SMAX, batch_cap, KG);
    if (!e) e = make_plane_map(&mLin, Lin, TB, 2 * SMAX, batch_cap);
    if (!e) e = make_plane_map(&mLg64, Lg, N, 2 * SMAX, batch_cap, KG, TB / 2);
    if (e) return e;
    // pairs: 0 one SM per tile; 1 two-SM tiles in complex form; 2 two-SM tiles
    // in real form (S = 2 only, else the complex form)
    const int emb = pairs == 2 && NS == 2 && pair_ready(NS, 1) ? 1 : 0;
    const bool use_pairs = pairs != 0 && pair_ready(NS, emb);
    TAGS_CUDA_OK(cudaMemsetAsync(info, 0, sizeof(int) * nb, st));
    const int G = group_panels < 1 ? 1 : (group_panels > GMAX ? GMAX : group_panels);

    auto base = [&]() {
        GemmArgs g{};
        g.nb = nb;
        g.Amat = A;
        g.ld = ld;
        g.mstride = mstride;
        g.dinv = dinv;
        g.dsq = dsq;
        g.pstride = gstride;
        g.npstride = pstride;
        g.R = N;
        g.err = err;
        g.f16 = f16;
        g.kblocks = KBLKS;
        return g;
    };
    // While the first zl_m columns (the ZL block of the ordering ZL, ZT,
    // nodes) are eliminated, rows/columns zl_m .. 2 zl_m (ZT) of the block
    // columns and of the trailing matrix stay exactly zero: with all
    // eliminated columns below `jend` <= zl_m, that band (relative to jend)
    // is skipped.
    auto band = [&](GemmArgs& g, int jend) {
        if (zl_m > 0 && jend <= zl_m) {
            g.zlo = zl_m - jend;
            g.zhi = 2 * zl_m - jend;
        }
    };
    auto diag = [&](int j0, int jb) {
        int pf = tags_prof_begin(TAGS_PROF_LDL_DIAG, st);
        k_ldl_diag<<<nb, 512, TB * DIAG_LD * sizeof(float2), st>>>(A, ld, mstride, j0, jb, Lin, dinv, dsq, info, L32,
                                                              ls, NS, f16, err);
        tags_prof_end(TAGS_PROF_LDL_DIAG, pf, st, 4.0 / 3.0 * jb * (double)jb * jb * nb, 16.0 * jb * jb * nb);
        tags_note_launch();
    };
    // W21 = A21 L11^{-T}, L21 = W21 D^{-1}, V21 = W21 D^{-1/2} for panel p of
    // the group starting at jg (columns jp = jg + 128 p .. jp + jb): FP32 L21
    // into A, V21 as split planes into the group buffer at rows (row - jg) and
    // columns 128 p ...
    auto panel = [&](int jg, int p, int jb, int rest, bool band_planes) {
        const int jp = jg + TB * p;
        GemmArgs g = base();
        band(g, jp + jb);
        g.band_planes = band_planes ? 1 : 0;
        g.M = rest;
        g.Nn = jb;
        g.mode = 1;
        g.tiles = (rest + TB - 1) / TB;
        g.row0 = jp + jb;
        g.col0 = jp;
        g.Lp = Lg;
        g.prow0 = jp + jb - jg;
        g.kcol0 = TB * p;
        g.neg_planes = use_pairs && emb;
        int pf = tags_prof_begin(TAGS_PROF_LDL_PANEL, st);
        int e1 = launch_gemm(NS, mA21, mLin, g, st);
        // triangular solve: r x jb unknowns against jb x jb (r = rest minus the band), 4 r jb^2 flops
        const double rp = rest - (double)(g.zhi - g.zlo);
        tags_prof_end(TAGS_PROF_LDL_PANEL, pf, st, 4.0 * rp * (double)jb * jb * nb,
                      (8.0 * rp * jb + 16.0 * rp * 128 * 2) * nb);
        return e1;
    };
    // C -= V V^T over the first `np` panels of the group starting at jg, on
    // rows (and, tri, columns) row0 .. row0 + M; the first tile column's new
    // values also become the next panel's block-column planes (Mn rows).
    auto update = [&](int jg, int np, int row0, int M, int Nn, bool tri, int Mn) {
        GemmArgs g = base();
        band(g, jg + TB * np);
        const int T = (M + TB - 1) / TB;
        g.M = M;
        g.Nn = Nn;
        g.mode = 0;
        g.tri = tri ? 1 : 0;
        g.tiles = tri ? T * (T + 1) / 2 : T;
        // the next panel (columns row0 ..) skips the band's rows while its
        // columns stay inside the ZL block: their planes are not written then
        const int jbn = std::min(TB, N - row0);
        g.np_band = zl_m > 0 && row0 + jbn <= zl_m ? 0 : 1;
        if (tri && g.zhi > g.zlo) {
            // tile rows/columns wholly inside the zero band leave the enumeration
            const int ba = (g.zlo + TB - 1) / TB, bb = std::min(T, g.zhi / TB);
            if (bb > ba) {
                g.ba = ba;
                g.bb = bb;
                g.tiles = tri_compact_count(T, ba, bb, Mn > 0, g.np_band != 0);
            }
        }
        g.row0 = row0;
        g.col0 = row0;
        g.off = row0 - jg;
        g.kblocks = KBLKS * np;
        g.Mn = Mn;
        g.Np = Mn > 0 ? A21p : nullptr;
        int pf = tags_prof_begin(TAGS_PROF_LDL_TRAIL, st);
        int e1 = use_pairs ? launch_gemm2(NS, emb, mLg, emb ? mLg : mLg64, g, st) : launch_gemm(NS, mLg, mLg, g, st);
        // rank-K update outside the zero band: 8 K cells flops (cells: the triangle or the block column)
        const double r = M - (double)(g.zhi - g.zlo);
        const double K = g.kblocks * BK;
        const double cells = tri ? 0.5 * r * (r + 1.0) : r * (double)Nn;
        tags_prof_end(TAGS_PROF_LDL_TRAIL, pf, st, 8.0 * K * cells * nb,
                      (16.0 * cells + 2.0 * r * K * 2.0 * NS) * nb);
        return e1;
    };

    // Groups of G panels of 128 columns: panel p of a group first takes the
    // update from panels 0 .. p-1 of its group on its own block column
    // (K = 128 p; this also yields its block-column planes), then its
    // diagonal block and panel GEMM; one trailing update with K = 128 G
    // follows each group.
    int jg = 0;
    bool done = false;
    while (!done && jg < N) {
        int np = 0;
        // the group's last update reaches column jg + 128 * panels: if that is past
        // the ZL block, it reads the band rows its panels skipped, so those panels
        // write zero planes there
        const int npg = std::min(G, (N - jg + TB - 1) / TB);
        const bool band_planes = zl_m > 0 && jg + TB * npg > zl_m;
        for (int p = 0; p < G; ++p) {
            const int jp = jg + TB * p;
            if (jp >= N) break;
            const int jb = N - jp < TB ? N - jp : TB;
            const int rest = N - jp - jb;
            if (p > 0) {
                e = update(jg, p, jp, N - jp, jb, false, rest);
                if (e) return e;
            }
            diag(jp, jb);
            np = p + 1;
            if (rest <= 0) {
                done = true;
                break;
            }
            if (jp == 0) {
                // later panels get their block column's planes from the update before them
                k_panel_planes<<<dim3((rest + 31) / 32, nb), 256, 0, st>>>(A, ld, mstride, jp, jb, rest, A21p,
                                                                           pstride, N, NS, f16, err);
                tags_note_launch();
            }
            e = panel(jg, p, jb, rest, band_planes);
            if (e) return e;
        }
        if (done) break;
        const int jt = jg + TB * np, rt = N - jt;
        if (rt <= 0) break;
        e = update(jg, np, jt, rt, rt, true, rt - (rt < TB ? rt : TB));
        if (e) return e;
        jg = jt;
    }
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

// ---- diagnostic entry points (declared in include/tags_gpu.h) -----------------------

static int debug_ldl_impl(tags_cdouble* a, tags_cdouble* b, int N, int nb, int pieces, int zl_m, int group);

static int g_debug_pairs = 0;     // tags_debug_ldl*: mode-0 updates on two-SM clusters

extern "C" int tags_debug_tc_pairs(int on) {
    if (on < 0 || on > 2) return tags_fail(TAGS_E_ARG, "tags_debug_tc_pairs: 0, 1 or 2");
    g_debug_pairs = on;
    return 0;
}

extern "C" int tags_debug_tri_tiles(int M, int zlo, int zhi, int planes, int planes_band, int* out, int cap) {
    if (M <= 0 || zlo < 0 || zhi < zlo || cap < 0 || (cap > 0 && !out))
        return tags_fail(TAGS_E_ARG, "tags_debug_tri_tiles: invalid argument");
    const int T = (M + TB - 1) / TB;
    const int ba = (zlo + TB - 1) / TB, bb = std::min(T, zhi / TB);
    if (zhi <= zlo || bb <= ba) {
        // no tile wholly inside a band: the kernel walks the full triangle
        const int n = T * (T + 1) / 2;
        for (int l = 0, I = 0; I < T; ++I)
            for (int J = 0; J <= I; ++J, ++l)
                if (l < cap) {
                    out[3 * l] = I;
                    out[3 * l + 1] = J;
                    out[3 * l + 2] = 0;
                }
        return n;
    }
    const int n = tri_compact_count(T, ba, bb, planes != 0, planes_band != 0);
    for (int l = 0; l < n && l < cap; ++l) {
        int I, J;
        bool skip;
        tri_compact_tile(l, ba, bb, planes != 0, planes_band != 0, I, J, skip);
        out[3 * l] = I;
        out[3 * l + 1] = J;
        out[3 * l + 2] = skip ? 1 : 0;
    }
    return n;
}

extern "C" int tags_debug_solve_path(int path) {
    if (path != -1 && path != 0 && path != 1 && path != 2 && path != 4 && path != 8)
        return tags_fail(TAGS_E_ARG, "tags_debug_solve_path: -1, 0, 1, 2, 4 or 8");
    g_solve_path = path;
    return 0;
}

extern "C" int tags_debug_tc_wait_limit(long long ns) {
    const unsigned long long v = ns > 0 ? (unsigned long long)ns : WAIT_NS;
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    TAGS_CUDA_OK(cudaDeviceSynchronize());          // no tensor-core kernel of this device is running
    TAGS_CUDA_OK(cudaMemcpyToSymbol(g_tc_wait_ns, &v, sizeof(v)));
    return 0;
}

extern "C" int tags_debug_ldl(tags_cdouble* a, int N, int nb, int pieces) {
    return debug_ldl_impl(a, nullptr, N, nb, pieces, 0, GMAX);
}

extern "C" int tags_debug_ldl_solve(tags_cdouble* a, tags_cdouble* b, int N, int nb, int pieces, int zl_m, int group) {
    if (!b || group < 1 || group > GMAX) return tags_fail(TAGS_E_ARG, "tags_debug_ldl_solve: invalid argument");
    return debug_ldl_impl(a, b, N, nb, pieces, zl_m, group);
}

static int debug_ldl_impl(tags_cdouble* a, tags_cdouble* b, int N, int nb, int pieces, int zl_m, int group) {
    if (!a || N <= 0 || nb <= 0 || zl_m < 0 || 2 * zl_m > N)
        return tags_fail(TAGS_E_ARG, "tags_debug_ldl: invalid argument");
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
        cudaMalloc(&err, 2 * sizeof(int)) != cudaSuccess) {
        rc = tags_fail(TAGS_E_NOMEM, "device allocation failed");
    }
    if (!rc && pieces != 2 && pieces != 3 && pieces != TAGS_SPLIT_F16)
        rc = tags_fail(TAGS_E_ARG, "tags_debug_ldl: pieces must be 2, 3 or 16");
    std::vector<float2> hf(NN * nb);
    float2* X = nullptr;
    std::vector<float2> hx;
    if (!rc && b) {
        if (cudaMalloc(&X, sizeof(float2) * N * nb) != cudaSuccess) rc = tags_fail(TAGS_E_NOMEM, "device allocation failed");
        hx.resize((size_t)N * nb);
        for (size_t q = 0; q < hx.size(); ++q) hx[q] = make_float2((float)b[q].re, (float)b[q].im);
    }
    if (!rc) {
        for (long long q = 0; q < NN * nb; ++q) hf[q] = make_float2((float)a[q].re, (float)a[q].im);
        cudaMemcpyAsync(A, hf.data(), sizeof(float2) * NN * nb, cudaMemcpyHostToDevice, st);
        // plane buffers start as NaN patterns: a read of a row no kernel wrote shows
        cudaMemsetAsync(ws, 0xFF, wsb, st);
        cudaMemsetAsync(err, 0, 2 * sizeof(int), st);
        rc = tags_ldl_tc(A, N, N, NN, nb, nb, ws, info, err, zl_m, pieces, group, st, g_debug_pairs);
        if (!rc && b) {
            cudaMemcpyAsync(X, hx.data(), sizeof(float2) * N * nb, cudaMemcpyHostToDevice, st);
            rc = tags_ldl_solve_c(A, N, N, NN, nb, nb, ws, X, N, zl_m, st);
            if (!rc) cudaMemcpyAsync(hx.data(), X, sizeof(float2) * N * nb, cudaMemcpyDeviceToHost, st);
        }
    }
    int herr[2] = {0, 0};
    std::vector<int> hinfo(nb, 0);
    if (!rc) {
        cudaMemcpyAsync(hf.data(), A, sizeof(float2) * NN * nb, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(herr, err, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * nb, cudaMemcpyDeviceToHost, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = tags_fail(TAGS_E_CUDA, "tags_debug_ldl: stream failed");
    }
    if (!rc) {
        for (long long q = 0; q < NN * nb; ++q) a[q] = {hf[q].x, hf[q].y};
        if (b)
            for (size_t q = 0; q < hx.size(); ++q) b[q] = {hx[q].x, hx[q].y};
        if (herr[0]) rc = tags_fail(TAGS_E_CUDA, "tags_debug_ldl: tensor-core wait ran out");
        else if (herr[1]) rc = tags_fail(TAGS_E_NONFINITE, "tags_debug_ldl: a value left the fp16 split's range");
        for (int q = 0; q < nb && !rc; ++q)
            if (hinfo[q]) rc = hinfo[q];
    }
    cudaFree(A);
    cudaFree(Ad);
    cudaFree(ws);
    cudaFree(info);
    cudaFree(err);
    if (X) cudaFree(X);
    return rc;
}
