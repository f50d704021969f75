// Post-processing of solved currents on GB300: the scalar potential, the
// magnetic vector potential, the electric field and the path voltage of the
// reference (src/electrode.c:434-668), and the closed-form mHEM ground
// potential that its examples evaluate (examples/visacro57emc01.c:406-430),
// batched over points x Laplace samples x injections.
//
// Electrode integrals. The reference integrates e^{-gamma r}/r (and its
// gradient) along every electrode with an adaptive 1-D cubature
// (src/electrode.c:199-218 and :495-520). Here each (point, electrode) pair
// gets a fixed rule from its geometry: the substitution
//     u = u0 + (d'/L) sinh v,   d' = max(d, 1e-6 L)
// about the foot u0 of the point on the electrode's line (d the distance to
// that line, L the electrode length) turns du / r into (d'/L) cosh v dv / r,
// which is smooth (and exactly dv / L when d' = d), so the near-singularity
// of points close to an electrode disappears. Gauss-Legendre panels of unit
// width in v, split further wherever |gamma| grows r by more than 1.5 across a
// panel, integrate what is left with 8 nodes per panel; against 1e-14 adaptive
// integrals over random geometries, frequencies and distances (1e-4 L to 5 L)
// the rule stays within 1e-12 relative.
//
// Path voltage. The reference integrates E . (p2 - p1) / |p2 - p1| over t in
// [0, 1] with a cubature whose integrand is itself a field cubature per
// electrode (src/electrode.c:599-668). The conservative part of E is exactly
// -grad u, so that part equals (u(p1) - u(p2)) / |p2 - p1|; the -s A part is a
// double integral of e^{-gamma r}/r between the path and each electrode, the
// pair integral of the impedance fill (fill.cu). Both are evaluated so here,
// without nesting; the result is the reference's (the path voltage divided by
// the path length).
//
// Layouts: currents il/it [sample][injection][electrode]; pot and gpd
// [sample][point][injection]; vecpot and efield [sample][point][injection][3];
// path voltages [sample][path][injection].
#include <algorithm>
#include <complex>
#include <cstring>
#include <mutex>
#include <vector>

#include "tags_common.cuh"
#include "tags_internal.h"
#include "../../include/tags_gpu.h"
#include "plan.h"

using zd = std::complex<double>;

namespace {

constexpr int FQ = 8;             // Gauss-Legendre nodes per panel
constexpr double FC = 1.5;        // largest |gamma| * (r growth) across a panel
constexpr int NB = 256;           // node buffer per warp (shared memory)
constexpr int FW = 4;             // warps per CTA
constexpr int RMAX = 4;           // injections per pass of a warp
constexpr int KMAX = 64;          // subpanels per unit panel (cap)

__constant__ double c_fx[FQ];     // nodes on [0, 1]
__constant__ double c_fw[FQ];     // weights on [0, 1]

struct NodeRec {
    double r, spar, jw;
};

struct WarpSmem {
    NodeRec node[NB];
    double lo[32], hi[32];
    int k[32], pre[32];
};

enum { WANT_POT = 1, WANT_VEC = 2, WANT_EF = 4 };

struct FieldArgs {
    const double* pts;      // P x 3
    const Seg* elec;        // m
    const double2* cur_t;   // [m][R][S]
    const double2* cur_l;   // [m][R][S]
    const double2* gamma;   // S
    const double2* kappa;   // S
    double mur;
    int P, m, R, S, G;      // G samples per warp (power of two <= 32)
    int want;
    int skip_pot;           // skip |it| < DBL_EPSILON in the potential (field convention)
    double2* pot;           // [S][P][R]
    double2* vec;           // [S][P][R][3]
    double2* ef;            // [S][P][R][3]
    int* status;
    unsigned long long* evals;  // node x sample evaluations (work counter)
    int nchunk;             // electrode chunks (warps per point and sample group)
    double2* part;          // [nchunk][S][P][R][7] raw sums: pot, vec xyz, ef xyz
};

TAGS_D double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

TAGS_D double2 shfl_xor2(double2 v, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
}

// One warp per (electrode chunk, point, group of G samples); lanes are
// (sample si = lane % G, node slice sub = lane / G). The rule's nodes of each
// electrode are built once per warp into shared memory and reused by all
// samples of the group. The electrode chunks spread one point's work over
// several warps so the grid fills the GPU evenly; k_fields_reduce adds them.
__global__ void __launch_bounds__(FW * 32) k_fields(FieldArgs a, int r0) {
    __shared__ WarpSmem sm_all[FW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    WarpSmem& sm = sm_all[warp];
    const int G = a.G, NS = 32 / G;
    const int ngroups = (a.S + G - 1) / G;
    const long long per_chunk = (long long)a.P * ngroups;
    const long long item_all = (long long)blockIdx.x * FW + warp;
    if (item_all >= per_chunk * a.nchunk) return;     // whole warp leaves together
    const int chunk = (int)(item_all / per_chunk);
    const long long item = item_all - (long long)chunk * per_chunk;
    const int p = (int)(item / ngroups), grp = (int)(item % ngroups);
    const int e_begin = (int)((long long)chunk * a.m / a.nchunk);
    const int e_end = (int)((long long)(chunk + 1) * a.m / a.nchunk);
    const int si = lane % G, sub = lane / G;
    const int smp = grp * G + si;
    const bool valid = smp < a.S;
    const int nr = min(RMAX, a.R - r0);
    const double2 gam = valid ? a.gamma[smp] : cz(0.0, 0.0);
    const double gmax = warp_max(valid ? sqrt(cabs2(gam)) : 0.0);
    const double P0 = a.pts[3 * p], P1 = a.pts[3 * p + 1], P2 = a.pts[3 * p + 2];
    const bool wv = (a.want & (WANT_VEC | WANT_EF)) != 0;

    double2 pot[RMAX], vec[RMAX][3], ef[RMAX][3];
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
        pot[r] = cz(0.0, 0.0);
#pragma unroll
        for (int c = 0; c < 3; ++c) { vec[r][c] = cz(0.0, 0.0); ef[r][c] = cz(0.0, 0.0); }
    }

    for (int e = e_begin; e < e_end; ++e) {
        const Seg& S = a.elec[e];
        const double D[3] = {S.b[0] - S.a[0], S.b[1] - S.a[1], S.b[2] - S.a[2]};
        const double L2 = D[0] * D[0] + D[1] * D[1] + D[2] * D[2];
        const double Lg = sqrt(L2);
        const double w0[3] = {P0 - S.a[0], P1 - S.a[1], P2 - S.a[2]};
        const double u0 = (w0[0] * D[0] + w0[1] * D[1] + w0[2] * D[2]) / L2;
        const double wp[3] = {w0[0] - u0 * D[0], w0[1] - u0 * D[1], w0[2] - u0 * D[2]};
        const double d = sqrt(wp[0] * wp[0] + wp[1] * wp[1] + wp[2] * wp[2]);
        const double dp = fmax(d, 1e-6 * Lg);
        // distance from the point to the segment itself
        const double uc = fmin(fmax(u0, 0.0), 1.0);
        const double du = (u0 - uc) * Lg;
        const double va = asinh(-u0 * Lg / dp), vb = asinh((1.0 - u0) * Lg / dp);
        // a point on the electrode (or a zero-length or non-finite record):
        // the integral diverges, the reference's result is undefined
        const bool degenerate = !(sqrt(d * d + du * du) > 1e-12 * Lg) || !isfinite(va) || !isfinite(vb);

        // unit panels: [va, 0] and [0, vb] when the foot is inside, else [va, vb]
        const bool split = va < 0.0 && vb > 0.0;
        const double la = split ? -va : vb - va, lb = split ? vb : 0.0;
        const int na = degenerate ? 0 : max(1, (int)ceil(la - 1e-12));
        const int nb2 = (degenerate || !split) ? 0 : max(1, (int)ceil(lb - 1e-12));
        const int nu = na + nb2;                       // <= 30 with d' >= 1e-6 L
        int kj = 0;
        if (lane < nu) {
            double lo, hi;
            if (lane < na) {
                const double h = la / na, base = va;
                lo = base + lane * h;
                hi = (lane == na - 1) ? (split ? 0.0 : vb) : base + (lane + 1) * h;
            } else {
                const int j = lane - na;
                const double h = lb / nb2;
                lo = j * h;
                hi = (j == nb2 - 1) ? vb : (j + 1) * h;
            }
            const double slo = dp * sinh(lo), shi = dp * sinh(hi);
            const double rlo = sqrt(d * d + slo * slo), rhi = sqrt(d * d + shi * shi);
            kj = min(KMAX, max(1, (int)ceil(gmax * fabs(rhi - rlo) / FC)));
            sm.lo[lane] = lo;
            sm.hi[lane] = hi;
            sm.k[lane] = kj;
        }
        // exclusive prefix of the subpanel counts
        int incl = kj;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane < nu) sm.pre[lane] = incl - kj;
        const int ksum = __shfl_sync(0xffffffffu, incl, 31);
        const int nodes = ksum * FQ;
        if (lane == 0 && a.evals) atomicAdd(a.evals, (unsigned long long)nodes * (unsigned long long)min(G, a.S - grp * G));
        __syncwarp();

        double2 J1 = cz(0.0, 0.0), Ap = cz(0.0, 0.0), Bp = cz(0.0, 0.0);
        for (int base = 0; base < nodes; base += NB) {
            const int cnt = min(NB, nodes - base);
            for (int t = lane; t < cnt; t += 32) {
                const int nid = base + t, spn = nid / FQ, q = nid - spn * FQ;
                int lo_i = 0, hi_i = nu - 1;                 // panel j with pre[j] <= spn
                while (lo_i < hi_i) {
                    int mid = (lo_i + hi_i + 1) >> 1;
                    if (sm.pre[mid] <= spn) lo_i = mid; else hi_i = mid - 1;
                }
                const int j = lo_i, kk = sm.k[j], loc = spn - sm.pre[j];
                const double h = (sm.hi[j] - sm.lo[j]) / kk;
                const double v = sm.lo[j] + (loc + c_fx[q]) * h;
                const double sv = sinh(v), cv = cosh(v);
                NodeRec nr_;
                nr_.spar = dp * sv;
                nr_.r = sqrt(d * d + nr_.spar * nr_.spar);
                nr_.jw = c_fw[q] * h * (dp / Lg) * cv;
                sm.node[t] = nr_;
            }
            __syncwarp();
            if (valid) {
                for (int t = sub; t < cnt; t += NS) {
                    const NodeRec nd = sm.node[t];
                    const double2 ex = cexp_d(cz(-gam.x * nd.r, -gam.y * nd.r));
                    const double ir = 1.0 / nd.r;
                    J1.x = fma(nd.jw * ir, ex.x, J1.x);
                    J1.y = fma(nd.jw * ir, ex.y, J1.y);
                    if (wv) {
                        // (1 + gamma r) e^{-gamma r} / r^3
                        const double2 f = cmul(cz(1.0 + gam.x * nd.r, gam.y * nd.r), ex);
                        const double sc = nd.jw * ir * ir * ir;
                        Ap.x = fma(sc, f.x, Ap.x);
                        Ap.y = fma(sc, f.y, Ap.y);
                        Bp.x = fma(sc * nd.spar, f.x, Bp.x);
                        Bp.y = fma(sc * nd.spar, f.y, Bp.y);
                    }
                }
            }
            __syncwarp();
        }
        // reduce over the node slices (lane bits >= log2 G)
        for (int o = G; o < 32; o <<= 1) {
            J1 = cadd(J1, shfl_xor2(J1, o));
            if (wv) {
                Ap = cadd(Ap, shfl_xor2(Ap, o));
                Bp = cadd(Bp, shfl_xor2(Bp, o));
            }
        }
        if (degenerate) {
            if (lane == 0) raise_status(a.status, TAGS_ST_DEGENERATE_PAIR);
            J1 = Ap = Bp = cz(nan(""), nan(""));
        }
        if (valid && sub == 0) {
            const double Dh[3] = {D[0] / Lg, D[1] / Lg, D[2] / Lg};
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                if (r >= nr) break;
                const long long ci = ((long long)e * a.R + r0 + r) * a.S + smp;
                if (a.want & (WANT_POT | WANT_EF)) {
                    const double2 ct = a.cur_t[ci];
                    const bool big = sqrt(cabs2(ct)) >= TAGS_DBL_EPSILON;
                    if (!a.skip_pot || big) pot[r] = cfma(ct, J1, pot[r]);
                    if ((a.want & WANT_EF) && big) {
                        const double2 ca = cmul(ct, Ap), cb = cmul(ct, Bp);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            ef[r][c].x += ca.x * wp[c] - cb.x * Dh[c];
                            ef[r][c].y += ca.y * wp[c] - cb.y * Dh[c];
                        }
                    }
                }
                if (a.want & WANT_VEC) {
                    const double2 cl = a.cur_l[ci];
                    if (sqrt(cabs2(cl)) >= TAGS_DBL_EPSILON) {
                        const double2 cj = cmul(cl, J1);
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            vec[r][c].x = fma(cj.x, D[c], vec[r][c].x);
                            vec[r][c].y = fma(cj.y, D[c], vec[r][c].y);
                        }
                    }
                }
            }
        }
        __syncwarp();
    }

    if (!valid || sub != 0) return;
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
        if (r >= nr) break;
        double2* o = a.part + ((((long long)chunk * a.S + smp) * a.P + p) * a.R + r0 + r) * 7;
        o[0] = pot[r];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            o[1 + c] = vec[r][c];
            o[4 + c] = ef[r][c];
        }
    }
}

// Sum of the electrode chunks and the scale factors: 1 / (4 pi kappa) for the
// potential and field, mur mu0 / (4 pi) for the vector potential.
__global__ void k_fields_reduce(FieldArgs a) {
    const long long n = (long long)a.S * a.P * a.R;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int smp = (int)(i / ((long long)a.P * a.R));
    double2 v[7];
#pragma unroll
    for (int c = 0; c < 7; ++c) v[c] = cz(0.0, 0.0);
    for (int ch = 0; ch < a.nchunk; ++ch) {
        const double2* q = a.part + ((long long)ch * n + i) * 7;
#pragma unroll
        for (int c = 0; c < 7; ++c) v[c] = cadd(v[c], q[c]);
    }
    const double2 i4pk = cdiv(cz(1.0, 0.0), cscale(a.kappa[smp], TAGS_FOUR_PI));
    const double u4pi = a.mur * TAGS_MU0 / TAGS_FOUR_PI;
    if (a.pot && (a.want & WANT_POT)) a.pot[i] = cmul(v[0], i4pk);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (a.vec && (a.want & WANT_VEC)) a.vec[3 * i + c] = cscale(v[1 + c], u4pi);
        if (a.ef && (a.want & WANT_EF)) a.ef[3 * i + c] = cmul(v[4 + c], i4pk);
    }
}

// Closed-form mHEM ground potential: warp per (point, sample group); the
// electrode terms log((r1 + r2 + L) / (r1 + r2 - L)) / L and the midpoint
// distance are computed once per warp (a lane per electrode) and shuffled to
// the samples.
__global__ void __launch_bounds__(FW * 32) k_gpd_mhem(const double* __restrict__ pts, const Seg* __restrict__ elec,
                                                      const double2* __restrict__ cur_t,
                                                      const double2* __restrict__ gamma,
                                                      const double2* __restrict__ kappa, int P, int m, int R,
                                                      int S, int G, int r0, double2* __restrict__ gpd) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NS = 32 / G;
    const int ngroups = (S + G - 1) / G;
    const long long item = (long long)blockIdx.x * FW + warp;
    if (item >= (long long)P * ngroups) return;
    const int p = (int)(item / ngroups), grp = (int)(item % ngroups);
    const int si = lane % G, sub = lane / G;
    const int smp = grp * G + si;
    const bool valid = smp < S;
    const int nr = min(RMAX, R - r0);
    const double2 gam = valid ? gamma[smp] : cz(0.0, 0.0);
    const double x = pts[3 * p], y = pts[3 * p + 1], z = pts[3 * p + 2];
    double2 acc[RMAX];
#pragma unroll
    for (int r = 0; r < RMAX; ++r) acc[r] = cz(0.0, 0.0);
    for (int e0 = 0; e0 < m; e0 += 32) {
        double rbar = 0.0, gv = 0.0;
        if (e0 + lane < m) {
            const Seg& s = elec[e0 + lane];
            // examples/visacro57emc01.c:417-421 (vector_length = root of the summed squares)
            const double dm0 = x - s.mid[0], dm1 = y - s.mid[1], dm2 = z - s.mid[2];
            const double da0 = x - s.a[0], da1 = y - s.a[1], da2 = z - s.a[2];
            const double db0 = x - s.b[0], db1 = y - s.b[1], db2 = z - s.b[2];
            rbar = sqrt(dm0 * dm0 + dm1 * dm1 + dm2 * dm2);
            const double r1 = sqrt(da0 * da0 + da1 * da1 + da2 * da2);
            const double r2 = sqrt(db0 * db0 + db1 * db1 + db2 * db2);
            const double r0v = (r1 + r2 + s.len) / (r1 + r2 - s.len);
            gv = log(r0v) / s.len;
        }
        const int cnt = min(32, m - e0);
        // the same trip count in every lane, so the shuffles stay warp-uniform
        for (int jb = 0; jb < cnt; jb += NS) {
            const int j = jb + sub;
            const double rb = __shfl_sync(0xffffffffu, rbar, j & 31);
            const double g = __shfl_sync(0xffffffffu, gv, j & 31);
            if (!valid || j >= cnt) continue;
            const double2 ex = cexp_d(cz(-gam.x * rb, -gam.y * rb));
            const double2 eg = cscale(ex, g);
#pragma unroll
            for (int r = 0; r < RMAX; ++r) {
                if (r >= nr) break;
                acc[r] = cfma(cur_t[((long long)(e0 + j) * R + r0 + r) * S + smp], eg, acc[r]);
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int r = 0; r < RMAX; ++r)
        for (int o = G; o < 32; o <<= 1) acc[r] = cadd(acc[r], shfl_xor2(acc[r], o));
    if (!valid || sub != 0) return;
    const double2 i4pk = cdiv(cz(1.0, 0.0), cscale(kappa[smp], TAGS_FOUR_PI));
#pragma unroll
    for (int r = 0; r < RMAX; ++r) {
        if (r >= nr) break;
        gpd[((long long)smp * P + p) * R + r0 + r] = cmul(i4pk, acc[r]);
    }
}

// [S][R][m] -> [m][R][S]
__global__ void k_cur_transpose(const double2* __restrict__ in, double2* __restrict__ out, int S, int R, int m) {
    const long long n = (long long)S * R * m;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(i % m);
        const long long sr = i / m;
        const int r = (int)(sr % R), s = (int)(sr / R);
        out[((long long)e * R + r) * S + s] = in[i];
    }
}

// Path voltage from the end-point potentials and the path/electrode pair
// integrals jj[(s * NL + l) * m + e] (unscaled double integrals over [0,1]^2).
__global__ void k_voltage(const double* __restrict__ paths, int NL, const Seg* __restrict__ elec, int m,
                          const double2* __restrict__ cur_l, const double2* __restrict__ upts,
                          const double2* __restrict__ jj, const double2* __restrict__ svals, double mur, int R,
                          int S, double2* __restrict__ v) {
    const long long n = (long long)S * NL * R;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = (int)(i % R);
    const long long sl = i / R;
    const int l = (int)(sl % NL), s = (int)(sl / NL);
    const double* pa = paths + 6LL * l;
    const double dx[3] = {pa[3] - pa[0], pa[4] - pa[1], pa[5] - pa[2]};
    const double len2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    if (len2 < TAGS_DBL_EPSILON) {
        // src/electrode.c:612: the integrand fails for a path this short
        v[i] = cz(nan(""), nan(""));
        return;
    }
    const double len = sqrt(len2);
    // potentials of the two ends: upts[(s * 2NL + 2l + {0,1}) * R + r]
    const double2 u1 = upts[((long long)s * 2 * NL + 2 * l) * R + r];
    const double2 u2 = upts[((long long)s * 2 * NL + 2 * l + 1) * R + r];
    double2 out = cscale(csub(u1, u2), 1.0 / len);
    const double2 sv = svals[s];
    if (sqrt(cabs2(sv)) > TAGS_DBL_EPSILON) {
        double2 acc = cz(0.0, 0.0);
        const double2* jrow = jj + ((long long)s * NL + l) * m;
        for (int e = 0; e < m; ++e) {
            const double2 cl = cur_l[((long long)e * R + r) * S + s];
            if (sqrt(cabs2(cl)) < TAGS_DBL_EPSILON) continue;
            const Seg& g = elec[e];
            const double proj = ((g.b[0] - g.a[0]) * dx[0] + (g.b[1] - g.a[1]) * dx[1] + (g.b[2] - g.a[2]) * dx[2]) / len;
            acc = cfma(cscale(cl, proj), jrow[e], acc);
        }
        out = csub(out, cscale(cmul(sv, acc), mur * TAGS_MU0 / TAGS_FOUR_PI));
    }
    v[i] = out;
}

bool g_tables_ready[64] = {};
unsigned long long* g_evals[64] = {};   // per-device work counter

int fields_tables(int dev) {
    if (dev < 0 || dev >= 64) return TAGS_E_CUDA;
    if (g_tables_ready[dev]) return 0;
    double x[FQ], w[FQ];
    tags_gauss_legendre(FQ, x, w);
    TAGS_CUDA_OK(cudaMemcpyToSymbol(c_fx, x, sizeof(x)));
    TAGS_CUDA_OK(cudaMemcpyToSymbol(c_fw, w, sizeof(w)));
    TAGS_CUDA_OK(cudaMalloc(&g_evals[dev], sizeof(unsigned long long)));
    TAGS_CUDA_OK(cudaMemset(g_evals[dev], 0, sizeof(unsigned long long)));
    g_tables_ready[dev] = true;
    return 0;
}

int samples_per_warp(size_t S) {
    int g = 1;
    while (g < 32 && (size_t)g < S) g <<= 1;
    return g;
}

// Samples per device pass, so the buffers of one pass stay near 1.5 GB.
size_t chunk_samples(size_t S, size_t per_sample) {
    size_t c = per_sample ? (size_t)1.5e9 / per_sample : S;
    return std::max<size_t>(1, std::min(S, c));
}

inline double2 D2(tags_cdouble v) { return make_double2(v.re, v.im); }

// Electrode chunks per (point, sample group): enough warps for about six
// waves of two 4-warp CTAs per SM (the register-limited residency), at least
// 16 electrodes per chunk, and partial sums of at most `part_cap` bytes.
int field_chunks(size_t P, size_t ns, size_t R, size_t m, size_t part_cap) {
    const size_t G = (size_t)samples_per_warp(ns);
    const size_t warps = P * ((ns + G - 1) / G);
    const size_t target = 152 * 8 * 6;
    size_t c = warps ? (target + warps - 1) / warps : 1;
    c = std::min<size_t>(c, std::max<size_t>(1, m / 16));
    c = std::min<size_t>(c, 64);
    const size_t per = 7 * sizeof(double2) * P * R * ns;
    if (per) c = std::min<size_t>(c, std::max<size_t>(1, part_cap / per));
    return (int)std::max<size_t>(1, c);
}

int launch_fields(const FieldArgs& base, cudaStream_t st) {
    const int ngroups = (base.S + base.G - 1) / base.G;
    const long long items = (long long)base.P * ngroups * base.nchunk;
    if (items == 0 || base.m == 0) return 0;
    const long long blocks = (items + FW - 1) / FW;
    if (blocks > 0x7fffffffLL) return tags_fail(TAGS_E_ARG, "too many points x samples for one launch");
    const int pf = tags_prof_begin(TAGS_PROF_FIELDS, st);
    for (int r0 = 0; r0 < base.R; r0 += RMAX) {
        k_fields<<<(unsigned)blocks, FW * 32, 0, st>>>(base, r0);
        tags_note_launch();
        TAGS_CUDA_OK(cudaGetLastError());
    }
    const long long n = (long long)base.S * base.P * base.R;
    k_fields_reduce<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(base);
    tags_prof_end(TAGS_PROF_FIELDS, pf, st, 0.0, 0.0);
    tags_note_launch();
    TAGS_CUDA_OK(cudaGetLastError());
    return 0;
}

struct FieldsIn {
    const double* points;
    size_t P;
    const Electrode* elec;
    size_t m;
    const tags_cdouble* il;
    const tags_cdouble* it;
    size_t R, S;
    const tags_cdouble* gamma;
    const tags_cdouble* kappa;
    double mur;
    int want, skip_pot;
    tags_cdouble *pot, *vec, *ef;
};

// Host driver of k_fields over sample chunks (slots 10..14 of the context's
// scratch; the caller holds the drop-in lock).
int fields_run(const FieldsIn& in) {
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    if (int e = fields_tables(c->device)) return e;
    cudaStream_t st = c->stream;
    const size_t P = in.P, m = in.m, R = in.R, S = in.S;
    const size_t per_sample = sizeof(double2) * (4 * R * m + P * R * 7 + 2);
    const size_t cs = chunk_samples(S, per_sample);
    const int nchunk = field_chunks(P, cs, R, m, (size_t)1e9);
    double* d_pts = (double*)c->scratch(10, sizeof(double) * 3 * P + 16);
    Seg* d_el = (Seg*)c->scratch(11, sizeof(Seg) * m + 16);
    double2* d_cur = (double2*)c->scratch(12, sizeof(double2) * 4 * R * m * cs + 16);
    double2* d_out = (double2*)c->scratch(13, sizeof(double2) * 7 * P * R * cs * (1 + (size_t)nchunk) + 16);
    double2* d_gk = (double2*)c->scratch(14, sizeof(double2) * 2 * cs + 16);
    if (!d_pts || !d_el || !d_cur || !d_out || !d_gk) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    TAGS_CUDA_OK(cudaMemcpyAsync(d_pts, in.points, sizeof(double) * 3 * P, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_el, in.elec, sizeof(Seg) * m, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemsetAsync(c->status, 0, sizeof(int), st));
    for (size_t s0 = 0; s0 < S; s0 += cs) {
        const size_t ns = std::min(cs, S - s0);
        const size_t nc = R * m * ns;
        double2* raw_t = d_cur;               // [ns][R][m] as given
        double2* raw_l = d_cur + nc;
        double2* cur_t = d_cur + 2 * nc;      // transposed [m][R][ns]
        double2* cur_l = d_cur + 3 * nc;
        const bool need_t = (in.want & (WANT_POT | WANT_EF)) != 0, need_l = (in.want & WANT_VEC) != 0;
        const int tb = 256, tg = (int)std::min<size_t>((nc + tb - 1) / tb, 152 * 16);
        if (need_t) {
            TAGS_CUDA_OK(cudaMemcpyAsync(raw_t, in.it + s0 * R * m, sizeof(double2) * nc, cudaMemcpyHostToDevice, st));
            k_cur_transpose<<<tg, tb, 0, st>>>(raw_t, cur_t, (int)ns, (int)R, (int)m);
            tags_note_launch();
            TAGS_CUDA_OK(cudaGetLastError());
        }
        if (need_l) {
            TAGS_CUDA_OK(cudaMemcpyAsync(raw_l, in.il + s0 * R * m, sizeof(double2) * nc, cudaMemcpyHostToDevice, st));
            k_cur_transpose<<<tg, tb, 0, st>>>(raw_l, cur_l, (int)ns, (int)R, (int)m);
            tags_note_launch();
            TAGS_CUDA_OK(cudaGetLastError());
        }
        TAGS_CUDA_OK(cudaMemcpyAsync(d_gk, in.gamma + s0, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_gk + ns, in.kappa + s0, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
        FieldArgs a{};
        a.pts = d_pts;
        a.elec = d_el;
        a.cur_t = cur_t;
        a.cur_l = cur_l;
        a.gamma = d_gk;
        a.kappa = d_gk + ns;
        a.mur = in.mur;
        a.P = (int)P;
        a.m = (int)m;
        a.R = (int)R;
        a.S = (int)ns;
        a.G = samples_per_warp(ns);
        a.want = in.want;
        a.skip_pot = in.skip_pot;
        a.pot = d_out;
        a.vec = d_out + P * R * ns;
        a.ef = d_out + 4 * P * R * ns;
        a.status = c->status;
        a.evals = g_evals[c->device];
        a.nchunk = nchunk;
        a.part = d_out + 7 * P * R * ns;
        if (int e = launch_fields(a, st)) return e;
        if (in.pot && (in.want & WANT_POT))
            TAGS_CUDA_OK(cudaMemcpyAsync(in.pot + s0 * P * R, a.pot, sizeof(double2) * P * R * ns,
                                         cudaMemcpyDeviceToHost, st));
        if (in.vec && (in.want & WANT_VEC))
            TAGS_CUDA_OK(cudaMemcpyAsync(in.vec + 3 * s0 * P * R, a.vec, sizeof(double2) * 3 * P * R * ns,
                                         cudaMemcpyDeviceToHost, st));
        if (in.ef && (in.want & WANT_EF))
            TAGS_CUDA_OK(cudaMemcpyAsync(in.ef + 3 * s0 * P * R, a.ef, sizeof(double2) * 3 * P * R * ns,
                                         cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    int status = 0;
    TAGS_CUDA_OK(cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    TAGS_CUDA_OK(cudaStreamSynchronize(st));
    return status & TAGS_ST_DEGENERATE_PAIR ? TAGS_E_GEOMETRY : 0;
}

bool bad_sizes(size_t P, size_t m, size_t R, size_t S) {
    return P > 0x7fffffffu || m > 0x7fffffffu || R > 0x7fffffffu || S > 0x7fffffffu;
}

}  // namespace

// ---- batched API -------------------------------------------------------------

extern "C" int tags_fields_batch(const double* points, size_t num_points, const Electrode* electrodes,
                                 size_t num_electrodes, const tags_cdouble* il, const tags_cdouble* it, size_t nrhs,
                                 size_t nsamples, const tags_cdouble* gamma, const tags_cdouble* kappa, double mur,
                                 tags_cdouble* pot, tags_cdouble* vecpot, tags_cdouble* efield) {
    if (num_points == 0 || nrhs == 0 || nsamples == 0) return 0;
    if (!points || !gamma || !kappa || (num_electrodes && !electrodes))
        return tags_fail(TAGS_E_ARG, "null pointer argument");
    if (bad_sizes(num_points, num_electrodes, nrhs, nsamples)) return tags_fail(TAGS_E_ARG, "size out of range");
    int want = (pot ? WANT_POT : 0) | (vecpot ? WANT_VEC : 0) | (efield ? WANT_EF : 0);
    if (((want & (WANT_POT | WANT_EF)) && !it) || ((want & WANT_VEC) && !il))
        return tags_fail(TAGS_E_ARG, "null current array");
    if (num_electrodes == 0) {
        const size_t n = num_points * nrhs * nsamples;
        if (pot) memset(pot, 0, sizeof(tags_cdouble) * n);
        if (vecpot) memset(vecpot, 0, sizeof(tags_cdouble) * 3 * n);
        if (efield) memset(efield, 0, sizeof(tags_cdouble) * 3 * n);
        return 0;
    }
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    FieldsIn in{points, num_points, electrodes, num_electrodes, il, it, nrhs, nsamples, gamma, kappa, mur,
                want, 0, pot, vecpot, efield};
    return fields_run(in);
}

extern "C" int tags_gpd_mhem_batch(const double* points, size_t num_points, const Electrode* electrodes,
                                   size_t num_electrodes, const tags_cdouble* it, size_t nrhs, size_t nsamples,
                                   const tags_cdouble* gamma, const tags_cdouble* kappa, tags_cdouble* gpd) {
    if (num_points == 0 || nrhs == 0 || nsamples == 0) return 0;
    if (!points || !gamma || !kappa || !gpd || (num_electrodes && (!electrodes || !it)))
        return tags_fail(TAGS_E_ARG, "null pointer argument");
    if (bad_sizes(num_points, num_electrodes, nrhs, nsamples)) return tags_fail(TAGS_E_ARG, "size out of range");
    if (num_electrodes == 0) {
        memset(gpd, 0, sizeof(tags_cdouble) * num_points * nrhs * nsamples);
        return 0;
    }
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    cudaStream_t st = c->stream;
    const size_t P = num_points, m = num_electrodes, R = nrhs, S = nsamples;
    const size_t cs = chunk_samples(S, sizeof(double2) * (2 * R * m + P * R + 2));
    double* d_pts = (double*)c->scratch(10, sizeof(double) * 3 * P + 16);
    Seg* d_el = (Seg*)c->scratch(11, sizeof(Seg) * m + 16);
    double2* d_cur = (double2*)c->scratch(12, sizeof(double2) * 2 * R * m * cs + 16);
    double2* d_out = (double2*)c->scratch(13, sizeof(double2) * P * R * cs + 16);
    double2* d_gk = (double2*)c->scratch(14, sizeof(double2) * 2 * cs + 16);
    if (!d_pts || !d_el || !d_cur || !d_out || !d_gk) return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    TAGS_CUDA_OK(cudaMemcpyAsync(d_pts, points, sizeof(double) * 3 * P, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_el, electrodes, sizeof(Seg) * m, cudaMemcpyHostToDevice, st));
    for (size_t s0 = 0; s0 < S; s0 += cs) {
        const size_t ns = std::min(cs, S - s0), nc = R * m * ns;
        TAGS_CUDA_OK(cudaMemcpyAsync(d_cur, it + s0 * R * m, sizeof(double2) * nc, cudaMemcpyHostToDevice, st));
        const int tb = 256, tg = (int)std::min<size_t>((nc + tb - 1) / tb, 152 * 16);
        k_cur_transpose<<<tg, tb, 0, st>>>(d_cur, d_cur + nc, (int)ns, (int)R, (int)m);
        tags_note_launch();
        TAGS_CUDA_OK(cudaGetLastError());
        TAGS_CUDA_OK(cudaMemcpyAsync(d_gk, gamma + s0, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_gk + ns, kappa + s0, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
        const int G = samples_per_warp(ns);
        const long long items = (long long)P * ((ns + G - 1) / G);
        const long long blocks = (items + FW - 1) / FW;
        if (blocks > 0x7fffffffLL) return tags_fail(TAGS_E_ARG, "too many points x samples for one launch");
        for (int r0 = 0; r0 < (int)R; r0 += RMAX) {
            k_gpd_mhem<<<(unsigned)blocks, FW * 32, 0, st>>>(d_pts, d_el, d_cur + nc, d_gk, d_gk + ns, (int)P, (int)m,
                                                             (int)R, (int)ns, G, r0, d_out);
            tags_note_launch();
            TAGS_CUDA_OK(cudaGetLastError());
        }
        TAGS_CUDA_OK(cudaMemcpyAsync(gpd + s0 * P * R, d_out, sizeof(double2) * P * R * ns, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    return 0;
}

extern "C" int tags_voltage_batch(const double* paths, size_t num_paths, const Electrode* electrodes,
                                  size_t num_electrodes, const tags_cdouble* il, const tags_cdouble* it, size_t nrhs,
                                  size_t nsamples, const tags_cdouble* gamma, const tags_cdouble* s,
                                  const tags_cdouble* kappa, double mur, tags_cdouble* v) {
    if (num_paths == 0 || nrhs == 0 || nsamples == 0) return 0;
    if (!paths || !gamma || !s || !kappa || !v || (num_electrodes && (!electrodes || !il || !it)))
        return tags_fail(TAGS_E_ARG, "null pointer argument");
    if (bad_sizes(2 * num_paths, num_electrodes, nrhs, nsamples)) return tags_fail(TAGS_E_ARG, "size out of range");
    const size_t NL = num_paths, m = num_electrodes, R = nrhs, S = nsamples;
    // potentials of the path ends with the field's convention (|it| below
    // DBL_EPSILON skipped, src/electrode.c:542)
    std::vector<tags_cdouble> upts(2 * NL * R * S);
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    if (m > 0) {
        FieldsIn in{paths, 2 * NL, electrodes, m, il, it, R, S, gamma, kappa, mur, WANT_POT, 1,
                    upts.data(), nullptr, nullptr};
        int e = fields_run(in);
        if (e && e != TAGS_E_GEOMETRY) return e;
    }
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    if (int e = fields_tables(c->device)) return e;
    cudaStream_t st = c->stream;
    const size_t cs =
        std::min<size_t>(65535, chunk_samples(S, sizeof(double2) * (2 * R * m + NL * m + 3 * NL * R + 4)));
    Seg* d_el = (Seg*)c->scratch(11, sizeof(Seg) * (m + NL) + 16);
    double* d_paths = (double*)c->scratch(10, sizeof(double) * 6 * NL + 16);
    double2* d_cur = (double2*)c->scratch(12, sizeof(double2) * 2 * R * m * cs + 16);
    double2* d_jj = (double2*)c->scratch(13, sizeof(double2) * (NL * m + 3 * NL * R) * cs + 16);
    double2* d_gk = (double2*)c->scratch(14, sizeof(double2) * 3 * cs + 16);
    SampleCoef* d_coef = (SampleCoef*)c->scratch(15, sizeof(SampleCoef) * cs + 16);
    if (!d_el || !d_paths || !d_cur || !d_jj || !d_gk || !d_coef)
        return tags_fail(TAGS_E_NOMEM, "device allocation failed");
    // paths as segment records after the electrodes (radius 0)
    std::vector<Seg> segs(m + NL);
    if (m) memcpy(segs.data(), electrodes, sizeof(Seg) * m);
    for (size_t l = 0; l < NL; ++l) {
        Seg& g = segs[m + l];
        const double* pa = paths + 6 * l;
        double len2 = 0.0;
        for (int k = 0; k < 3; ++k) {
            g.a[k] = pa[k];
            g.b[k] = pa[3 + k];
            g.mid[k] = (pa[k] + pa[3 + k]) / 2.0;
            len2 += (pa[3 + k] - pa[k]) * (pa[3 + k] - pa[k]);
        }
        g.len = sqrt(len2);
        g.radius = 0.0;
    }
    TAGS_CUDA_OK(cudaMemcpyAsync(d_el, segs.data(), sizeof(Seg) * (m + NL), cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemcpyAsync(d_paths, paths, sizeof(double) * 6 * NL, cudaMemcpyHostToDevice, st));
    TAGS_CUDA_OK(cudaMemsetAsync(c->status, 0, sizeof(int), st));
    for (size_t s0 = 0; s0 < S; s0 += cs) {
        const size_t ns = std::min(cs, S - s0), nc = R * m * ns;
        double2* cur_l = d_cur + nc;
        double2* jj = d_jj;
        double2* d_u = d_jj + NL * m * ns;
        double2* d_v = d_u + 2 * NL * R * ns;
        if (m) {
            TAGS_CUDA_OK(cudaMemcpyAsync(d_cur, il + s0 * R * m, sizeof(double2) * nc, cudaMemcpyHostToDevice, st));
            const int tb = 256, tg = (int)std::min<size_t>((nc + tb - 1) / tb, 152 * 16);
            k_cur_transpose<<<tg, tb, 0, st>>>(d_cur, cur_l, (int)ns, (int)R, (int)m);
            tags_note_launch();
            TAGS_CUDA_OK(cudaGetLastError());
            std::vector<SampleCoef> coef(ns);
            for (size_t k = 0; k < ns; ++k) {
                coef[k] = SampleCoef{};
                coef[k].gamma = D2(gamma[s0 + k]);
            }
            TAGS_CUDA_OK(cudaMemcpyAsync(d_coef, coef.data(), sizeof(SampleCoef) * ns, cudaMemcpyHostToDevice, st));
            if (int e = tags_launch_path_pairs((const double*)d_el, (int)m, (const double*)(d_el + m), (int)NL, d_coef,
                                               (int)ns, jj, c->status, st))
                return e;
        }
        TAGS_CUDA_OK(cudaMemcpyAsync(d_u, upts.data() + s0 * 2 * NL * R, sizeof(double2) * 2 * NL * R * ns,
                                     cudaMemcpyHostToDevice, st));
        TAGS_CUDA_OK(cudaMemcpyAsync(d_gk, s + s0, sizeof(double2) * ns, cudaMemcpyHostToDevice, st));
        const long long n = (long long)ns * NL * R;
        k_voltage<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(d_paths, (int)NL, d_el, (int)m, cur_l, d_u, jj, d_gk, mur,
                                                               (int)R, (int)ns, d_v);
        tags_note_launch();
        TAGS_CUDA_OK(cudaGetLastError());
        TAGS_CUDA_OK(cudaMemcpyAsync(v + s0 * NL * R, d_v, sizeof(double2) * n, cudaMemcpyDeviceToHost, st));
        TAGS_CUDA_OK(cudaStreamSynchronize(st));
    }
    return 0;
}

extern "C" int tags_fields_evaluations(unsigned long long* count, int reset) {
    if (!count) return tags_fail(TAGS_E_ARG, "null pointer argument");
    std::lock_guard<std::mutex> lk(tags_dropin_mutex());
    DeviceCtx* c = tags_ctx();
    if (!c) return tags_fail(TAGS_E_CUDA, "no usable CUDA device");
    if (int e = fields_tables(c->device)) return e;
    TAGS_CUDA_OK(cudaMemcpyAsync(count, g_evals[c->device], sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                 c->stream));
    if (reset) TAGS_CUDA_OK(cudaMemsetAsync(g_evals[c->device], 0, sizeof(unsigned long long), c->stream));
    TAGS_CUDA_OK(cudaStreamSynchronize(c->stream));
    return 0;
}

// ---- drop-ins with the reference's signatures -----------------------------------
// The reference's tolerance arguments (max_eval, req_abs_error, req_rel_error)
// are accepted and unused: the GPU rules are fixed at ~1e-12 relative.

extern "C" tags_cdouble electric_potential(const double* point, const Electrode* electrodes, size_t num_electrodes,
                                           const tags_cdouble* it, tags_cdouble gamma, tags_cdouble kappa,
                                           size_t max_eval, double req_abs_error, double req_rel_error) {
    (void)max_eval, (void)req_abs_error, (void)req_rel_error;
    tags_cdouble out{0.0, 0.0};
    // a point on an electrode leaves NaN in out (TAGS_E_GEOMETRY)
    int e = tags_fields_batch(point, 1, electrodes, num_electrodes, nullptr, it, 1, 1, &gamma, &kappa, 1.0, &out,
                              nullptr, nullptr);
    if (e && e != TAGS_E_GEOMETRY) out.re = out.im = nan("");
    return out;
}

extern "C" int magnetic_potential(const double* point, const Electrode* electrodes, size_t num_electrodes,
                                  const tags_cdouble* il, tags_cdouble gamma, double mur, size_t max_eval,
                                  double req_abs_error, double req_rel_error, tags_cdouble* va) {
    (void)max_eval, (void)req_abs_error, (void)req_rel_error;
    if (!va) return tags_fail(TAGS_E_ARG, "null pointer argument");
    const tags_cdouble kappa{1.0, 0.0};
    return tags_fields_batch(point, 1, electrodes, num_electrodes, il, nullptr, 1, 1, &gamma, &kappa, mur, nullptr,
                             va, nullptr);
}

extern "C" int electric_field(const double* point, const Electrode* electrodes, size_t num_electrodes,
                              const tags_cdouble* il, const tags_cdouble* it, tags_cdouble gamma, tags_cdouble s,
                              double mur, tags_cdouble kappa, size_t max_eval, double req_abs_error,
                              double req_rel_error, tags_cdouble* ve) {
    (void)max_eval, (void)req_abs_error, (void)req_rel_error;
    if (!ve) return tags_fail(TAGS_E_ARG, "null pointer argument");
    tags_cdouble va[3] = {}, ec[3] = {};
    const bool mag = std::abs(zd(s.re, s.im)) > TAGS_DBL_EPSILON;
    int e = tags_fields_batch(point, 1, electrodes, num_electrodes, il, it, 1, 1, &gamma, &kappa, mur, nullptr,
                              mag ? va : nullptr, ec);
    if (e && e != TAGS_E_GEOMETRY) return e;
    // src/electrode.c:530-535: with |s| > DBL_EPSILON ve is overwritten by
    // -s A, otherwise the conservative part is added to what ve holds
    for (int k = 0; k < 3; ++k) {
        zd base = mag ? -zd(s.re, s.im) * zd(va[k].re, va[k].im) : zd(ve[k].re, ve[k].im);
        zd r = base + zd(ec[k].re, ec[k].im);
        ve[k] = {r.real(), r.imag()};
    }
    return e;
}

extern "C" tags_cdouble voltage(const double* point1, const double* point2, const Electrode* electrodes,
                                size_t num_electrodes, const tags_cdouble* il, const tags_cdouble* it,
                                tags_cdouble gamma, tags_cdouble s, double mur, tags_cdouble kappa, size_t max_eval,
                                double req_abs_error, double req_rel_error) {
    (void)max_eval, (void)req_abs_error, (void)req_rel_error;
    double path[6];
    tags_cdouble out{nan(""), nan("")};
    if (!point1 || !point2) return out;
    memcpy(path, point1, sizeof(double) * 3);
    memcpy(path + 3, point2, sizeof(double) * 3);
    if (tags_voltage_batch(path, 1, electrodes, num_electrodes, il, it, 1, 1, &gamma, &s, &kappa, mur, &out))
        out.re = out.im = nan("");
    return out;
}
