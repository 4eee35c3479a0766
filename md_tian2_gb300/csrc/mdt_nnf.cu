// mdt_nnf.cu -- FP32 fast path of the HDNNP / EMT-surrogate force evaluation and MD step.
//
// Same results as the generic kernels of mdt_nn.cu (RuNNer's short-range prediction,
// src/pes_nene_mod.f90:7145-7368, with the symmetry functions of
// RuNNer_src/atomsymfunction2.f90 and atomsymfunction3Andi.f90) for the models that
// FastNN::ok admits, organised for throughput:
//
//  * CTA = 8 warps on one bead; warps take central atoms from a shared counter.
//  * Neighbour list of atom i, built by its warp: lane L takes atoms j = j0 + L and
//    visits only the image shifts whose fractional offset can lie inside the cutoff
//    (|f_d + n_d| <= rc |b_d|, b_d the reciprocal vectors), n1 -> n2 -> n3 ascending, so
//    a warp prefix sum over lanes yields RuNNer's order (neighbor_para_short.f90:117-163).
//    Distances are screened in FP32 from a hi/lo split of the wrapped positions; within
//    1e-4 (relative) of the cutoff the exact FP64 test of mdt_acsf.cuh decides.
//  * Neighbour rows (d, 1/r, fc, (dfc/dr)/r, exp(-eta_m r^2)) are computed once per pair.
//  * Triplets (q3 < q4) with r_jk <= rc and the G3 element pair are compacted per row
//    pair (rows p and n-2-p hold n candidates together, one lane per row pair) into
//    byte lists; the forward and the force walk then give every lane an equal share
//    of the compacted list, so no lane idles on a rejected triplet.
//  * fc(r_jk) and its derivative come from the Taylor series of cos(pi sqrt(s)/2) in
//    s = r_jk^2 / rc^2 (no square root, sine or cosine per triplet); with
//    h = (1 + lambda cos)/2, 2^(1-zeta) (1 + lambda cos)^zeta = 2 h^zeta, and every
//    h^zeta, h^(zeta-1) for zeta = 2^b comes from one squaring ladder.
//  * Forces: reverse mode as in mdt_acsf.cuh (dE/dG from the network, then
//    dE/dG . dG/dx per triplet in factored form), slot forces of the current row in
//    registers, of the second neighbour by shared-memory atomics; the central atom's
//    force is minus the sum of its slot forces (translation invariance of E_i).
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"
#include "mdt_acsf.cuh"
#include "mdt_prop.cuh"

namespace mdt {

namespace {

constexpr int kFW = 8;
constexpr int kFBlock = 32 * kFW;
constexpr double kHa2eVF = 27.21138602;

// Cosine cutoff fc = (cos(pi r/rc) + 1)/2 = c^2 with c = cos(pi sqrt(s)/2), s = r^2/rc^2.
// c is the Taylor series sum_n (-pi^2 s/4)^n / (2n)! truncated after n = 7 (remainder
// below 1e-10 on [0, 1], alternating terms no larger than 1.24, so FP32 Horner loses
// little), and fc = c^2 keeps the absolute error vanishing at the cutoff.
constexpr double half_cos_sqrt_coef(int n) {
    double c = 1.0;
    for (int k = 1; k <= n; ++k) c *= -(kPi * kPi / 4.0) / ((2.0 * k - 1.0) * (2.0 * k));
    return c;
}
constexpr float kCs0 = (float)half_cos_sqrt_coef(0), kCs1 = (float)half_cos_sqrt_coef(1),
                kCs2 = (float)half_cos_sqrt_coef(2), kCs3 = (float)half_cos_sqrt_coef(3),
                kCs4 = (float)half_cos_sqrt_coef(4), kCs5 = (float)half_cos_sqrt_coef(5),
                kCs6 = (float)half_cos_sqrt_coef(6), kCs7 = (float)half_cos_sqrt_coef(7);

// fc(s)
__device__ __forceinline__ float fc_of_s(float s) {
    float c = kCs7;
    c = fmaf(c, s, kCs6);
    c = fmaf(c, s, kCs5);
    c = fmaf(c, s, kCs4);
    c = fmaf(c, s, kCs3);
    c = fmaf(c, s, kCs2);
    c = fmaf(c, s, kCs1);
    c = fmaf(c, s, kCs0);
    return c * c;
}

// fc(s) and dfc/ds = 2 c c'(s) (Horner with derivative)
__device__ __forceinline__ void fc_of_s_d(float s, float &fc, float &dfds) {
    float c = kCs7, d = 0.f;
#define MDT_STEP(k)        \
    d = fmaf(d, s, c);     \
    c = fmaf(c, s, k);
    MDT_STEP(kCs6) MDT_STEP(kCs5) MDT_STEP(kCs4) MDT_STEP(kCs3) MDT_STEP(kCs2) MDT_STEP(kCs1) MDT_STEP(kCs0)
#undef MDT_STEP
    fc = c * c;
    dfds = 2.f * c * d;
}

// Activations in FP32.  Softplus in the form that cannot overflow (identical to
// log(exp(x) + 1) and (exp(v) - 1)/exp(v) of calconenn.f90 / getdnodes_values.f90 to
// FP32 rounding where those are finite).
__device__ __forceinline__ float act_f(uint8_t a, float x) {
    if (a == 'p') return x > 15.f ? x + __expf(-x) : log1pf(__expf(x));
    return act_fn<float>(a, x);
}
__device__ __forceinline__ float act_df(uint8_t a, float sum, float val) {
    if (a == 'p') return -expm1f(-val);
    return act_dfn<float>(a, sum, val);
}

constexpr int popc5(int m) { return (m & 1) + ((m >> 1) & 1) + ((m >> 2) & 1) + ((m >> 3) & 1) + ((m >> 4) & 1); }
constexpr int topbit5(int m) { return (m & 16) ? 4 : (m & 8) ? 3 : (m & 4) ? 2 : (m & 2) ? 1 : 0; }

// P[k] = h^zeta_k and (if Q) Q[k] = h^(zeta_k - 1) for the k-th zeta = 2^b of ZM:
// P_0 = h, Q_0 = 1, P_{b+1} = P_b^2, Q_{b+1} = P_b Q_b.
template <int ZM, bool WITHQ>
__device__ __forceinline__ void zeta_powers(float h, float *P, float *Q) {
    float p = h, q = 1.f;
    int k = 0;
#pragma unroll
    for (int b = 0; b < 5; ++b) {
        if (ZM & (1 << b)) {
            P[k] = p;
            if (WITHQ) Q[k] = q;
            ++k;
        }
        if (b < topbit5(ZM)) {
            if (WITHQ) q *= p;
            p *= p;
        }
    }
}

struct FLaunch {
    int max_atoms, maxnb, npmax, hsize;  // hsize: floats per warp for the network sums/values
    int surrogate;
};

// Shared memory of one CTA.  The per-warp area is also where the EMT fallback of a
// flagged bead carves its arrays (the network part of that bead is finished by then).
struct SmemF {
    double *px, *py, *pz;                // wrapped positions (bohr)
    float *xh, *yh, *zh, *xl, *yl, *zl;  // their FP32 hi/lo split
    int8_t *elem;
    float *fx, *fy, *fz;                 // bead force accumulators (Ha/bohr)
    double *lat;                         // 9 lattice rows + 9 inverse (bohr)
    float *latf, *ginv, *wk;             // FP32 lattice rows, inverse rows, image half-widths
    double *red;                         // block reductions
    double *cjk;                         // ring-polymer transform of the trajectory
    int *misc;                           // [0] range flag, [1] atom counter
    unsigned char *warp_base;            // per-warp areas
    size_t warp_bytes;
};

struct WarpF {
    float4 *ra, *rb, *rc;  // [q]: (dx, dy, dz, 1/r), (fc, E0, E1, E2), ((dfc/dr)/r, r, j | elem << 16, E3)
    uint8_t *code;         // [q]: bit 0 elem == pair_a, bit 1 elem == pair_b
    int *word;             // [q]: packed (j, image)
    float *sfx, *sfy, *sfz;
    uint8_t *tq4;          // [row pair][maxnb] second neighbours of the valid triplets
    int16_t *tcnt, *tsplit;
    int *tpre;
    float *G, *dG, *hs, *hv;
};

__host__ __device__ inline size_t r16f(size_t b) { return (b + 15) & ~size_t(15); }

__host__ __device__ inline size_t warp_bytes_f(int maxnb, int npmax, int hsize) {
    return 3 * r16f(16 * (size_t)maxnb) + r16f(maxnb) + r16f(4 * (size_t)maxnb) + 3 * r16f(4 * (size_t)maxnb) +
           r16f((size_t)npmax * maxnb) + 2 * r16f(2 * (size_t)npmax) + r16f(4 * ((size_t)npmax + 1)) +
           2 * r16f(4 * kMaxSF) + 2 * r16f(4 * (size_t)hsize);
}

__host__ __device__ inline size_t shared_bytes_f(int max_atoms, int max_beads) {
    return 3 * r16f(8 * (size_t)max_atoms) + 6 * r16f(4 * (size_t)max_atoms) + r16f(max_atoms) +
           3 * r16f(4 * (size_t)max_atoms) + r16f(8 * 18) + 3 * r16f(4 * 9) + r16f(8 * 64) +
           r16f(8 * (size_t)max_beads * max_beads) + 16;
}

size_t nnf_smem_bytes(int max_atoms, int max_beads, int maxnb, int npmax, int hsize) {
    const size_t wb = kFW * warp_bytes_f(maxnb, npmax, hsize);
    const size_t emt = smem_bytes(max_atoms, max_beads, 8);
    return shared_bytes_f(max_atoms, max_beads) + (wb > emt ? wb : emt);
}

__device__ SmemF carve_f(unsigned char *base, const FLaunch &L, int max_beads) {
    SmemF s;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += r16f(bytes);
        return p;
    };
    const int na = L.max_atoms;
    s.px = (double *)take(8 * na);
    s.py = (double *)take(8 * na);
    s.pz = (double *)take(8 * na);
    s.xh = (float *)take(4 * na);
    s.yh = (float *)take(4 * na);
    s.zh = (float *)take(4 * na);
    s.xl = (float *)take(4 * na);
    s.yl = (float *)take(4 * na);
    s.zl = (float *)take(4 * na);
    s.elem = (int8_t *)take(na);
    s.fx = (float *)take(4 * na);
    s.fy = (float *)take(4 * na);
    s.fz = (float *)take(4 * na);
    s.lat = (double *)take(8 * 18);
    s.latf = (float *)take(4 * 9);
    s.ginv = (float *)take(4 * 9);
    s.wk = (float *)take(4 * 9);
    s.red = (double *)take(8 * 64);
    s.cjk = (double *)take(8 * (size_t)max_beads * max_beads);
    s.misc = (int *)take(16);
    s.warp_base = base + off;
    s.warp_bytes = warp_bytes_f(L.maxnb, L.npmax, L.hsize);
    return s;
}

__device__ WarpF carve_warp(const SmemF &S, const FLaunch &L, int warp) {
    WarpF w;
    unsigned char *base = S.warp_base + (size_t)warp * S.warp_bytes;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += r16f(bytes);
        return p;
    };
    const int nb = L.maxnb;
    w.ra = (float4 *)take(16 * (size_t)nb);
    w.rb = (float4 *)take(16 * (size_t)nb);
    w.rc = (float4 *)take(16 * (size_t)nb);
    w.code = (uint8_t *)take(nb);
    w.word = (int *)take(4 * (size_t)nb);
    w.sfx = (float *)take(4 * (size_t)nb);
    w.sfy = (float *)take(4 * (size_t)nb);
    w.sfz = (float *)take(4 * (size_t)nb);
    w.tq4 = (uint8_t *)take((size_t)L.npmax * nb);
    w.tcnt = (int16_t *)take(2 * (size_t)L.npmax);
    w.tsplit = (int16_t *)take(2 * (size_t)L.npmax);
    w.tpre = (int *)take(4 * ((size_t)L.npmax + 1));
    w.G = (float *)take(4 * kMaxSF);
    w.dG = (float *)take(4 * kMaxSF);
    w.hs = (float *)take(4 * (size_t)L.hsize);
    w.hv = (float *)take(4 * (size_t)L.hsize);
    return w;
}

__device__ __forceinline__ int warp_excl_scan(int v, int &total) {
    const int lane = threadIdx.x & 31;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// exact FP64 cutoff test of one image (the oracle's operation order, no fused operations)
__device__ __forceinline__ bool exact_in_cutoff(const SmemF &S, int i, int j, int n1, int n2, int n3, double cut2) {
    const double *L = S.lat;
    const double d1n = n1, d2n = n2, d3n = n3;
    const double xt =
        __dadd_rn(__dadd_rn(__dadd_rn(S.px[j], __dmul_rn(d1n, L[0])), __dmul_rn(d2n, L[3])), __dmul_rn(d3n, L[6]));
    const double yt =
        __dadd_rn(__dadd_rn(__dadd_rn(S.py[j], __dmul_rn(d1n, L[1])), __dmul_rn(d2n, L[4])), __dmul_rn(d3n, L[7]));
    const double zt =
        __dadd_rn(__dadd_rn(__dadd_rn(S.pz[j], __dmul_rn(d1n, L[2])), __dmul_rn(d2n, L[5])), __dmul_rn(d3n, L[8]));
    const double e1 = __dsub_rn(xt, S.px[i]), e2 = __dsub_rn(yt, S.py[i]), e3 = __dsub_rn(zt, S.pz[i]);
    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(e1, e1), __dmul_rn(e2, e2)), __dmul_rn(e3, e3));
    return rr <= cut2;
}

// Image box of pair (i, j) and the per-image test.  Visits images in RuNNer's order.
template <bool WRITE>
__device__ __forceinline__ int visit_images(const SmemF &S, const FastNN &F, double cut2, int i, int j, float dx,
                                            float dy, float dz, const int *na, int *out, int pos, int cap) {
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float f = S.ginv[3 * d] * dx + S.ginv[3 * d + 1] * dy + S.ginv[3 * d + 2] * dz;
        lo[d] = max(-na[d], (int)ceilf(-f - S.wk[d]));
        hi[d] = min(na[d], (int)floorf(-f + S.wk[d]));
    }
    const float *Lf = S.latf;
    int c = 0;
    for (int n1 = lo[0]; n1 <= hi[0]; ++n1)
        for (int n2 = lo[1]; n2 <= hi[1]; ++n2)
            for (int n3 = lo[2]; n3 <= hi[2]; ++n3) {
                if (i == j && n1 == 0 && n2 == 0 && n3 == 0) continue;
                const float ex = dx + (float)n1 * Lf[0] + (float)n2 * Lf[3] + (float)n3 * Lf[6];
                const float ey = dy + (float)n1 * Lf[1] + (float)n2 * Lf[4] + (float)n3 * Lf[7];
                const float ez = dz + (float)n1 * Lf[2] + (float)n2 * Lf[5] + (float)n3 * Lf[8];
                const float rf = ex * ex + ey * ey + ez * ez;
                if (rf > F.cut2_hi) continue;
                if (!(rf < F.cut2_lo) && !exact_in_cutoff(S, i, j, n1, n2, n3, cut2)) continue;
                if (WRITE && pos + c < cap) out[pos + c] = pack_nb(j, n1, n2, n3);
                ++c;
            }
    return c;
}

// ---- one central atom: neighbour list, rows, descriptors, network, forces ----------
template <int NG, int ZM>
__device__ void nnf_atom(const NNDev &M, const FastNN &F, const NNScratch &X, const SmemF &S, const WarpF &W,
                         const FLaunch &L, int t, int i, int N, const int *na, bool do_forces, double &e_acc) {
    constexpr int NZ = popc5(ZM), NQ = 2 * NZ;
    static_assert(NQ <= kFNQ, "too many (lambda, zeta) cells");
    const int lane = threadIdx.x & 31;
    const int ei = S.elem[i];
    const double cut2 = __dmul_rn(M.maxcut, M.maxcut);

    // ---- neighbour list (RuNNer order) ---------------------------------------------------
    const float xhi = S.xh[i], yhi = S.yh[i], zhi = S.zh[i], xli = S.xl[i], yli = S.yl[i], zli = S.zl[i];
    int cnt = 0;
    for (int j0 = 0; j0 < N; j0 += 32) {
        const int j = j0 + lane;
        float dx = 0.f, dy = 0.f, dz = 0.f;
        int c = 0;
        if (j < N) {
            dx = (S.xh[j] - xhi) + (S.xl[j] - xli);
            dy = (S.yh[j] - yhi) + (S.yl[j] - yli);
            dz = (S.zh[j] - zhi) + (S.zl[j] - zli);
            c = visit_images<false>(S, F, cut2, i, j, dx, dy, dz, na, nullptr, 0, 0);
        }
        int tot;
        const int ex = warp_excl_scan(c, tot);
        if (c > 0) visit_images<true>(S, F, cut2, i, j, dx, dy, dz, na, W.word, cnt + ex, L.maxnb);
        cnt += tot;
    }
    if (cnt > L.maxnb) {
        if (lane == 0) X.nnstatus[t] = 1;
        cnt = L.maxnb;
    }
    __syncwarp();

    // ---- neighbour rows ------------------------------------------------------------------
    const int pa = F.pair_a[ei], pb = F.pair_b[ei];
    float g3l2[NG];
#pragma unroll
    for (int m = 0; m < NG; ++m) g3l2[m] = F.g3l2[ei][m];
    for (int q = lane; q < cnt; q += 32) {
        const int w = W.word[q];
        const int j = w & 0xFFFF;
        const float n1 = (float)(((w >> 16) & 15) - 8), n2 = (float)(((w >> 20) & 15) - 8),
                    n3 = (float)(((w >> 24) & 15) - 8);
        const float *Lf = S.latf;
        const float dx = ((S.xh[j] - xhi) + (S.xl[j] - xli)) + (n1 * Lf[0] + n2 * Lf[3] + n3 * Lf[6]);
        const float dy = ((S.yh[j] - yhi) + (S.yl[j] - yli)) + (n1 * Lf[1] + n2 * Lf[4] + n3 * Lf[7]);
        const float dz = ((S.zh[j] - zhi) + (S.zl[j] - zli)) + (n1 * Lf[2] + n2 * Lf[5] + n3 * Lf[8]);
        const float r2 = dx * dx + dy * dy + dz * dz;
        const float r = sqrtf(r2);
        const float rinv = 1.f / r;
        float fc, dfds;
        fc_of_s_d(fminf(r2 * F.inv_rc2, 1.f), fc, dfds);
        float E[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int m = 0; m < NG; ++m) E[m] = exp2f(g3l2[m] * r2);
        const int el = S.elem[j];
        W.ra[q] = make_float4(dx, dy, dz, rinv);
        W.rb[q] = make_float4(fc, E[0], E[1], E[2]);
        W.rc[q] = make_float4(2.f * dfds * F.inv_rc2, r, __int_as_float(j | (el << 16)), E[3]);
        W.code[q] = (uint8_t)((el == pa ? 1 : 0) | (el == pb ? 2 : 0));
    }
    __syncwarp();

    // ---- radial functions ----------------------------------------------------------------
    const int ng2 = F.ng2[ei];
    {
        float acc[kFMaxG2];
#pragma unroll
        for (int s = 0; s < kFMaxG2; ++s) acc[s] = 0.f;
        for (int q = lane; q < cnt; q += 32) {
            const float4 b = W.rb[q], c = W.rc[q];
            const int el = __float_as_int(c.z) >> 16;
#pragma unroll
            for (int s = 0; s < kFMaxG2; ++s) {
                if (s >= ng2) break;
                if (F.g2e[ei][s] != el) continue;
                const float u = c.y - F.g2rs[ei][s];
                acc[s] += exp2f(F.g2l2[ei][s] * u * u) * b.x;
            }
        }
#pragma unroll
        for (int s = 0; s < kFMaxG2; ++s) {
            if (s >= ng2) break;
            const float v = warp_sum(acc[s]);
            if (lane == 0) W.G[F.g2sf[ei][s]] = v;
        }
    }

    // ---- triplet lists -------------------------------------------------------------------
    const bool g3 = F.hasg3[ei] != 0;
    const int nrows = cnt - 1, npairs = (g3 && nrows > 0) ? (nrows + 1) / 2 : 0;
    int T = 0;
    if (npairs > 0) {
        const bool same = pa == pb;
        for (int p = lane; p < npairs; p += 32) {
            const int r0 = p, r1 = nrows - 1 - p, len0 = cnt - 1 - r0;
            const int tot = (r1 == r0) ? len0 : cnt;
            const float4 a0 = W.ra[r0], a1 = W.ra[r1];
            const int c0 = W.code[r0], c1 = W.code[r1];
            uint8_t *dst = W.tq4 + (size_t)p * L.maxnb;
            int n = 0, sp = 0;
            for (int c = 0; c < tot; ++c) {
                const bool first = c < len0;
                if (c == len0) sp = n;
                const int q4 = first ? r0 + 1 + c : c;
                const float4 k = W.ra[q4];
                const int ck = W.code[q4], cj = first ? c0 : c1;
                const float jx = (first ? a0.x : a1.x) - k.x, jy = (first ? a0.y : a1.y) - k.y,
                            jz = (first ? a0.z : a1.z) - k.z;
                const float r2 = jx * jx + jy * jy + jz * jz;
                const bool ok = r2 <= F.rc2 && (cj | ck) == 3 && (!same || (cj & ck) == 3);
                if (ok) dst[n++] = (uint8_t)q4;
            }
            if (tot == len0) sp = n;
            W.tcnt[p] = (int16_t)n;
            W.tsplit[p] = (int16_t)sp;
        }
        __syncwarp();
        int run = 0;
        for (int p0 = 0; p0 < npairs; p0 += 32) {
            const int p = p0 + lane;
            const int v = p < npairs ? W.tcnt[p] : 0;
            int tot;
            const int ex = warp_excl_scan(v, tot);
            if (p < npairs) W.tpre[p] = run + ex;
            run += tot;
        }
        if (lane == 0) W.tpre[npairs] = run;
        T = run;
        __syncwarp();
    }

    // equal share of the compacted list: [e0, e1), starting in row pair p at position pos
    auto share = [&](int &e0, int &e1, int &p, int &pos) {
        const int K = (T + 31) >> 5;
        e0 = min(T, lane * K);
        e1 = min(T, e0 + K);
        int lo = 0, hi = npairs - 1;  // last p with tpre[p] <= e0
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (W.tpre[mid] <= e0) lo = mid;
            else hi = mid - 1;
        }
        p = lo;
        pos = e0 - W.tpre[p];
    };

    // ---- G3 forward ----------------------------------------------------------------------
    if (T > 0) {
        float acc[NG][NQ];
#pragma unroll
        for (int m = 0; m < NG; ++m)
#pragma unroll
            for (int q = 0; q < NQ; ++q) acc[m][q] = 0.f;
        int e0, e1, p, pos;
        share(e0, e1, p, pos);
        int pc = W.tcnt[p], psp = W.tsplit[p], cq3 = -1;
        float4 JA = make_float4(0.f, 0.f, 0.f, 0.f), JB = JA, JC = JA;
        for (int e = e0; e < e1; ++e) {
            while (pos >= pc) {
                ++p;
                pos = 0;
                pc = W.tcnt[p];
                psp = W.tsplit[p];
            }
            const int q3 = pos < psp ? p : nrows - 1 - p;
            const int q4 = W.tq4[(size_t)p * L.maxnb + pos];
            ++pos;
            if (q3 != cq3) {
                cq3 = q3;
                JA = W.ra[q3];
                JB = W.rb[q3];
                if (NG == 4) JC = W.rc[q3];
            }
            const float4 KA = W.ra[q4], KB = W.rb[q4];
            const float jx = JA.x - KA.x, jy = JA.y - KA.y, jz = JA.z - KA.z;
            const float rjk2 = jx * jx + jy * jy + jz * jz;
            const float fcjk = fc_of_s(fminf(rjk2 * F.inv_rc2, 1.f));
            const float u = (JA.x * KA.x + JA.y * KA.y + JA.z * KA.z) * (JA.w * KA.w);
            const float pf = JB.x * KB.x * fcjk;
            float Xm[NG];
            const float Ej[4] = {JB.y, JB.z, JB.w, JC.w};
            float Ek[4] = {KB.y, KB.z, KB.w, 0.f};
            if (NG == 4) Ek[3] = W.rc[q4].w;
#pragma unroll
            for (int m = 0; m < NG; ++m) Xm[m] = Ej[m] * Ek[m] * exp2f(g3l2[m] * rjk2) * pf;
            float Pp[NZ], Pm[NZ];
            zeta_powers<ZM, false>(fmaf(0.5f, u, 0.5f), Pp, nullptr);
            zeta_powers<ZM, false>(fmaf(-0.5f, u, 0.5f), Pm, nullptr);
#pragma unroll
            for (int m = 0; m < NG; ++m)
#pragma unroll
                for (int k = 0; k < NZ; ++k) {
                    acc[m][2 * k] = fmaf(Xm[m], Pp[k], acc[m][2 * k]);
                    acc[m][2 * k + 1] = fmaf(Xm[m], Pm[k], acc[m][2 * k + 1]);
                }
        }
#pragma unroll
        for (int m = 0; m < NG; ++m)
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const float v = warp_sum(acc[m][q]);
                const int s = F.cell_sf[ei][m][q];
                if (lane == 0 && s >= 0) W.G[s] = 2.f * v;
            }
    } else if (g3) {
        for (int q = lane; q < NG * NQ; q += 32) {
            const int s = F.cell_sf[ei][q / NQ][q % NQ];
            if (s >= 0) W.G[s] = 0.f;
        }
    }
    __syncwarp();

    // ---- scaling, range check (getshortatomic.f90:174-236) and network ------------------
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    for (int s = lane; s < nsf; s += 32) {
        const float g = W.G[s];
        const float4 sc = F.scal[sfb + s];
        if (g < sc.z || g > sc.w) S.misc[0] = 1;
        W.hv[s] = fmaf(sc.x, g, sc.y);
    }
    __syncwarp();
    const float *we = M.wf + (size_t)ei * M.maxweights;
    const int hs0 = kMaxNodes;  // stride of a layer in hs/hv is M.maxnodes' bound below
    const int ls = L.hsize / (M.nlayers + 1);
    (void)hs0;
    for (int l = 1; l <= M.nlayers; ++l) {
        const int nprev = M.nodes[ei][l - 1], ncur = M.nodes[ei][l];
        const float *wl = we + M.woff[ei][l];
        for (int n = lane; n < ncur; n += 32) {
            float z = 0.f;
            for (int p = 0; p < nprev; ++p) z = fmaf(__ldg(wl + p * ncur + n), W.hv[(l - 1) * ls + p], z);
            z += __ldg(wl + nprev * ncur + n);
            if (M.normnodes) z /= (float)nprev;
            W.hs[l * ls + n] = z;
            W.hv[l * ls + n] = act_f(M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n], z);
        }
        __syncwarp();
    }
    if (lane == 0) e_acc += (double)W.hv[M.nlayers * ls] + (M.remove_atom_energies ? M.atom_energy[ei] : 0.0);
    if (!do_forces) {
        __syncwarp();
        return;
    }
    float *delta = W.hs;
    for (int l = M.nlayers; l >= 1; --l) {
        const int ncur = M.nodes[ei][l];
        const float norm = M.normnodes ? 1.f / (float)M.nodes[ei][l - 1] : 1.f;
        for (int n = lane; n < ncur; n += 32) {
            const uint8_t a = M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n];
            const float dn = norm * act_df(a, W.hs[l * ls + n], W.hv[l * ls + n]);
            float up = 1.f;
            if (l < M.nlayers) {
                const int nn = M.nodes[ei][l + 1];
                const float *wl = we + M.woff[ei][l + 1];
                up = 0.f;
                for (int m = 0; m < nn; ++m) up = fmaf(__ldg(wl + n * nn + m), delta[(l + 1) * ls + m], up);
            }
            delta[l * ls + n] = dn * up;
        }
        __syncwarp();
    }
    {
        const int n1 = M.nodes[ei][1];
        const float *wl = we + M.woff[ei][1];
        for (int s = lane; s < nsf; s += 32) {
            float v = 0.f;
            for (int n = 0; n < n1; ++n) v = fmaf(__ldg(wl + s * n1 + n), delta[ls + n], v);
            W.dG[s] = v * F.dscal[sfb + s];
        }
    }
    __syncwarp();

    // ---- forces: radial part ---------------------------------------------------------------
    for (int q = lane; q < cnt; q += 32) {
        const float4 a = W.ra[q], b = W.rb[q], c = W.rc[q];
        const int el = __float_as_int(c.z) >> 16;
        const float dfc = c.x * c.y;
        float dsum = 0.f;
#pragma unroll
        for (int s = 0; s < kFMaxG2; ++s) {
            if (s >= ng2) break;
            if (F.g2e[ei][s] != el) continue;
            const float u = c.y - F.g2rs[ei][s];
            const float ex = exp2f(F.g2l2[ei][s] * u * u);
            dsum = fmaf(W.dG[F.g2sf[ei][s]], ex * fmaf(-2.f * F.g2eta[ei][s] * u, b.x, dfc), dsum);
        }
        const float fr = dsum * a.w;
        W.sfx[q] = -fr * a.x;
        W.sfy[q] = -fr * a.y;
        W.sfz[q] = -fr * a.z;
    }
    __syncwarp();

    // ---- forces: angular part ----------------------------------------------------------------
    if (T > 0) {
        float Wy[NG][NQ], Wz[NG][NQ], eta[NG];
#pragma unroll
        for (int m = 0; m < NG; ++m) {
            eta[m] = F.g3eta[ei][m];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const int s = F.cell_sf[ei][m][q];
                const float c = s >= 0 ? W.dG[s] : 0.f;
                Wy[m][q] = 2.f * c;
                Wz[m][q] = F.cell_lz[q] * c;
            }
        }
        int e0, e1, p, pos;
        share(e0, e1, p, pos);
        int pc = W.tcnt[p], psp = W.tsplit[p], cq3 = -1;
        float4 JA = make_float4(0.f, 0.f, 0.f, 0.f), JB = JA, JC = JA;
        float fjx = 0.f, fjy = 0.f, fjz = 0.f;
        for (int e = e0; e < e1; ++e) {
            while (pos >= pc) {
                ++p;
                pos = 0;
                pc = W.tcnt[p];
                psp = W.tsplit[p];
            }
            const int q3 = pos < psp ? p : nrows - 1 - p;
            const int q4 = W.tq4[(size_t)p * L.maxnb + pos];
            ++pos;
            if (q3 != cq3) {
                if (cq3 >= 0) {
                    atomicAdd(&W.sfx[cq3], fjx);
                    atomicAdd(&W.sfy[cq3], fjy);
                    atomicAdd(&W.sfz[cq3], fjz);
                }
                fjx = fjy = fjz = 0.f;
                cq3 = q3;
                JA = W.ra[q3];
                JB = W.rb[q3];
                JC = W.rc[q3];
            }
            const float4 KA = W.ra[q4], KB = W.rb[q4], KC = W.rc[q4];
            const float jx = JA.x - KA.x, jy = JA.y - KA.y, jz = JA.z - KA.z;
            const float rjk2 = jx * jx + jy * jy + jz * jz;
            float fcjk, dfds;
            fc_of_s_d(fminf(rjk2 * F.inv_rc2, 1.f), fcjk, dfds);
            const float dfcrjk = 2.f * dfds * F.inv_rc2;
            const float rr = JA.w * KA.w;
            const float u = (JA.x * KA.x + JA.y * KA.y + JA.z * KA.z) * rr;
            const float Ej[4] = {JB.y, JB.z, JB.w, JC.w};
            const float Ek[4] = {KB.y, KB.z, KB.w, KC.w};
            float Xm[NG];
#pragma unroll
            for (int m = 0; m < NG; ++m) Xm[m] = Ej[m] * Ek[m] * exp2f(g3l2[m] * rjk2);
            float Pp[NZ], Pm[NZ], Qp[NZ], Qm[NZ];
            zeta_powers<ZM, true>(fmaf(0.5f, u, 0.5f), Pp, Qp);
            zeta_powers<ZM, true>(fmaf(-0.5f, u, 0.5f), Pm, Qm);
            float A1 = 0.f, A2 = 0.f, Bs = 0.f;
#pragma unroll
            for (int m = 0; m < NG; ++m) {
                float Y = 0.f, Z = 0.f;
#pragma unroll
                for (int k = 0; k < NZ; ++k) {
                    Y = fmaf(Wy[m][2 * k], Pp[k], Y);
                    Y = fmaf(Wy[m][2 * k + 1], Pm[k], Y);
                    Z = fmaf(Wz[m][2 * k], Qp[k], Z);
                    Z = fmaf(Wz[m][2 * k + 1], Qm[k], Z);
                }
                A1 = fmaf(Xm[m], Z, A1);
                const float xy = Xm[m] * Y;
                Bs += xy;
                A2 = fmaf(eta[m], xy, A2);
            }
            const float pfc = JB.x * KB.x * fcjk;
            const float t1 = pfc * A1, t2 = pfc * A2;
            const float gj = -t1 * u * JA.w * JA.w - 4.f * t2 + Bs * KB.x * fmaf(JC.x, fcjk, JB.x * dfcrjk);
            const float gk = -t1 * u * KA.w * KA.w - 4.f * t2 + Bs * JB.x * fmaf(KC.x, fcjk, KB.x * dfcrjk);
            const float gx = t1 * rr + 2.f * t2 - Bs * JB.x * KB.x * dfcrjk;
            fjx -= gj * JA.x + gx * KA.x;
            fjy -= gj * JA.y + gx * KA.y;
            fjz -= gj * JA.z + gx * KA.z;
            atomicAdd(&W.sfx[q4], -(gk * KA.x + gx * JA.x));
            atomicAdd(&W.sfy[q4], -(gk * KA.y + gx * JA.y));
            atomicAdd(&W.sfz[q4], -(gk * KA.z + gx * JA.z));
        }
        if (cq3 >= 0) {
            atomicAdd(&W.sfx[cq3], fjx);
            atomicAdd(&W.sfy[cq3], fjy);
            atomicAdd(&W.sfz[cq3], fjz);
        }
    }
    __syncwarp();

    // ---- scatter: neighbours get their slot forces, the centre minus their sum ----------
    float fix = 0.f, fiy = 0.f, fiz = 0.f;
    for (int q = lane; q < cnt; q += 32) {
        const int j = __float_as_int(W.rc[q].z) & 0xFFFF;
        const float sx = W.sfx[q], sy = W.sfy[q], sz = W.sfz[q];
        atomicAdd(&S.fx[j], sx);
        atomicAdd(&S.fy[j], sy);
        atomicAdd(&S.fz[j], sz);
        fix -= sx;
        fiy -= sy;
        fiz -= sz;
    }
    fix = warp_sum(fix);
    fiy = warp_sum(fiy);
    fiz = warp_sum(fiz);
    if (lane == 0) {
        atomicAdd(&S.fx[i], fix);
        atomicAdd(&S.fy[i], fiy);
        atomicAdd(&S.fz[i], fiz);
    }
    __syncwarp();
}

// ---- one bead ---------------------------------------------------------------------------
template <int NG, int ZM>
__device__ bool nnf_bead(const Batch &B, const NNDev &M, const FastNN &F, const NNScratch &X, const SmemF &S,
                         const FLaunch &L, int t, int b, bool do_forces, bool skip_if_flagged) {
    const int N = B.natoms[t];
    const int64_t base = B.ba_off[t] + (int64_t)b * N;
    const int aoff = B.atom_off[t];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        acsf_lattice(B.box + 9 * t, S.lat);
        S.misc[0] = 0;
        S.misc[1] = 0;
    }
    __syncthreads();
    if (tid < 9) {
        S.latf[tid] = (float)S.lat[tid];
        S.ginv[tid] = (float)S.lat[9 + tid];
    }
    if (tid < 3) {
        const double *I = S.lat + 9 + 3 * tid;
        const double bn = sqrt(I[0] * I[0] + I[1] * I[1] + I[2] * I[2]);
        S.wk[tid] = (float)(M.maxcut * bn * (1.0 + 1e-4) + 1e-4);
    }
    for (int i = tid; i < N; i += nt) {
        double x, y, z;
        acsf_wrap_one(B.rx[base + i], B.ry[base + i], B.rz[base + i], S.lat, x, y, z);
        S.px[i] = x;
        S.py[i] = y;
        S.pz[i] = z;
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        S.xh[i] = xh;
        S.yh[i] = yh;
        S.zh[i] = zh;
        S.xl[i] = (float)(x - (double)xh);
        S.yl[i] = (float)(y - (double)yh);
        S.zl[i] = (float)(z - (double)zh);
        S.elem[i] = (int8_t)M.elem_of_type[B.type[aoff + i]];
        S.fx[i] = 0.f;
        S.fy[i] = 0.f;
        S.fz[i] = 0.f;
    }
    __syncthreads();
    const int na[3] = {X.img[3 * t], X.img[3 * t + 1], X.img[3 * t + 2]};
    const WarpF W = carve_warp(S, L, warp);
    double e_warp = 0.0;
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(&S.misc[1], 1);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= N) break;
        if (S.elem[i] < 0) continue;
        nnf_atom<NG, ZM>(M, F, X, S, W, L, t, i, N, na, do_forces, e_warp);
    }
    const double etot = block_sum(e_warp, S.red);  // contains __syncthreads: flag visible
    const bool flagged = S.misc[0] != 0;
    if (skip_if_flagged && flagged) {
        __syncthreads();
        return true;
    }
    if (tid == 0) B.epot[B.bead_off[t] + b] += etot * kHa2eVF;
    if (do_forces) {
        const double c = kHa2eVF * kAng2BohrD;
        for (int i = tid; i < N; i += nt) {
            B.fx[base + i] += (double)S.fx[i] * c;
            B.fy[base + i] += (double)S.fy[i] * c;
            B.fz[base + i] += (double)S.fz[i] * c;
        }
    }
    __syncthreads();
    return flagged;
}

// calc_force (force.f90:40-86) with the network: zero, free ring-polymer step, per-bead
// prediction (EMT for a flagged bead of the surrogate), accelerations.
template <int NG, int ZM>
__device__ void nnf_calc_force(const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                               const NNScratch &X, const PropParams &P, const SmemF &S, const SmemEmt<double> &SE,
                               const FLaunch &L, const TrajView &T, bool do_forces) {
    const int tot = T.N * T.nb;
    for (int s = threadIdx.x; s < tot; s += blockDim.x) {
        const int64_t k = T.base + s;
        B.fx[k] = 0.0; B.fy[k] = 0.0; B.fz[k] = 0.0;
        B.ax[k] = 0.0; B.ay[k] = 0.0; B.az[k] = 0.0;
    }
    for (int b = threadIdx.x; b < T.nb; b += blockDim.x) B.epot[B.bead_off[T.t] + b] = 0.0;
    __syncthreads();
    if (T.nb > 1) ring_polymer_step(B, P, T, S.cjk);
    for (int b = 0; b < T.nb; ++b) {
        const bool flagged = nnf_bead<NG, ZM>(B, M, F, X, S, L, T.t, b, do_forces, L.surrogate != 0);
        if (L.surrogate && flagged) {
            emt_bead<double>(B, E, SE, T.t, b, do_forces);
            if (threadIdx.x == 0) X.fallback[T.t] += 1;
        }
    }
    if (do_forces) {
        for (int s = threadIdx.x; s < tot; s += blockDim.x) {
            const int64_t k = T.base + s;
            const int i = s % T.N;
            const double m = B.mass[T.aoff + i];
            const uint8_t fx = B.fixed[k];
            if (!(fx & 1)) B.ax[k] = B.fx[k] / m;
            if (!(fx & 2)) B.ay[k] = B.fy[k] / m;
            if (!(fx & 4)) B.az[k] = B.fz[k] / m;
        }
    }
    __syncthreads();
}

// mode 0: forces, 1: energies only, 2: nsteps fused MD steps (propagate_1, forces,
// propagate_2, exit test), as the generic network kernels.
template <int NG, int ZM>
__global__ void __launch_bounds__(kFBlock, 2)
    nnf_kernel(Batch B, NNDev M, FastNN F, EmtConst E, NNScratch X, PropParams P, FLaunch L, const int *order,
               int *counter, int nsteps, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    const SmemF S = carve_f(smem_raw, L, B.max_beads);
    SmemEmt<double> SE = carve_smem<double>(S.warp_base, B.max_atoms, B.max_beads);
    SE.red = S.red;
    SE.cjk = S.cjk;
    for (;;) {
        if (threadIdx.x == 0) work_slot = atomicAdd(counter, 1);
        __syncthreads();
        const int w = work_slot;
        __syncthreads();
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, S.cjk);
        if (mode != 2) {
            nnf_calc_force<NG, ZM>(B, M, F, E, X, P, S, SE, L, T, mode == 0);
            continue;
        }
        const int ty0 = B.type[T.aoff];
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, S.cjk, step, S.red);
            nnf_calc_force<NG, ZM>(B, M, F, E, X, P, S, SE, L, T, true);
            propagate_2(B, P, T, step);
            if (threadIdx.x == 0) {
                B.steps_done[t] = step;
                if (P.use_exit && B.is_proj[ty0] && B.status[t] == kStatusRunning) {
                    bool up = true, lo = true;
                    for (int b = 0; b < T.nb; ++b) {
                        const double z = B.rz[T.base + (int64_t)b * T.N];
                        up = up && (z > P.pul);
                        lo = lo && (z < P.pll);
                    }
                    if (up) B.status[t] = kStatusExitUpper;
                    else if (lo) B.status[t] = kStatusExitLower;
                }
            }
            __syncthreads();
        }
    }
}

template <int NG, int ZM>
cudaError_t nnf_launch_t(const LaunchCfg &c, const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                         const NNScratch &X, const PropParams &P, const FLaunch &L, size_t sm, int nsteps, int mode) {
    cudaError_t e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(nnf_kernel<NG, ZM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    nnf_kernel<NG, ZM><<<c.grid, kFBlock, sm, c.stream>>>(B, M, F, E, X, P, L, c.order, c.counter, nsteps, mode);
    return cudaGetLastError();
}

template <int NG, int ZM>
int nnf_occupancy_t(size_t sm) {
    int n = 0;
    cudaFuncSetAttribute(nnf_kernel<NG, ZM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nnf_kernel<NG, ZM>, kFBlock, sm);
    return n;
}

FLaunch flaunch(const Batch &B, const NNDev &M, int surrogate) {
    FLaunch L;
    L.max_atoms = B.max_atoms;
    L.maxnb = M.maxnb;
    L.npmax = (M.maxnb + 1) / 2;
    int mx = 1;
    for (int e = 0; e < M.nelem; ++e)
        for (int l = 0; l <= M.nlayers; ++l) mx = mx > M.nodes[e][l] ? mx : M.nodes[e][l];
    L.hsize = (M.nlayers + 1) * mx;
    L.surrogate = surrogate;
    return L;
}

}  // namespace

// Kernels exist for the zeta set {1, 4, 16} (a subset runs with zero-weight cells) and
// 1..4 eta slots.
int nnf_zm_supported(int zm) { return (zm & ~0x15) == 0 ? 0x15 : 0; }

#define MDT_NNF_DISPATCH(CALL)                                               \
    switch (F.ng) {                                                          \
        case 1: CALL(1, 0x15); case 2: CALL(2, 0x15); case 3: CALL(3, 0x15); \
        case 4: CALL(4, 0x15); default: break;                               \
    }

size_t nnf_total_smem(const Batch &B, const NNDev &M) {
    const FLaunch L = flaunch(B, M, 0);
    return nnf_smem_bytes(B.max_atoms, B.max_beads, L.maxnb, L.npmax, L.hsize);
}

int nnf_resident_ctas(const Batch &B, const NNDev &M, const FastNN &F) {
    const size_t sm = nnf_total_smem(B, M);
#define MDT_OCC(NG, ZM) return std::max(1, nnf_occupancy_t<NG, ZM>(sm));
    MDT_NNF_DISPATCH(MDT_OCC)
#undef MDT_OCC
    return 1;
}

cudaError_t launch_nnf(const LaunchCfg &c, const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                       const NNScratch &X, const PropParams &P, int nsteps, int mode, bool surrogate) {
    const FLaunch L = flaunch(B, M, surrogate ? 1 : 0);
    const size_t sm = nnf_smem_bytes(B.max_atoms, B.max_beads, L.maxnb, L.npmax, L.hsize);
#define MDT_LAUNCH(NG, ZM) return nnf_launch_t<NG, ZM>(c, B, M, F, E, X, P, L, sm, nsteps, mode);
    MDT_NNF_DISPATCH(MDT_LAUNCH)
#undef MDT_LAUNCH
    return cudaErrorInvalidValue;
}

}  // namespace mdt
