// mdt_nnf.cu -- FP32 fast path of the HDNNP / EMT-surrogate force evaluation and MD step.
//
// Same results as the generic kernels of mdt_nn.cu (RuNNer's short-range prediction,
// src/pes_nene_mod.f90:7145-7368, with the symmetry functions of
// RuNNer_src/atomsymfunction2.f90 and atomsymfunction3Andi.f90) for the models that
// FastNN::ok admits, organised for throughput:
//
//  * CTA = 8 warps on one bead, in three phases separated by CTA barriers:
//      descriptors  warp per central atom (atoms from a shared counter): neighbour
//                   list, neighbour rows, G2 and G3 into the bead's descriptor array;
//      network      warp per group of 4 atoms of one element (lanes = nodes, four
//                   independent dot products per lane), dE/dG over the descriptors;
//      forces       warp per central atom again (rows rebuilt from the neighbour words
//                   the first phase left in global scratch).
//  * Neighbour list of atom i, built by its warp: lane L takes atoms j = j0 + L and
//    visits only the image shifts whose fractional offset can lie inside the cutoff
//    (|f_d + n_d| <= rc |b_d|, b_d the reciprocal vectors), n1 -> n2 -> n3 ascending, so
//    a warp prefix sum over lanes yields RuNNer's order (neighbor_para_short.f90:117-163).
//    Distances are screened in FP32 from a hi/lo split of the wrapped positions; within
//    1e-4 (relative) of the cutoff the exact FP64 test of mdt_acsf.cuh decides.
//  * Neighbour rows (d, 1/r, fc, (dfc/dr)/r, exp(-eta_m r^2)) are computed once per pair.
//  * Radial functions in one pass over the neighbours (each function predicated on the
//    neighbour's element), per-lane partial sums combined by one reduce-scatter (31
//    shuffles for 32 values).
//  * Triplets (q3 < q4) with r_jk <= rc and the G3 element pair: lane p owns the row
//    pair (p, n-2-p) of the upper triangle (n candidates together) and marks the valid
//    second neighbours of both rows in bit masks.  The forward and the force walk visit
//    only set bits, in chunks: the lanes feed their rows' triplets into a warp buffer and
//    take equal contiguous blocks of it (valid triplets fall unevenly on the row pairs:
//    walked by their owners, half the lanes idled).
//  * fc(r_jk) and its derivative come from the Taylor series of cos(pi sqrt(s)/2) in
//    s = r_jk^2 / rc^2 (no square root, sine or cosine per triplet); with
//    h = (1 + lambda cos)/2, 2^(1-zeta) (1 + lambda cos)^zeta = 2 h^zeta, and every
//    h^zeta, h^(zeta-1) for zeta = 2^b comes from one squaring ladder.
//  * Network: weights of all elements in shared memory, rows padded to a stride of
//    4 (mod 8) floats so that lanes reading different rows hit different banks.
//  * Forces: reverse mode as in mdt_acsf.cuh (dE/dG from the network, then
//    dE/dG . dG/dx per triplet in factored form).  The first neighbour's force of a
//    triplet accumulates in the row owner's registers, the second neighbour's by a
//    shared-memory atomic; every warp adds its slot forces into its own copy of the
//    bead's force array (plain adds, atomics only for repeated images of one atom).
//    The central atom's force is minus the sum of its slot forces (translation
//    invariance of E_i).
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_fastmath.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"
#include "mdt_acsf.cuh"
#include "mdt_prop.cuh"

namespace mdt {

namespace {

constexpr int kFW = 8;
constexpr int kFBlock = 32 * kFW;
constexpr double kHa2eVF = 27.21138602;

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
    int max_atoms, maxnb, mw, ls, sgs;  // mw: mask words per row (0 without G3); ls: node stride; sgs: descriptor stride
    int surrogate, netshape;            // netshape: all layers fit the 4-atom network kernel
};

// Shared memory of one CTA.  The per-warp area also holds the network buffers of the
// network phase and the EMT fallback of a flagged bead.
struct SmemF {
    double *px, *py, *pz;                // wrapped positions (bohr)
    float *xh, *yh, *zh, *xl, *yl, *zl;  // their FP32 hi/lo split
    int8_t *elem;
    int *fold;                           // fold counts of the wrapping, 3 x 8 bits (+128)
    int *byel;                           // atoms ordered by element; [max_atoms + kMaxElem + 1] offsets after
    float *f3;                           // [3][max_atoms] bead force accumulators (Ha/bohr)
    double *lat;                         // 9 lattice rows + 9 inverse (bohr)
    float *latf, *ginv, *wk;             // FP32 lattice rows, inverse rows, image half-widths (cutoff, skin list)
    double *red;                         // block reductions
    double *cjk;                         // ring-polymer transform of the trajectory
    int *misc;                           // [0] range flag, [1] group counter, [2] rebuild skin lists, [3] max displacement
    float *w;                            // network weights (FastNN::wofs layout)
    float4 *g2;                          // radial-function table (FastNN::g2tab)
    unsigned char *warp_base;            // per-warp areas
    size_t warp_bytes;
};

struct WarpF {
    float4 *ra, *rb, *rc;  // [q]: (dx, dy, dz, 1/r), (fc, E0, E1, E2), ((dfc/dr)/r, r, j | elem << 16, E3)
    uint8_t *code;         // [q]: bit 0 elem == pair_a, bit 1 elem == pair_b
    unsigned *mask;        // [q][mw]: valid second neighbours q4 > q of row q
    int *rcnt;             // [q]: valid triplets of row q
    uint16_t *tbuf;        // [kTB]: a chunk of the warp's triplets, q3 | q4 << 8 (G3 models)
    float *sfx, *sfy, *sfz;
    float *gb;             // [kNAmax][sgs]: descriptors G, then dE/dG, of the atoms in flight
};

constexpr int kNAmax = 4;  // atoms per warp in the network phase
constexpr int kTB = 1024;  // triplets per chunk of the balanced triplet walk

__host__ __device__ inline size_t r16f(size_t b) { return (b + 15) & ~size_t(15); }

__host__ __device__ inline size_t warp_bytes_f(int maxnb, int mw, int nlayers, int ls, int sgs) {
    const size_t rows = 3 * r16f(16 * (size_t)maxnb) + r16f(maxnb) + r16f(4 * (size_t)maxnb * mw) +
                        r16f(4 * ((size_t)maxnb + 1)) + (mw > 0 ? r16f(2 * (size_t)kTB) : 0) +
                        3 * r16f(4 * (size_t)maxnb);
    const size_t net = 2 * r16f(4 * (size_t)kNAmax * (nlayers + 1) * ls);
    return (rows > net ? rows : net) + r16f(4 * (size_t)kNAmax * sgs);
}

__host__ __device__ inline size_t shared_bytes_f(int max_atoms, int max_beads, int wtotal, int nelem) {
    return 3 * r16f(8 * (size_t)max_atoms) + 6 * r16f(4 * (size_t)max_atoms) + r16f(max_atoms) +
           r16f(4 * (size_t)max_atoms) + r16f(4 * ((size_t)max_atoms + kMaxElem + 1)) +
           3 * r16f(4 * (size_t)max_atoms) + r16f(8 * 18) + 3 * r16f(4 * 9) + r16f(8 * 64) +
           r16f(8 * rp_cells(max_beads)) + 16 + r16f(4 * (size_t)wtotal) +
           r16f(16 * (size_t)nelem * kFMaxG2);
}

FLaunch flaunch(const Batch &B, const NNDev &M, int surrogate) {
    FLaunch L;
    L.max_atoms = B.max_atoms;
    L.maxnb = M.maxnb;
    L.mw = 0;
    for (int e = 0; e < M.nelem; ++e)
        if (M.g3fast[e]) L.mw = (M.maxnb + 31) / 32;
    int mx = 1;
    for (int e = 0; e < M.nelem; ++e)
        for (int l = 0; l <= M.nlayers; ++l) mx = mx > M.nodes[e][l] ? mx : M.nodes[e][l];
    L.ls = (mx + 3) & ~3;
    L.sgs = (M.maxsf + 3) & ~3;
    L.surrogate = surrogate;
    L.netshape = 1;
    for (int e = 0; e < M.nelem; ++e)
        for (int l = 1; l <= M.nlayers; ++l)
            if (M.nodes[e][l] > 32 || M.nodes[e][l - 1] > 32) L.netshape = 0;
    return L;
}

size_t nnf_smem_total(const Batch &B, const NNDev &M, const FastNN &F) {
    const FLaunch L = flaunch(B, M, 0);
    const size_t wb = kFW * warp_bytes_f(L.maxnb, L.mw, M.nlayers, L.ls, L.sgs);
    const size_t emt = smem_bytes(B.max_atoms, B.max_beads, 8);
    return shared_bytes_f(B.max_atoms, B.max_beads, F.wtotal, M.nelem) + (wb > emt ? wb : emt);
}

__device__ SmemF carve_f(unsigned char *base, const FLaunch &L, int max_beads, int wtotal, int nelem,
                         int nlayers) {
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
    s.fold = (int *)take(4 * (size_t)na);
    s.byel = (int *)take(4 * ((size_t)na + kMaxElem + 1));
    s.f3 = (float *)take(4 * 3 * (size_t)na);
    s.lat = (double *)take(8 * 18);
    s.latf = (float *)take(4 * 9);
    s.ginv = (float *)take(4 * 9);
    s.wk = (float *)take(4 * 9);
    s.red = (double *)take(8 * 64);
    s.cjk = (double *)take(8 * rp_cells(max_beads));
    s.misc = (int *)take(16);
    s.w = (float *)take(4 * (size_t)wtotal);
    s.g2 = (float4 *)take(16 * (size_t)nelem * kFMaxG2);
    s.warp_base = base + off;
    s.warp_bytes = warp_bytes_f(L.maxnb, L.mw, nlayers, L.ls, L.sgs);
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
    w.mask = (unsigned *)take(4 * (size_t)nb * L.mw);
    w.rcnt = (int *)take(4 * ((size_t)nb + 1));
    w.tbuf = (uint16_t *)take(L.mw > 0 ? 2 * (size_t)kTB : 0);
    w.sfx = (float *)take(4 * (size_t)nb);
    w.sfy = (float *)take(4 * (size_t)nb);
    w.sfz = (float *)take(4 * (size_t)nb);
    w.gb = (float *)(base + S.warp_bytes - r16f(4 * (size_t)kNAmax * L.sgs));
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

// Reduce-scatter of NV (power of two, <= 32) per-lane partial sums: afterwards v[0] of
// lane L holds the warp total of index L & (NV - 1).
template <int NV>
__device__ __forceinline__ void reduce_scatter(float (&v)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = 16; off >= NV; off >>= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], off);
#pragma unroll
    for (int w = NV / 2; w >= 1; w >>= 1) {
        const bool up = (lane & w) != 0;
#pragma unroll
        for (int k = 0; k < w; ++k) {
            const float keep = up ? v[k + w] : v[k], give = up ? v[k] : v[k + w];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, give, w);
        }
    }
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

// acsf_wrap_one (translate.f90) with the fold counts s_d = floor(f_d) it applied
__device__ __forceinline__ void wrap_fold(double xa, double ya, double za, const double *lat, double &x, double &y,
                                          double &z, int &fold) {
    x = __dmul_rn(xa, kAng2BohrD);
    y = __dmul_rn(ya, kAng2BohrD);
    z = __dmul_rn(za, kAng2BohrD);
    const double *I = lat + 9;
    double f[3];
    for (int d = 0; d < 3; ++d)
        f[d] = __dadd_rn(__dadd_rn(__dmul_rn(I[3 * d], x), __dmul_rn(I[3 * d + 1], y)), __dmul_rn(I[3 * d + 2], z));
    fold = 0;
    for (int d = 0; d < 3; ++d) {
        const double s = floor(f[d]);
        if (s != 0.0) {
            x = __dsub_rn(x, __dmul_rn(s, lat[3 * d]));
            y = __dsub_rn(y, __dmul_rn(s, lat[3 * d + 1]));
            z = __dsub_rn(z, __dmul_rn(s, lat[3 * d + 2]));
        }
        const int si = (int)fmax(-120.0, fmin(120.0, s));
        fold |= (si + 128) << (8 * d);
    }
}

__device__ __forceinline__ int unpack8(int v, int d) { return ((v >> (8 * d)) & 0xFF) - 128; }

// Skin-list images of pair (i, j): every image within the skin-list cutoff (FP32 screen
// with margin; the exact test is the filter's), stored as (j, image in the unwrapped
// frame) so that later wrapping changes only shift images by the fold counts.
template <bool WRITE>
__device__ __forceinline__ int visit_skin(const SmemF &S, const FastNN &F, int i, int j, float dx, float dy,
                                          float dz, const int *na, int2 *out, int pos, int cap, int fi, int fj) {
    int lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float f = S.ginv[3 * d] * dx + S.ginv[3 * d + 1] * dy + S.ginv[3 * d + 2] * dz;
        lo[d] = max(-na[d] - 2, (int)ceilf(-f - S.wk[3 + d]));
        hi[d] = min(na[d] + 2, (int)floorf(-f + S.wk[3 + d]));
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
                if (ex * ex + ey * ey + ez * ez > F.cut2s) continue;
                if (WRITE && pos + c < cap) {
                    const int u0 = n1 - unpack8(fj, 0) + unpack8(fi, 0), u1 = n2 - unpack8(fj, 1) + unpack8(fi, 1),
                              u2 = n3 - unpack8(fj, 2) + unpack8(fi, 2);
                    out[pos + c] = make_int2(j, (u0 + 128) | ((u1 + 128) << 8) | ((u2 + 128) << 16));
                }
                ++c;
            }
    return c;
}

// Iterator over the set bits of one lane's rows (row pair p: rows p and n-2-p) in
// row-major order; yields (q3, q4).
struct RowBits {
    const unsigned *mask;
    int mw, r1, row, w;
    unsigned m;
    __device__ __forceinline__ void start(const unsigned *mk, int mwords, int p, int nrows) {
        mask = mk;
        mw = mwords;
        r1 = nrows - 1 - p;
        row = p;
        w = (p + 1) >> 5;
        m = mask[row * mw + w];
    }
    // next valid (q3, q4); the caller knows how many there are
    __device__ __forceinline__ void next(int &q3, int &q4) {
        while (m == 0) {
            if (++w >= mw) {
                row = r1;
                w = (r1 + 1) >> 5;
            }
            m = mask[row * mw + w];
        }
        const int b = __ffs(m) - 1;
        m &= m - 1;
        q3 = row;
        q4 = (w << 5) + b;
    }
};

// The triplets of a warp in chunks of at most kTB, so that every lane takes the same
// share however unevenly the valid triplets fall on the lanes' row pairs: each lane feeds
// the triplets of its row pairs (p = lane, lane + 32, ...; row-major) into the warp's
// buffer behind the lanes before it, and the lanes then take equal contiguous blocks of
// the chunk (consecutive entries mostly share their first neighbour q3).
struct TripletFeed {
    RowBits it;
    const unsigned *mask;
    const int *rcnt;
    int mw, npairs, nrows, p, left, total;  // current row pair, its triplets not yet fed; the lane's
    __device__ __forceinline__ void init(const unsigned *mk, int mwords, const int *rc, int lane, int np, int nr) {
        mask = mk;
        rcnt = rc;
        mw = mwords;
        npairs = np;
        nrows = nr;
        total = 0;
        for (int q = lane; q < np; q += 32) {
            const int r1 = nr - 1 - q;
            total += rc[q] + (r1 != q ? rc[r1] : 0);
        }
        p = lane - 32;
        left = 0;
    }
    __device__ __forceinline__ void next(int &q3, int &q4) {
        while (left == 0) {  // a later row pair of the lane holds the triplet (total > 0)
            p += 32;
            const int r1 = nrows - 1 - p;
            left = rcnt[p] + (r1 != p ? rcnt[r1] : 0);
            if (left) it.start(mask, mw, p, nrows);
        }
        it.next(q3, q4);
        --left;
    }
    // the next chunk into buf; returns its size (0: every triplet of the warp was fed)
    __device__ __forceinline__ int fill(uint16_t *buf) {
        int all;
        warp_excl_scan(total, all);
        const int take = all <= kTB ? total : (total < kTB / 32 ? total : kTB / 32);
        int tot;
        const int pos = warp_excl_scan(take, tot);
        for (int e = 0; e < take; ++e) {
            int q3, q4;
            next(q3, q4);
            buf[pos + e] = (uint16_t)(q3 | (q4 << 8));
        }
        total -= take;
        __syncwarp();
        return tot;
    }
};

// Neighbour rows of atom i from its packed words (global scratch), elements codes.
template <int NG>
__device__ __forceinline__ void build_rows(const FastNN &F, const SmemF &S, const WarpF &W, const int *words,
                                           int cnt, int i, int ei, const float *g3l2) {
    const int lane = threadIdx.x & 31;
    const int pa = F.pair_a[ei], pb = F.pair_b[ei];
    const float xhi = S.xh[i], yhi = S.yh[i], zhi = S.zh[i], xli = S.xl[i], yli = S.yl[i], zli = S.zl[i];
    for (int q = lane; q < cnt; q += 32) {
        const int w = words[q];
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
}

// ---- phase 1: neighbour list, rows, descriptors of one central atom ---------------------
template <int NG, int ZM, bool G3ON>
__device__ void nnf_descriptors(const NNDev &M, const FastNN &F, const NNScratch &X, const SmemF &S,
                                const WarpF &W, const FLaunch &L, int t, int64_t base, int i, int N, const int *na,
                                unsigned *mglob, bool rebuild, float *G) {
    constexpr int NZ = popc5(ZM), NQ = 2 * NZ;
    static_assert(NG * NQ <= 32, "too many G3 cells");
    const int lane = threadIdx.x & 31;
    const int ei = S.elem[i];
    const double cut2 = __dmul_rn(M.maxcut, M.maxcut);
    const int mw = L.mw;
    int *words = X.nbw + (base + i) * (int64_t)M.maxnb;

    // ---- neighbour list (RuNNer order) into the global word slot of the bead-atom ------
    // From the atom's skin list when it is valid: its entries are in RuNNer order (j,
    // then images; a fold change shifts all images of one j alike), and each gets the
    // same FP32 screen / exact FP64 test as a full build, so the list is identical.
    int cnt = 0;
    {
        const float xhi = S.xh[i], yhi = S.yh[i], zhi = S.zh[i], xli = S.xl[i], yli = S.yl[i], zli = S.zl[i];
        const int fi = S.fold[i];
        int2 *sk = X.skw + (base + i) * (int64_t)X.skcap;
        int ns = -1;
        if (F.skin > 0.f) {
            ns = X.skcnt[base + i];
            if (rebuild) {
                ns = 0;
                for (int j0 = 0; j0 < N; j0 += 32) {
                    const int j = j0 + lane;
                    float dx = 0.f, dy = 0.f, dz = 0.f;
                    int c = 0;
                    if (j < N) {
                        dx = (S.xh[j] - xhi) + (S.xl[j] - xli);
                        dy = (S.yh[j] - yhi) + (S.yl[j] - yli);
                        dz = (S.zh[j] - zhi) + (S.zl[j] - zli);
                        c = visit_skin<false>(S, F, i, j, dx, dy, dz, na, nullptr, 0, 0, fi, 0);
                    }
                    int tot;
                    const int ex = warp_excl_scan(c, tot);
                    if (c > 0) visit_skin<true>(S, F, i, j, dx, dy, dz, na, sk, ns + ex, X.skcap, fi, S.fold[j]);
                    ns += tot;
                }
                if (ns > X.skcap) ns = -1;
                if (lane == 0) X.skcnt[base + i] = ns;
                __syncwarp();
            }
        }
        if (ns >= 0) {
            const double *Ld = S.lat;
            for (int e0 = 0; e0 < ns; e0 += 32) {
                const int e = e0 + lane;
                bool in = false;
                int word = 0;
                if (e < ns) {
                    const int2 v = sk[e];
                    const int j = v.x, fj = S.fold[j];
                    const int n1 = unpack8(v.y, 0) + unpack8(fj, 0) - unpack8(fi, 0),
                              n2 = unpack8(v.y, 1) + unpack8(fj, 1) - unpack8(fi, 1),
                              n3 = unpack8(v.y, 2) + unpack8(fj, 2) - unpack8(fi, 2);
                    if (abs(n1) <= na[0] && abs(n2) <= na[1] && abs(n3) <= na[2]) {
                        const float *Lf = S.latf;
                        const float ex = ((S.xh[j] - xhi) + (S.xl[j] - xli)) + (float)n1 * Lf[0] + (float)n2 * Lf[3] +
                                         (float)n3 * Lf[6];
                        const float ey = ((S.yh[j] - yhi) + (S.yl[j] - yli)) + (float)n1 * Lf[1] + (float)n2 * Lf[4] +
                                         (float)n3 * Lf[7];
                        const float ez = ((S.zh[j] - zhi) + (S.zl[j] - zli)) + (float)n1 * Lf[2] + (float)n2 * Lf[5] +
                                         (float)n3 * Lf[8];
                        const float rf = ex * ex + ey * ey + ez * ez;
                        in = rf < F.cut2_lo || (rf <= F.cut2_hi && exact_in_cutoff(S, i, j, n1, n2, n3, cut2));
                        word = pack_nb(j, n1, n2, n3);
                    }
                    (void)Ld;
                }
                const unsigned bal = __ballot_sync(0xffffffffu, in);
                const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
                if (in && pos < L.maxnb) words[pos] = word;
                cnt += __popc(bal);
            }
        } else {
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
                if (c > 0) visit_images<true>(S, F, cut2, i, j, dx, dy, dz, na, words, cnt + ex, L.maxnb);
                cnt += tot;
            }
        }
    }
    if (cnt > L.maxnb) {
        if (lane == 0) X.nnstatus[t] = 1;
        cnt = L.maxnb;
    }
    if (lane == 0) X.nbcnt[base + i] = cnt;
    __syncwarp();
    float g3l2[NG];
#pragma unroll
    for (int m = 0; m < NG; ++m) g3l2[m] = F.g3l2[ei][m];
    build_rows<NG>(F, S, W, words, cnt, i, ei, g3l2);

    // ---- radial functions: lane k owns function k and loops over the neighbours (row data
    // are broadcast reads), so no cross-lane reduction and little code ------------------
    const float4 *g2e = S.g2 + ei * kFMaxG2;
    const int ng2 = F.ng2[ei];
    {
        const bool own = lane < ng2;
        const float4 g = own ? g2e[lane] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int gel = own ? (__float_as_int(g.w) >> 8) : -2;
        float a0 = 0.f, a1 = 0.f;
        int q = 0;
        for (; q + 2 <= cnt; q += 2) {
            const float4 c0 = W.rc[q], c1 = W.rc[q + 1];
            const float f0 = W.rb[q].x, f1 = W.rb[q + 1].x;
            const float u0 = c0.y - g.y, u1 = c1.y - g.y;
            const float e0 = ex2a(g.x * u0 * u0), e1 = ex2a(g.x * u1 * u1);
            if ((__float_as_int(c0.z) >> 16) == gel) a0 = fmaf(e0, f0, a0);
            if ((__float_as_int(c1.z) >> 16) == gel) a1 = fmaf(e1, f1, a1);
        }
        if (q < cnt) {
            const float4 c0 = W.rc[q];
            const float u0 = c0.y - g.y;
            if ((__float_as_int(c0.z) >> 16) == gel) a0 = fmaf(ex2a(g.x * u0 * u0), W.rb[q].x, a0);
        }
        if (own) G[__float_as_int(g.w) & 0xFF] = a0 + a1;
    }

    // ---- triplet masks and G3 ----------------------------------------------------------------
    const bool g3 = G3ON && F.hasg3[ei] != 0;
    const int nrows = cnt - 1, npairs = (g3 && nrows > 0) ? (nrows + 1) / 2 : 0;
    if (g3 && npairs == 0) {
        for (int q = lane; q < NG * NQ; q += 32) {
            const int sidx = F.cell_sf[ei][q / NQ][q % NQ];
            if (sidx >= 0) G[sidx] = 0.f;
        }
    }
    if (npairs == 0) return;
    const bool same = F.pair_a[ei] == F.pair_b[ei];
    for (int k = lane; k < cnt * mw; k += 32) W.mask[k] = 0u;
    __syncwarp();
    for (int p = lane; p < npairs; p += 32) {
        const int r0 = p, r1 = nrows - 1 - p, len0 = cnt - 1 - r0;
        const int tot = (r1 == r0) ? len0 : cnt;
        const float4 a0 = W.ra[r0], a1 = W.ra[r1];
        const int c0 = W.code[r0], c1 = W.code[r1];
        unsigned word = 0u;
        int wcur = (r0 + 1) >> 5, row = r0, n0 = 0, n1 = 0;
        for (int c = 0; c < tot; ++c) {
            const bool first = c < len0;
            const int q4 = first ? r0 + 1 + c : c;
            if (!first && row == r0) {  // switch to the second row
                W.mask[row * mw + wcur] = word;
                word = 0u;
                row = r1;
                wcur = q4 >> 5;
            }
            if ((q4 >> 5) != wcur) {
                W.mask[row * mw + wcur] = word;
                word = 0u;
                wcur = q4 >> 5;
            }
            const float4 k = W.ra[q4];
            const int ck = W.code[q4], cj = first ? c0 : c1;
            const float jx = (first ? a0.x : a1.x) - k.x, jy = (first ? a0.y : a1.y) - k.y,
                        jz = (first ? a0.z : a1.z) - k.z;
            const float r2 = jx * jx + jy * jy + jz * jz;
            const bool ok = r2 <= F.rc2 && (cj | ck) == 3 && (!same || (cj & ck) == 3);
            word |= (ok ? 1u : 0u) << (q4 & 31);
            if (first) n0 += ok;
            else n1 += ok;
        }
        if (tot > 0) W.mask[row * mw + wcur] = word;
        W.rcnt[r0] = n0;
        if (r1 != r0) W.rcnt[r1] = n1;
    }
    __syncwarp();
    for (int k = lane; k < cnt * mw; k += 32) mglob[k] = W.mask[k];  // for the force phase

    float acc[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) acc[c] = 0.f;
    TripletFeed tf;
    tf.init(W.mask, mw, W.rcnt, lane, npairs, nrows);
    for (int tot; (tot = tf.fill(W.tbuf)) > 0;) {
        const int e0 = (lane * tot) >> 5, e1 = ((lane + 1) * tot) >> 5;
        int cq3 = -1;
        float4 JA = make_float4(0.f, 0.f, 0.f, 0.f), JB = JA;
        float EJ3 = 0.f;
        for (int e = e0; e < e1; ++e) {
            const int v = W.tbuf[e], q3 = v & 0xFF, q4 = v >> 8;
            if (q3 != cq3) {
                cq3 = q3;
                JA = W.ra[q3];
                JB = W.rb[q3];
                if (NG == 4) EJ3 = W.rc[q3].w;
            }
            const float4 KA = W.ra[q4], KB = W.rb[q4];
            const float jx = JA.x - KA.x, jy = JA.y - KA.y, jz = JA.z - KA.z;
            const float rjk2 = jx * jx + jy * jy + jz * jz;
            const float fcjk = fc_of_s(fminf(rjk2 * F.inv_rc2, 1.f));
            const float u = (JA.x * KA.x + JA.y * KA.y + JA.z * KA.z) * (JA.w * KA.w);
            const float pf = JB.x * KB.x * fcjk;
            const float Ej[4] = {JB.y, JB.z, JB.w, EJ3};
            float Ek[4] = {KB.y, KB.z, KB.w, 0.f};
            if (NG == 4) Ek[3] = W.rc[q4].w;
            float Xm[NG];
#pragma unroll
            for (int m = 0; m < NG; ++m) Xm[m] = Ej[m] * Ek[m] * exp2f(g3l2[m] * rjk2) * pf;
            float Pp[NZ], Pm[NZ];
            zeta_powers<ZM, false>(fmaf(0.5f, u, 0.5f), Pp, nullptr);
            zeta_powers<ZM, false>(fmaf(-0.5f, u, 0.5f), Pm, nullptr);
#pragma unroll
            for (int m = 0; m < NG; ++m)
#pragma unroll
                for (int z = 0; z < NZ; ++z) {
                    acc[m * NQ + 2 * z] = fmaf(Xm[m], Pp[z], acc[m * NQ + 2 * z]);
                    acc[m * NQ + 2 * z + 1] = fmaf(Xm[m], Pm[z], acc[m * NQ + 2 * z + 1]);
                }
        }
        __syncwarp();  // the chunk is read before the next one overwrites it
    }
    reduce_scatter<32>(acc);
    if (lane < NG * NQ) {
        const int sidx = F.cell_sf[ei][lane / NQ][lane % NQ];
        if (sidx >= 0) G[sidx] = 2.f * acc[0];
    }
}

// ---- network for up to kNA atoms of element e (lanes = nodes) --------------------------
// calconenn.f90:83-153 forward, getdnodes_values.f90 + getshortatomic.f90:263-291 back;
// scaling and range check of getshortatomic.f90:174-236.  Replaces the descriptors of
// the descriptors in gb by dE/dG (raw G); returns the energy sum of the group (lane 0).
template <int kNA>
__device__ double nnf_network(const NNDev &M, const FastNN &F, const SmemF &S, const FLaunch &L, float *hs,
                              float *hv, int ei, float *gb, int na, bool do_forces) {
    const int lane = threadIdx.x & 31;
    const int ls = L.ls, lstr = (M.nlayers + 1) * ls;  // per-atom stride in hs/hv
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    for (int s = lane; s < nsf; s += 32) {
        const float4 sc = F.scal[sfb + s];
#pragma unroll
        for (int a = 0; a < kNA; ++a) {
            float v = 0.f;
            if (a < na) {
                const float g = gb[a * L.sgs + s];
                if (g < sc.z || g > sc.w) S.misc[0] = 1;
                v = fmaf(sc.x, g, sc.y);
            }
            hv[a * lstr + s] = v;
        }
    }
    for (int s = nsf + lane; s < ls; s += 32)
#pragma unroll
        for (int a = 0; a < kNA; ++a) hv[a * lstr + s] = 0.f;
    __syncwarp();
    double eout = 0.0;  // per-atom outputs summed in FP64: independent of the grouping
    for (int l = 1; l <= M.nlayers; ++l) {
        const int nprev = M.nodes[ei][l - 1], ncur = M.nodes[ei][l];
        const float *Wl = S.w + F.wofs[ei][l];
        const int str = F.wstr[ei][l];
        const float rn = M.normnodes ? 1.f / (float)nprev : 1.f;
        const uint8_t *act = M.act + (ei * kMaxLayers + (l - 1)) * kMaxNodes;
        if (ncur == 1) {
            float z[kNA];
#pragma unroll
            for (int a = 0; a < kNA; ++a) z[a] = 0.f;
            for (int p = lane; p < nprev; p += 32) {
                const float w = Wl[p * str];
#pragma unroll
                for (int a = 0; a < kNA; ++a) z[a] = fmaf(w, hv[a * lstr + (l - 1) * ls + p], z[a]);
            }
            const uint8_t ac = __ldg(act);
#pragma unroll
            for (int a = 0; a < kNA; ++a) {
                const float zz = (warp_sum(z[a]) + Wl[nprev * str]) * rn;
                const float v = act_f(ac, zz);
                if (lane == 0) {
                    hs[a * lstr + l * ls] = zz;
                    hv[a * lstr + l * ls] = v;
                }
                if (l == M.nlayers && a < na) eout += (double)v;
            }
        } else {
            for (int n = lane; n < ncur; n += 32) {
                float z[kNA];
#pragma unroll
                for (int a = 0; a < kNA; ++a) z[a] = 0.f;
                int p = 0;
                for (; p + 4 <= nprev; p += 4) {
                    const float w0 = Wl[p * str + n], w1 = Wl[(p + 1) * str + n], w2 = Wl[(p + 2) * str + n],
                                w3 = Wl[(p + 3) * str + n];
#pragma unroll
                    for (int a = 0; a < kNA; ++a) {
                        const float4 x = *reinterpret_cast<const float4 *>(hv + a * lstr + (l - 1) * ls + p);
                        z[a] = fmaf(w0, x.x, fmaf(w1, x.y, fmaf(w2, x.z, fmaf(w3, x.w, z[a]))));
                    }
                }
                for (; p < nprev; ++p) {
                    const float w = Wl[p * str + n];
#pragma unroll
                    for (int a = 0; a < kNA; ++a) z[a] = fmaf(w, hv[a * lstr + (l - 1) * ls + p], z[a]);
                }
                const float b = Wl[nprev * str + n];
                const uint8_t ac = __ldg(act + n);
#pragma unroll
                for (int a = 0; a < kNA; ++a) {
                    const float zz = (z[a] + b) * rn;
                    hs[a * lstr + l * ls + n] = zz;
                    hv[a * lstr + l * ls + n] = act_f(ac, zz);
                }
            }
            for (int n = ncur + lane; n < ls; n += 32)
#pragma unroll
                for (int a = 0; a < kNA; ++a) hv[a * lstr + l * ls + n] = 0.f;
        }
        __syncwarp();
    }
    if (!do_forces) return eout;
    // deltas over hs, from the top layer down
    for (int l = M.nlayers; l >= 1; --l) {
        const int ncur = M.nodes[ei][l];
        const float rn = M.normnodes ? 1.f / (float)M.nodes[ei][l - 1] : 1.f;
        const uint8_t *act = M.act + (ei * kMaxLayers + (l - 1)) * kMaxNodes;
        const int nn = l < M.nlayers ? M.nodes[ei][l + 1] : 0;
        const float *Wn = l < M.nlayers ? S.w + F.wofs[ei][l + 1] : nullptr;
        const int strn = l < M.nlayers ? F.wstr[ei][l + 1] : 0;
        for (int n = lane; n < ncur; n += 32) {
            const uint8_t ac = __ldg(act + n);
            float up[kNA];
#pragma unroll
            for (int a = 0; a < kNA; ++a) up[a] = 1.f;
            if (l < M.nlayers) {
#pragma unroll
                for (int a = 0; a < kNA; ++a) up[a] = 0.f;
                const float *row = Wn + n * strn;
                int m = 0;
                for (; m + 4 <= nn; m += 4) {
                    const float4 wv = *reinterpret_cast<const float4 *>(row + m);
#pragma unroll
                    for (int a = 0; a < kNA; ++a) {
                        const float4 dv = *reinterpret_cast<const float4 *>(hs + a * lstr + (l + 1) * ls + m);
                        up[a] = fmaf(wv.x, dv.x, fmaf(wv.y, dv.y, fmaf(wv.z, dv.z, fmaf(wv.w, dv.w, up[a]))));
                    }
                }
                for (; m < nn; ++m)
#pragma unroll
                    for (int a = 0; a < kNA; ++a) up[a] = fmaf(row[m], hs[a * lstr + (l + 1) * ls + m], up[a]);
            }
            float d[kNA];
#pragma unroll
            for (int a = 0; a < kNA; ++a)
                d[a] = rn * act_df(ac, hs[a * lstr + l * ls + n], hv[a * lstr + l * ls + n]) * up[a];
#pragma unroll
            for (int a = 0; a < kNA; ++a) hs[a * lstr + l * ls + n] = d[a];
        }
        for (int n = ncur + lane; n < ls; n += 32)
#pragma unroll
            for (int a = 0; a < kNA; ++a) hs[a * lstr + l * ls + n] = 0.f;
        __syncwarp();
    }
    {
        const int n1 = M.nodes[ei][1];
        for (int s = lane; s < nsf; s += 32) {
            const float *row = S.w + F.wofs[ei][1] + s * F.wstr[ei][1];
            float u[kNA];
#pragma unroll
            for (int a = 0; a < kNA; ++a) u[a] = 0.f;
            int m = 0;
            for (; m + 4 <= n1; m += 4) {
                const float4 wv = *reinterpret_cast<const float4 *>(row + m);
#pragma unroll
                for (int a = 0; a < kNA; ++a) {
                    const float4 dv = *reinterpret_cast<const float4 *>(hs + a * lstr + ls + m);
                    u[a] = fmaf(wv.x, dv.x, fmaf(wv.y, dv.y, fmaf(wv.z, dv.z, fmaf(wv.w, dv.w, u[a]))));
                }
            }
            for (; m < n1; ++m)
#pragma unroll
                for (int a = 0; a < kNA; ++a) u[a] = fmaf(row[m], hs[a * lstr + ls + m], u[a]);
            const float dsc = F.dscal[sfb + s];
#pragma unroll
            for (int a = 0; a < kNA; ++a)
                if (a < na) gb[a * L.sgs + s] = u[a] * dsc;
        }
    }
    __syncwarp();
    return eout;
}

// ---- phase 3: forces of one central atom ---------------------------------------------
template <int NG, int ZM, bool G3ON>
__device__ void nnf_forces(const NNDev &M, const FastNN &F, const NNScratch &X, const SmemF &S, const WarpF &W,
                           const FLaunch &L, int64_t base, int i, const unsigned *mglob, const float *dG) {
    constexpr int NZ = popc5(ZM), NQ = 2 * NZ;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int ei = S.elem[i];
    const int mw = L.mw;
    const int cnt = X.nbcnt[base + i];
    const int *words = X.nbw + (base + i) * (int64_t)M.maxnb;
    float g3l2[NG];
#pragma unroll
    for (int m = 0; m < NG; ++m) g3l2[m] = F.g3l2[ei][m];
    build_rows<NG>(F, S, W, words, cnt, i, ei, g3l2);

    // ---- radial part: slot forces start here -----------------------------------------------
    for (int q = lane; q < cnt; q += 32) {
        W.sfx[q] = 0.f;
        W.sfy[q] = 0.f;
        W.sfz[q] = 0.f;
    }
    // d/dr sum_k c_k exp(-eta_k (r - rs_k)^2) fc = sum_k c_k e_k (dfc - 2 eta_k (r - rs_k) fc);
    // lanes = neighbours, a short loop over the functions (table and c_k broadcast)
    const float4 *g2e = S.g2 + ei * kFMaxG2;
    const int ng2 = F.ng2[ei];
    for (int q = lane; q < cnt; q += 32) {
        const float4 c = W.rc[q], av = W.ra[q];
        const int el = __float_as_int(c.z) >> 16;
        const float fc = W.rb[q].x, dfc = c.x * c.y, r = c.y;
        float dsum = 0.f;
#pragma unroll 2
        for (int k = 0; k < ng2; ++k) {
            const float4 g = g2e[k];
            const int gw = __float_as_int(g.w);
            const float u = r - g.y;
            const float t = dG[gw & 0xFF] * ex2a(g.x * u * u) * fmaf(g.z * u, fc, dfc);
            if ((gw >> 8) == el) dsum += t;
        }
        const float fr = dsum * av.w;
        W.sfx[q] -= fr * av.x;
        W.sfy[q] -= fr * av.y;
        W.sfz[q] -= fr * av.z;
    }

    // ---- angular part ------------------------------------------------------------------------
    const bool g3 = G3ON && F.hasg3[ei] != 0;
    const int nrows = cnt - 1, npairs = (g3 && nrows > 0) ? (nrows + 1) / 2 : 0;
    if (npairs > 0) {
        for (int k = lane; k < cnt * mw; k += 32) W.mask[k] = mglob[k];
        __syncwarp();
        for (int q = lane; q < nrows; q += 32) {
            int c = 0;
            for (int w = (q + 1) >> 5; w < mw; ++w) c += __popc(W.mask[q * mw + w]);
            W.rcnt[q] = c;
        }
        float Wy[NG][NQ], Wz[NG][NQ], eta[NG];
#pragma unroll
        for (int m = 0; m < NG; ++m) {
            eta[m] = F.g3eta[ei][m];
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const int sidx = F.cell_sf[ei][m][q];
                const float c = sidx >= 0 ? dG[sidx] : 0.f;
                Wy[m][q] = 2.f * c;
                Wz[m][q] = F.cell_lz[q] * c;
            }
        }
        __syncwarp();
        TripletFeed tf;
        tf.init(W.mask, mw, W.rcnt, lane, npairs, nrows);
        for (int tot; (tot = tf.fill(W.tbuf)) > 0;) {
            const int e0 = (lane * tot) >> 5, e1 = ((lane + 1) * tot) >> 5;
            int cq3 = -1;
            float4 JA = make_float4(0.f, 0.f, 0.f, 0.f), JB = JA, JC = JA;
            float fjx = 0.f, fjy = 0.f, fjz = 0.f;
            for (int e = e0; e < e1; ++e) {
                const int v = W.tbuf[e], q3 = v & 0xFF, q4 = v >> 8;
                if (q3 != cq3) {
                    if (cq3 >= 0) {
                        red_shared(&W.sfx[cq3], fjx);
                        red_shared(&W.sfy[cq3], fjy);
                        red_shared(&W.sfz[cq3], fjz);
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
                    for (int z = 0; z < NZ; ++z) {
                        Y = fmaf(Wy[m][2 * z], Pp[z], Y);
                        Y = fmaf(Wy[m][2 * z + 1], Pm[z], Y);
                        Z = fmaf(Wz[m][2 * z], Qp[z], Z);
                        Z = fmaf(Wz[m][2 * z + 1], Qm[z], Z);
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
                red_shared(&W.sfx[q4], -(gk * KA.x + gx * JA.x));
                red_shared(&W.sfy[q4], -(gk * KA.y + gx * JA.y));
                red_shared(&W.sfz[q4], -(gk * KA.z + gx * JA.z));
            }
            if (cq3 >= 0) {
                red_shared(&W.sfx[cq3], fjx);
                red_shared(&W.sfy[cq3], fjy);
                red_shared(&W.sfz[cq3], fjz);
            }
            __syncwarp();  // the chunk is read before the next one overwrites it
        }
    }
    __syncwarp();

    // ---- scatter: neighbours get their slot forces, the centre minus their sum ----------
    float *fx = S.f3, *fy = fx + L.max_atoms, *fz = fy + L.max_atoms;
    float fix = 0.f, fiy = 0.f, fiz = 0.f;
    for (int q = lane; q < cnt; q += 32) {
        const int j = __float_as_int(W.rc[q].z) & 0xFFFF;
        const float sx = W.sfx[q], sy = W.sfy[q], sz = W.sfz[q];
        red_shared(&fx[j], sx);
        red_shared(&fy[j], sy);
        red_shared(&fz[j], sz);
        fix -= sx;
        fiy -= sy;
        fiz -= sz;
    }
    fix = warp_sum(fix);
    fiy = warp_sum(fiy);
    fiz = warp_sum(fiz);
    if (lane == 0) {
        red_shared(&fx[i], fix);
        red_shared(&fy[i], fiy);
        red_shared(&fz[i], fiz);
    }
    __syncwarp();
}

// lattice rows and inverse (bohr), their FP32 copies and the image half-widths of the
// list cutoff (0..2) and the skin-list cutoff (3..5) of trajectory t
__device__ void cell_setup(const Batch &B, const NNDev &M, const FastNN &F, const SmemF &S, int t) {
    const int tid = threadIdx.x;
    if (tid == 0) acsf_lattice(B.box + 9 * t, S.lat);
    __syncthreads();
    if (tid < 9) {
        S.latf[tid] = (float)S.lat[tid];
        S.ginv[tid] = (float)S.lat[9 + tid];
    }
    if (tid < 6) {
        const int d = tid % 3;
        const double *I = S.lat + 9 + 3 * d;
        const double bn = sqrt(I[0] * I[0] + I[1] * I[1] + I[2] * I[2]);
        const double rc = tid < 3 ? M.maxcut : M.maxcut + (double)F.skin;
        S.wk[tid] = (float)(rc * bn * (1.0 + 1e-4) + 1e-4);
    }
    __syncthreads();
}

// atoms of the trajectory ordered by element (network groups share an element)
__device__ void order_by_element(const NNDev &M, const SmemF &S, const FLaunch &L, int N) {
    if (threadIdx.x == 0) {
        int *off = S.byel + L.max_atoms;
        int k = 0;
        for (int e = 0; e < M.nelem; ++e) {
            off[e] = k;
            for (int i = 0; i < N; ++i)
                if (S.elem[i] == e) S.byel[k++] = i;
        }
        off[M.nelem] = k;
    }
    __syncthreads();
}

// ---- one bead ---------------------------------------------------------------------------
// Warps take 2 or 4 atoms at a time: descriptors of each atom, the network of each run of
// one element, forces of each atom; no CTA barrier between the stages.  The lattice
// tables (S.lat, latf, ginv, wk) are set once per trajectory by cell_setup.
template <int NG, int ZM, bool G3ON>
__device__ bool nnf_bead(const Batch &B, const NNDev &M, const FastNN &F, const NNScratch &X, const SmemF &S,
                         const FLaunch &L, int t, int b, bool do_forces, bool skip_if_flagged) {
    const int N = B.natoms[t];
    const int64_t base = B.ba_off[t] + (int64_t)b * N;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int bead = B.bead_off[t] + b;
    if (tid == 0) {
        S.misc[0] = 0;
        S.misc[1] = 0;
        S.misc[3] = 0;
    }
    __syncthreads();
    float d2max = 0.f;
    for (int i = tid; i < N; i += nt) {
        double x, y, z;
        int fold;
        const double rx = B.rx[base + i], ry = B.ry[base + i], rz = B.rz[base + i];
        wrap_fold(rx, ry, rz, S.lat, x, y, z, fold);
        S.px[i] = x;
        S.py[i] = y;
        S.pz[i] = z;
        S.fold[i] = fold;
        const float xh = (float)x, yh = (float)y, zh = (float)z;
        S.xh[i] = xh;
        S.yh[i] = yh;
        S.zh[i] = zh;
        S.xl[i] = (float)(x - (double)xh);
        S.yl[i] = (float)(y - (double)yh);
        S.zl[i] = (float)(z - (double)zh);
        if (F.skin > 0.f) {
            const double *r0 = X.skref + 3 * (base + i);
            const float ddx = (float)(rx - r0[0]), ddy = (float)(ry - r0[1]), ddz = (float)(rz - r0[2]);
            d2max = fmaxf(d2max, ddx * ddx + ddy * ddy + ddz * ddz);
        }
    }
    if (do_forces)
        for (int k = tid; k < 3 * L.max_atoms; k += nt) S.f3[k] = 0.f;
    if (F.skin > 0.f) atomicMax(&S.misc[3], __float_as_int(d2max));  // non-negative floats order as ints
    __syncthreads();
    // skin lists are rebuilt when invalid or when some atom moved more than half the skin
    // (positions in A; the skin is in bohr)
    if (tid == 0) {
        const float half = 0.5f * F.skin * (float)kBohr2Ang;
        S.misc[2] = F.skin > 0.f && (X.skok[bead] == 0 || __int_as_float(S.misc[3]) > half * half) ? 1 : 0;
    }
    __syncthreads();
    const bool rebuild = S.misc[2] != 0;
    if (F.skin > 0.f) {
        if (rebuild) {
            for (int i = tid; i < N; i += nt) {
                double *r0 = X.skref + 3 * (base + i);
                r0[0] = B.rx[base + i];
                r0[1] = B.ry[base + i];
                r0[2] = B.rz[base + i];
            }
            if (tid == 0) X.skok[bead] = 1;
        }
    }
    const int na[3] = {X.img[3 * t], X.img[3 * t + 1], X.img[3 * t + 2]};
    unsigned *mscr = X.mscr + (size_t)blockIdx.x * X.mcap;
    const size_t mstride = (size_t)L.maxnb * L.mw;
    const int *off = S.byel + L.max_atoms;
    const int nnn = off[M.nelem];  // network atoms, ordered by element
    double e_warp = 0.0;
    float *hs = (float *)(S.warp_base + (size_t)warp * S.warp_bytes);
    float *hv = hs + kNAmax * (M.nlayers + 1) * L.ls;
    const WarpF W = carve_warp(S, L, warp);
    // grabs of 4 atoms (network ILP) on large beads, of 2 on small ones (tail balance);
    // a grab that spans two elements runs the network once per element
    const int gsz = N >= 96 ? 4 : 2;
    for (;;) {
        int st = 0, n = 0;
        if (lane == 0) {
            st = atomicAdd(&S.misc[1], gsz);
            n = min(gsz, nnn - st);
        }
        st = __shfl_sync(0xffffffffu, st, 0);
        n = __shfl_sync(0xffffffffu, n, 0);
        if (n <= 0) break;
        const int *atoms = S.byel + st;
        for (int a = 0; a < n; ++a)
            nnf_descriptors<NG, ZM, G3ON>(M, F, X, S, W, L, t, base, atoms[a], N, na, mscr + (size_t)atoms[a] * mstride,
                                    rebuild, W.gb + a * L.sgs);
        __syncwarp();
        for (int r0 = 0; r0 < n;) {  // runs of one element
            const int e = S.elem[atoms[r0]];
            int r1 = r0 + 1;
            while (r1 < n && S.elem[atoms[r1]] == e) ++r1;
            const int m = r1 - r0;
            float *gb = W.gb + r0 * L.sgs;
            const double en = nnf_network<4>(M, F, S, L, hs, hv, e, gb, m, do_forces);
            if (lane == 0) e_warp += en + m * (M.remove_atom_energies ? M.atom_energy[e] : 0.0);
            r0 = r1;
        }
        if (do_forces)
            for (int a = 0; a < n; ++a)
                nnf_forces<NG, ZM, G3ON>(M, F, X, S, W, L, base, atoms[a], mscr + (size_t)atoms[a] * mstride,
                                   W.gb + a * L.sgs);
    }
    const double etot = block_sum(e_warp, S.red);  // contains __syncthreads: flag visible
    if (F.skin > 0.f && rebuild) {
        // an overflowing skin list invalidates the bead's lists: rebuilt on the next step
        for (int k = tid; k < N; k += nt)
            if (X.skcnt[base + k] < 0) X.skok[bead] = 0;
    }
    const bool flagged = S.misc[0] != 0;
    if (skip_if_flagged && flagged) {
        __syncthreads();
        return true;
    }
    if (tid == 0) B.epot[bead] += etot * kHa2eVF;
    if (!do_forces) {
        __syncthreads();
        return flagged;
    }
    const double c = kHa2eVF * kAng2BohrD;
    for (int i = tid; i < N; i += nt) {
        const float fx = S.f3[i], fy = S.f3[L.max_atoms + i], fz = S.f3[2 * L.max_atoms + i];
        B.fx[base + i] += (double)fx * c;
        B.fy[base + i] += (double)fy * c;
        B.fz[base + i] += (double)fz * c;
    }
    __syncthreads();
    return flagged;
}

// calc_force (force.f90:40-86) with the network: zero, free ring-polymer step, per-bead
// prediction (EMT for a flagged bead of the surrogate), accelerations.
template <int NG, int ZM, bool G3ON>
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
        const bool flagged = nnf_bead<NG, ZM, G3ON>(B, M, F, X, S, L, T.t, b, do_forces, L.surrogate != 0);
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

// network weights into their padded shared-memory layout; radial-function table
__device__ void load_model_smem(const NNDev &M, const FastNN &F, const SmemF &S) {
    for (int e = 0; e < M.nelem; ++e)
        for (int l = 1; l <= M.nlayers; ++l) {
            const int nprev = M.nodes[e][l - 1], ncur = M.nodes[e][l], str = F.wstr[e][l];
            const float *src = M.wf + (size_t)e * M.maxweights + M.woff[e][l];
            float *dst = S.w + F.wofs[e][l];
            for (int k = threadIdx.x; k < (nprev + 1) * str; k += blockDim.x) {
                const int p = k / str, n = k % str;
                dst[k] = n < ncur ? src[p * ncur + n] : 0.f;
            }
        }
    for (int k = threadIdx.x; k < M.nelem * kFMaxG2; k += blockDim.x) S.g2[k] = F.g2tab[k];
    __syncthreads();
}

// mode 0: forces, 1: energies only, 2: nsteps fused MD steps (propagate_1, forces,
// propagate_2, exit test), as the generic network kernels.
// Angular models run two CTAs per SM with up to 128 registers a thread (at the HDNNP
// benchmark shape their shared memory, 97 KB a CTA, leaves no room for a third, and under
// the 80 registers of three CTAs the triplet walks spilled); radial-only models keep three.
template <int NG, int ZM, bool G3ON>
__global__ void __launch_bounds__(kFBlock, G3ON ? 2 : 3)
    nnf_kernel(Batch B, NNDev M, FastNN F, EmtConst E, NNScratch X, PropParams P, FLaunch L, const int *order,
               int *counter, int nsteps, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    const SmemF S = carve_f(smem_raw, L, B.max_beads, F.wtotal, M.nelem, M.nlayers);
    SmemEmt<double> SE = carve_smem<double>(S.warp_base, B.max_atoms, B.max_beads);
    SE.red = S.red;
    SE.cjk = S.cjk;
    load_model_smem(M, F, S);
    for (;;) {
        if (threadIdx.x == 0) work_slot = atomicAdd(counter, 1);
        __syncthreads();
        const int w = work_slot;
        __syncthreads();
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, S.cjk);
        for (int i = threadIdx.x; i < T.N; i += blockDim.x) S.elem[i] = (int8_t)M.elem_of_type[B.type[T.aoff + i]];
        __syncthreads();
        order_by_element(M, S, L, T.N);
        cell_setup(B, M, F, S, t);
        if (mode != 2) {
            nnf_calc_force<NG, ZM, G3ON>(B, M, F, E, X, P, S, SE, L, T, mode == 0);
            continue;
        }
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, S.cjk, step, S.red);
            nnf_calc_force<NG, ZM, G3ON>(B, M, F, E, X, P, S, SE, L, T, true);
            propagate_2(B, P, T, step);
            {
                int near;
                double rv[3];
                const double dmin = closest_approach_step(B, T, SE.cell, SE.red, &near, rv);
                if (threadIdx.x == 0) observe_step(B, P, T, step, dmin, near, rv[0], rv[1], rv[2]);
            }
            end_of_step(B, P, T, step);
        }
    }
}

template <int NG, int ZM, bool G3ON>
cudaError_t nnf_launch_t(const LaunchCfg &c, const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                         const NNScratch &X, const PropParams &P, const FLaunch &L, size_t sm, int nsteps, int mode) {
    cudaError_t e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(nnf_kernel<NG, ZM, G3ON>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    nnf_kernel<NG, ZM, G3ON><<<c.grid, kFBlock, sm, c.stream>>>(B, M, F, E, X, P, L, c.order, c.counter, nsteps, mode);
    return cudaGetLastError();
}

template <int NG, int ZM, bool G3ON>
int nnf_occupancy_t(size_t sm) {
    int n = 0;
    cudaFuncSetAttribute(nnf_kernel<NG, ZM, G3ON>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nnf_kernel<NG, ZM, G3ON>, kFBlock, sm);
    return n;
}

}  // namespace

// Kernels exist for the zeta set {1, 4, 16} (a subset runs with zero-weight cells) and
// 1..4 eta slots.
int nnf_zm_supported(int zm) { return (zm & ~0x15) == 0 ? 0x15 : 0; }

// radial-only models (no G3 anywhere) get a kernel without the angular stages
#define MDT_NNF_DISPATCH(CALL)                                                                       \
    if (!F.anyg3) {                                                                                  \
        CALL(1, 0x15, false);                                                                        \
    } else {                                                                                         \
        switch (F.ng) {                                                                              \
            case 1: CALL(1, 0x15, true); case 2: CALL(2, 0x15, true); case 3: CALL(3, 0x15, true);   \
            case 4: CALL(4, 0x15, true); default: break;                                             \
        }                                                                                            \
    }

size_t nnf_total_smem(const Batch &B, const NNDev &M, const FastNN &F) { return nnf_smem_total(B, M, F); }

int nnf_warps_per_cta() { return kFW; }

int nnf_resident_ctas(const Batch &B, const NNDev &M, const FastNN &F) {
    const size_t sm = nnf_smem_total(B, M, F);
#define MDT_OCC(NG, ZM, G3ON) return std::max(1, nnf_occupancy_t<NG, ZM, G3ON>(sm));
    MDT_NNF_DISPATCH(MDT_OCC)
#undef MDT_OCC
    return 1;
}

cudaError_t launch_nnf(const LaunchCfg &c, const Batch &B, const NNDev &M, const FastNN &F, const EmtConst &E,
                       const NNScratch &X, const PropParams &P, int nsteps, int mode, bool surrogate) {
    const FLaunch L = flaunch(B, M, surrogate ? 1 : 0);
    const size_t sm = nnf_smem_total(B, M, F);
#define MDT_LAUNCH(NG, ZM, G3ON) return nnf_launch_t<NG, ZM, G3ON>(c, B, M, F, E, X, P, L, sm, nsteps, mode);
    MDT_NNF_DISPATCH(MDT_LAUNCH)
#undef MDT_LAUNCH
    return cudaErrorInvalidValue;
}

}  // namespace mdt
