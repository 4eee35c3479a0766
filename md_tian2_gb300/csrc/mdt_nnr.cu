// mdt_nnr.cu -- FP32 thread-per-atom force evaluation and MD step for radial-only HDNNP /
// EMT-surrogate models (every symmetry function a G2 shifted Gaussian under one cosine
// cutoff, at most two elements, one or two hidden layers of at most 32 nodes).
//
// Same prediction as the generic and warp-per-atom kernels (RuNNer's short-range
// network, src/pes_nene_mod.f90:7145-7368 with RuNNer_src/atomsymfunction2.f90 and
// calconenn.f90 / getdnodes_values.f90 / getshortatomic.f90), organised so that a
// thread owns one atom from its neighbour list to its force:
//
//  * CTA = a pack of whole trajectories (host-planned, atoms of all of them <= block):
//    thread k is atom k of the pack; positions, forces and per-thread network buffers
//    in shared memory; CTA barriers only around the propagator half-steps and the
//    per-trajectory reductions.
//  * Verlet skin lists per bead-atom, entry-major per bead (entry e of atom i at
//    e*N + i, so a warp's loads coalesce), entries grouped by neighbour element, each
//    (j, image in the unwrapped frame): distances come from unwrapped positions, so the
//    lists survive wrapping.  Rebuilt when some atom of the trajectory moved more than
//    half the skin.
//  * Radial functions: every centre element carries the same (eta, r_s) list per
//    neighbour element (the admission test), so the Gaussian loop is uniform across
//    lanes and its parameters are constant-bank operands; descriptors accumulate in
//    registers (template group sizes KA, KB).
//  * Network: lane = atom; the weights of both elements sit in shared memory (element 1
//    shifted by 64 bytes so a warp with both elements reads two rows in one pass), rows
//    broadcast with 128-bit loads against 32 register accumulators; hidden layers padded
//    to 32 nodes with zero weights (exact).  The backward pass keeps the activation
//    derivatives of the forward pass, so dE/dG costs three matrix-vector products.
//  * Forces: reverse mode; the neighbour's share by a shared-memory reduction, the
//    centre's in registers.
//  * A trajectory whose descriptors leave the training range is recomputed by FP64 EMT
//    (surrogate) with the whole CTA, before the second propagator half-step.
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_fastmath.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"
#include "mdt_acsf.cuh"
#include "mdt_prop.cuh"
#include "mdt_tc.cuh"
#include "../../include/mdt_gpu.h"

namespace mdt {

namespace {

constexpr int kRW = 32;          // padded hidden width
constexpr double kHa2eVR = 27.21138602;

struct SmemR {
    float4 *ph, *pl;                     // [slot] unwrapped positions (bohr), FP32 hi/lo split (x, y, z, 0)
    float *f3;                           // [3][bs] neighbour force accumulators (Ha/bohr)
    double *ea;                          // [slot] atomic energies (Ha)
    double *lc;                          // [8][slot] Langevin coefficients of the atom (see LcR)
    double *im;                          // [slot] 1 / mass
    int8_t *elem;                        // [slot]
    float *hb;                           // [hbw][bs] per-thread network buffer
    float *w;                            // weight blocks of the elements
    float4 *scal;                        // [e][q]: scaled = x g + y, range [z, w]
    float *dscal;                        // [e][q]
    int *tr_t, *tr_st, *tr_n;
    // per-step flags, buffered by step (step & 1; tr_stat by step % 3): descriptors out of
    // range, largest squared displacement, skin-list overflow, state not finite, running
    // during the step
    int *tr_flag, *tr_d2, *tr_over, *tr_bad, *tr_stat;
    // tensor-core network (TC kernels): A-operand tiles (alias hb), bf16 B operands and FP32
    // vectors of both elements, one mbarrier per 128-row tile, the TMEM base address
    unsigned char *at, *wb;
    float *wv;
    uint64_t *tcbar;
    uint32_t *tslot;
    float *tr_lat;                       // [s][24]: lattice rows (9), inverse rows (9), skin half-widths (3)
    double *red;
    int *misc;                           // [0] pack taken from the work queue
    unsigned char *emt;                  // EMT fallback area (aliases hb)
};

__host__ __device__ constexpr size_t r16r(size_t b) { return (b + 15) & ~size_t(15); }

// Shared memory of a CTA, laid out for kRS threads whatever the block (every offset a
// compile-time constant of the shape, so no shared-memory address occupies a register)
constexpr int kRS = kRBlockMax;

// per-thread network buffer (FP32 network) or operand tiles (tensor-core network); either
// doubles as the EMT fallback area
// tcm: 0 FP32 network, 1 BF16 operands, 2 BF16 operands split in a high and a low part
// (the A tiles and the B operands exist twice)
__host__ __device__ constexpr size_t hb_bytes(int nin, int nh, int tcm) {
    return tcm == 0 ? 4 * (size_t)nnr_hbw(nin, nh) * kRS
                    : (tcm == 2 && 2 * (size_t)kTcTiles * 128 * nnr_tw(nin) * 2 > nnr_tc_hb(nin)
                           ? 2 * (size_t)kTcTiles * 128 * nnr_tw(nin) * 2
                           : nnr_tc_hb(nin));
}
__host__ __device__ constexpr size_t w_bytes(int nin, int nh, int tcm) {
    return tcm == 0 ? 4 * (size_t)nnr_wtotal(nin, nh)
                    : (size_t)(tcm == 2 ? 2 : 1) * 2 * nnr_tc_bel(nin) + 2 * 4 * (size_t)kTcVec;
}

__host__ __device__ constexpr size_t smem_r(int nin, int nh, int tc) {
    return 2 * r16r(16 * (size_t)kRS) + r16r(12 * (size_t)kRS) + r16r(8 * (size_t)kRS) + r16r(64 * (size_t)kRS) +
           r16r(8 * (size_t)kRS) + r16r(kRS) + r16r(hb_bytes(nin, nh, tc)) + r16r(w_bytes(nin, nh, tc)) +
           r16r(16 * 2 * (size_t)nin) + r16r(4 * 2 * (size_t)nin) + 3 * r16r(4 * kRMaxTraj) + 4 * r16r(8 * kRMaxTraj) +
           r16r(12 * kRMaxTraj) + r16r(4 * 24 * kRMaxTraj) + r16r(8 * 64) + r16r(16) + r16r(8 * kTcTiles) + r16r(16);
}

template <int NIN, int NH, int TC>
__device__ __forceinline__ SmemR carve_r(unsigned char *base) {
    SmemR s;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += r16r(bytes);
        return p;
    };
    s.ph = (float4 *)take(16 * (size_t)kRS);
    s.pl = (float4 *)take(16 * (size_t)kRS);
    s.f3 = (float *)take(12 * (size_t)kRS);
    s.ea = (double *)take(8 * (size_t)kRS);
    s.lc = (double *)take(64 * (size_t)kRS);
    s.im = (double *)take(8 * (size_t)kRS);
    s.elem = (int8_t *)take(kRS);
    s.hb = (float *)take(hb_bytes(NIN, NH, TC));
    s.emt = (unsigned char *)s.hb;
    s.at = (unsigned char *)s.hb;
    s.w = (float *)take(w_bytes(NIN, NH, TC));
    s.wb = (unsigned char *)s.w;
    s.wv = (float *)(s.wb + (size_t)(TC == 2 ? 2 : 1) * 2 * nnr_tc_bel(NIN));
    s.scal = (float4 *)take(16 * 2 * (size_t)NIN);
    s.dscal = (float *)take(4 * 2 * (size_t)NIN);
    s.tr_t = (int *)take(4 * kRMaxTraj);
    s.tr_st = (int *)take(4 * kRMaxTraj);
    s.tr_n = (int *)take(4 * kRMaxTraj);
    s.tr_flag = (int *)take(8 * kRMaxTraj);
    s.tr_d2 = (int *)take(8 * kRMaxTraj);
    s.tr_over = (int *)take(8 * kRMaxTraj);
    s.tr_bad = (int *)take(8 * kRMaxTraj);
    s.tr_stat = (int *)take(12 * kRMaxTraj);
    s.tr_lat = (float *)take(4 * 24 * kRMaxTraj);
    s.red = (double *)take(8 * 64);
    s.misc = (int *)take(16);
    s.tcbar = (uint64_t *)take(8 * kTcTiles);
    s.tslot = (uint32_t *)take(16);
    return s;
}

// small non-negative integer b (< 2^23) to float by the exponent trick (two full-rate
// instructions instead of a conversion)
__device__ __forceinline__ float small_to_float(unsigned b) {
    return __int_as_float(0x4B000000 | b) - 8388608.f;
}

// One thread's view of its atom.
struct AtomR {
    int s, i, st, N, ei, algo;    // pack trajectory, atom, first slot, atoms, element, propagator
    int64_t base;                 // bead-atom slot of atom 0 of the bead
    float xhi, yhi, zhi, xli, yli, zli;
    float L[9];                   // lattice rows (bohr)
};

__device__ __forceinline__ void rel_pos(const SmemR &S, const AtomR &A, int js, float &dx, float &dy, float &dz) {
    const float4 h = S.ph[js], l = S.pl[js];  // one 16-byte load per part
    dx = (h.x - A.xhi) + (l.x - A.xli);
    dy = (h.y - A.yhi) + (l.y - A.yli);
    dz = (h.z - A.zhi) + (l.z - A.zli);
}

// Skin-list entry: j (bits 0-9) and the image (n1, n2, n3) in the unwrapped frame, each
// + 64 in 7 bits (bits 10-16, 17-23, 24-30).  An image outside [-63, 63] (atoms that
// drifted more than 63 cells apart) does not fit: the list overflows and the atom takes
// the full scan.
constexpr int kImgBias = 64;
__device__ __forceinline__ unsigned pack_entry(int j, int n1, int n2, int n3) {
    return (unsigned)j | (unsigned)(n1 + kImgBias) << 10 | (unsigned)(n2 + kImgBias) << 17 |
           (unsigned)(n3 + kImgBias) << 24;
}
__device__ __forceinline__ bool image_fits(int n) { return n >= -63 && n <= 63; }

// Image range of dimension d for the displacement with fractional coordinate f: the n
// with |f + n| <= w.  Returns false for a non-finite or absurd displacement; the range
// holds at most 65 images.
__device__ __forceinline__ bool image_range(float f, float w, int &lo, int &hi) {
    if (!(fabsf(f) < 1e6f) || !(w < 64.f)) return false;
    lo = (int)ceilf(-f - w);
    hi = (int)floorf(-f + w);
    return true;
}

// Calls fn(group g as integral constant, pack slot of j, d, r^2) for every neighbour of
// the atom inside the cutoff: from the skin list when it is valid (cnt >= 0; the skin
// shell's entries beyond the cutoff are passed too and fn masks them), else by a full image
// scan of the trajectory.
// SPREAD: each lane starts its list at its own fraction of the list ((lane * len) / 32) and
// wraps around.  Neighbouring atoms of a warp have nearly the same sorted lists, so walking
// them in step sends the lanes to the same neighbour j at once; where fn adds into j's
// shared-memory force (red.shared) those lanes serialise on one address.  Spread, the lanes
// meet different j.  (The descriptor walk keeps list order: there equal j make its position
// loads broadcasts.)
template <int G> struct GC { static constexpr int value = G; };

// UNR: unroll of the list walk (measured per network arithmetic: 1 with the tensor-core
// network, 3 with the FP32 network; each about 1-2 % faster than the other choices)
template <bool SPREAD = false, int UNR = 2, class Fn>
__device__ __forceinline__ void for_neighbours(const RadialNN &R, const SmemR &S, const AtomR &A, const unsigned *sk,
                                               int cnt, Fn &&fn) {
    if (cnt >= 0) {
        const int n0 = cnt & 0xFFFF, n1 = cnt >> 16;
        // entries two iterations ahead are in flight while one is processed
        auto walk = [&](auto gc, int e0, int e1) {
            const int len = e1 - e0;
            const unsigned *p = sk + (size_t)e0 * A.N + A.i;
            // entry q of the walk's order sits at list position q (or at q shifted by the
            // lane's start, modulo len)
            int q0 = SPREAD ? (int)(((unsigned)(threadIdx.x & 31) * (unsigned)len) >> 5) : 0;
            auto next = [&](int q) { return q + 1 == len ? 0 : q + 1; };
            unsigned w0 = len > 0 ? p[(size_t)q0 * A.N] : 0u;
            int q1 = next(q0);
            unsigned w1 = len > 1 ? p[(size_t)q1 * A.N] : 0u;
            int q2 = next(q1);
#pragma unroll UNR
            for (int e = 0; e < len; ++e) {
                const unsigned v = w0;
                w0 = w1;
                if (e + 2 < len) {
                    w1 = p[(size_t)q2 * A.N];
                    q2 = next(q2);
                }
                const int js = A.st + (int)(v & 1023u);
                const float m1 = small_to_float((v >> 10) & 127u) - (float)kImgBias;
                const float m2 = small_to_float((v >> 17) & 127u) - (float)kImgBias;
                const float m3 = small_to_float((v >> 24) & 127u) - (float)kImgBias;
                float dx, dy, dz;
                rel_pos(S, A, js, dx, dy, dz);
                dx += fmaf(m1, A.L[0], fmaf(m2, A.L[3], m3 * A.L[6]));
                dy += fmaf(m1, A.L[1], fmaf(m2, A.L[4], m3 * A.L[7]));
                dz += fmaf(m1, A.L[2], fmaf(m2, A.L[5], m3 * A.L[8]));
                // entries of the skin shell (r >= rc) go through the same arithmetic with the
                // cutoff function masked to zero: no divergent branch in the walk
                fn(gc, js, dx, dy, dz, dx * dx + dy * dy + dz * dz);
            }
        };
        walk(GC<0>{}, 0, n0);
        walk(GC<1>{}, n0, n0 + n1);
        return;
    }
    // full scan (skin list overflowed or skin off): images with |f + n| <= rc |b_d|
    const float *T = S.tr_lat + 24 * A.s;
    for (int j = 0; j < A.N; ++j) {
        const int js = A.st + j;
        const int ej = S.elem[js];
        float dx0, dy0, dz0;
        rel_pos(S, A, js, dx0, dy0, dz0);
        int lo[3], hi[3];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const float f = T[9 + 3 * d] * dx0 + T[9 + 3 * d + 1] * dy0 + T[9 + 3 * d + 2] * dz0;
            ok &= image_range(f, R.rc_b * T[21 + d] + 1e-4f, lo[d], hi[d]);
        }
        if (!ok) continue;
        for (int n1 = lo[0]; n1 <= hi[0]; ++n1)
            for (int n2 = lo[1]; n2 <= hi[1]; ++n2)
                for (int n3 = lo[2]; n3 <= hi[2]; ++n3) {
                    if (j == A.i && n1 == 0 && n2 == 0 && n3 == 0) continue;
                    const float m1 = (float)n1, m2 = (float)n2, m3 = (float)n3;
                    const float dx = dx0 + fmaf(m1, A.L[0], fmaf(m2, A.L[3], m3 * A.L[6]));
                    const float dy = dy0 + fmaf(m1, A.L[1], fmaf(m2, A.L[4], m3 * A.L[7]));
                    const float dz = dz0 + fmaf(m1, A.L[2], fmaf(m2, A.L[5], m3 * A.L[8]));
                    const float r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 < R.rc2)) continue;
                    if (ej == 0) fn(GC<0>{}, js, dx, dy, dz, r2);
                    else if (ej == 1) fn(GC<1>{}, js, dx, dy, dz, r2);
                }
    }
}

// Skin list of one atom: every image of every atom of the trajectory within the skin
// cutoff, element 0 first.  Returns the packed count (n0 | n1 << 16), or -1 when the list
// does not fit (more than skcap entries, or an image outside the entry's range).
__device__ int build_skin(const RadialNN &R, const SmemR &S, const AtomR &A, unsigned *sk, int skcap) {
    const float *T = S.tr_lat + 24 * A.s;
    int tot = 0, n0 = 0;
    bool over = false;
    for (int g = 0; g < 2; ++g) {
        for (int j = 0; j < A.N; ++j) {
            const int js = A.st + j;
            if (S.elem[js] != g) continue;
            float dx0, dy0, dz0;
            rel_pos(S, A, js, dx0, dy0, dz0);
            int lo[3], hi[3];
            bool ok = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                const float f = T[9 + 3 * d] * dx0 + T[9 + 3 * d + 1] * dy0 + T[9 + 3 * d + 2] * dz0;
                ok &= image_range(f, T[18 + d], lo[d], hi[d]);
            }
            if (!ok) {
                over = true;
                continue;
            }
            for (int n1 = lo[0]; n1 <= hi[0]; ++n1)
                for (int n2 = lo[1]; n2 <= hi[1]; ++n2)
                    for (int n3 = lo[2]; n3 <= hi[2]; ++n3) {
                        if (j == A.i && n1 == 0 && n2 == 0 && n3 == 0) continue;
                        const float m1 = (float)n1, m2 = (float)n2, m3 = (float)n3;
                        const float dx = dx0 + fmaf(m1, A.L[0], fmaf(m2, A.L[3], m3 * A.L[6]));
                        const float dy = dy0 + fmaf(m1, A.L[1], fmaf(m2, A.L[4], m3 * A.L[7]));
                        const float dz = dz0 + fmaf(m1, A.L[2], fmaf(m2, A.L[5], m3 * A.L[8]));
                        if (dx * dx + dy * dy + dz * dz > R.cut2s) continue;
                        if (tot < skcap && image_fits(n1) && image_fits(n2) && image_fits(n3))
                            sk[(size_t)tot * A.N + A.i] = pack_entry(j, n1, n2, n3);
                        else
                            over = true;
                        ++tot;
                        if (g == 0) ++n0;
                    }
        }
    }
    return over ? -1 : (n0 | ((tot - n0) << 16));
}

// Activations ('p' softplus, 't' tanh, 's' sigmoid, 'l' linear): the value, and the
// derivative from the value as getdnodes_values.f90 forms it ((e^v - 1)/e^v = 1 - e^-v for
// softplus, 1 - v^2, v (1 - v), 1), so a layer's derivatives need no stored pre-activations.
template <char A> __device__ __forceinline__ float act_v(float z) {
    if (A == 'p') {
        const float e = ex2a(-fabsf(z) * kLog2eF);
        return fmaf(lg2a(1.f + e), kLn2F, fmaxf(z, 0.f));
    } else if (A == 't') {
        return tanhf(z);
    } else if (A == 's') {
        return rcpa(1.f + ex2a(-z * kLog2eF));
    }
    return z;
}
template <char A> __device__ __forceinline__ float act_dv(float v) {
    if (A == 'p') return 1.f - ex2a(-v * kLog2eF);
    if (A == 't') return fmaf(-v, v, 1.f);
    if (A == 's') return v * (1.f - v);
    return 1.f;
}
__device__ __forceinline__ void act_d(uint8_t a, float z, float &v, float &dv) {
    if (a == 'p') {
        softplus_d(z, v, dv);
    } else if (a == 't') {
        v = act_v<'t'>(z);
        dv = act_dv<'t'>(v);
    } else if (a == 's') {
        v = act_v<'s'>(z);
        dv = act_dv<'s'>(v);
    } else {
        v = z;
        dv = 1.f;
    }
}
// z[n] <- act(z[n] rn) for a whole layer (kind uniform per layer)
template <char A> __device__ __forceinline__ void act_layer_k(float (&z)[kRW], float rn) {
#pragma unroll
    for (int n = 0; n < kRW; ++n) z[n] = act_v<A>(z[n] * rn);
}
__device__ __forceinline__ void act_layer(uint8_t a, float (&z)[kRW], float rn) {
    if (a == 'p') act_layer_k<'p'>(z, rn);
    else if (a == 't') act_layer_k<'t'>(z, rn);
    else if (a == 's') act_layer_k<'s'>(z, rn);
    else act_layer_k<'l'>(z, rn);
}
// d[n] <- act'(v[n]) c[n] from the layer's values
template <char A> __device__ __forceinline__ void act_dv_layer_k(const float (&v)[kRW], float (&d)[kRW]) {
#pragma unroll
    for (int n = 0; n < kRW; ++n) d[n] *= act_dv<A>(v[n]);
}
__device__ __forceinline__ void act_dv_layer(uint8_t a, const float (&v)[kRW], float (&d)[kRW]) {
    if (a == 'p') act_dv_layer_k<'p'>(v, d);
    else if (a == 't') act_dv_layer_k<'t'>(v, d);
    else if (a == 's') act_dv_layer_k<'s'>(v, d);
}

// z[0..32) += x[p] W[p][0..32) over p < np, x from the per-thread buffer (stride bs),
// W rows of 32 floats broadcast from shared memory
template <int NP>
__device__ __forceinline__ void rowmv(float (&z)[kRW], const float *W, const float *x) {
#pragma unroll 2
    for (int p = 0; p < NP; ++p) {
        const float xv = x[p * kRS];
        const float4 *row = reinterpret_cast<const float4 *>(W + p * kRW);
#pragma unroll
        for (int n4 = 0; n4 < kRW / 4; ++n4) {
            const float4 w = row[n4];
            z[4 * n4] = fmaf(w.x, xv, z[4 * n4]);
            z[4 * n4 + 1] = fmaf(w.y, xv, z[4 * n4 + 1]);
            z[4 * n4 + 2] = fmaf(w.z, xv, z[4 * n4 + 2]);
            z[4 * n4 + 3] = fmaf(w.w, xv, z[4 * n4 + 3]);
        }
    }
}
__device__ __forceinline__ void load_row(float (&z)[kRW], const float *b) {
    const float4 *b4 = reinterpret_cast<const float4 *>(b);
#pragma unroll
    for (int n4 = 0; n4 < kRW / 4; ++n4) {
        const float4 v = b4[n4];
        z[4 * n4] = v.x;
        z[4 * n4 + 1] = v.y;
        z[4 * n4 + 2] = v.z;
        z[4 * n4 + 3] = v.w;
    }
}

// ---- network of one atom (lane = atom) ---------------------------------------------------
// Inputs x[q] = scaled descriptors in the per-thread buffer; returns the atomic energy
// (output node, Ha) and leaves dE/dG (raw descriptors, padded grouped order) in the
// buffer when do_forces.  Weight block of an element (floats, rows of 32):
//   W1 [nin][32], b1 [32], then NH = 2: W2 [32][32], b2 [32], W2T [32][32], w3 [32], b3
//                               NH = 1: w2 [32], b2
// Padded hidden nodes have zero weights in and out, so they change nothing.
template <int NIN, int NH>
__device__ __forceinline__ float nnr_network(const RadialNN &R, const SmemR &S, int ei, int tid, bool do_forces) {
    constexpr int nin = NIN, bs = kRS;
    const float *wb = S.w + (ei == 0 ? 0 : nnr_wofs1(NIN, NH));
    float *hb = S.hb + tid;
    const float rn1 = R.rn[0];
    float z[kRW];
    load_row(z, wb + nin * kRW);
    rowmv<nin>(z, wb, hb);
    act_layer(R.act[0], z, rn1);  // z = layer-1 values
    float d1[kRW];                // becomes dE/d(layer-1 sum) times rn1
    float out;
    if (NH == 2) {
#pragma unroll
        for (int n = 0; n < kRW; ++n) hb[n * bs] = z[n];
        const float *w2 = wb + (nin + 1) * kRW;
        const float *w3 = w2 + 2 * kRW * kRW + kRW;
        load_row(z, w2 + kRW * kRW);
        rowmv<kRW>(z, w2, hb);
        const float rn2 = R.rn[1];
        const uint8_t a2 = R.act[1];
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int n = 0; n < kRW; ++n) {
            float v, dv;
            act_d(a2, z[n] * rn2, v, dv);
            const float w = w3[n];
            o[n & 3] = fmaf(w, v, o[n & 3]);
            z[n] = w * dv;  // d(output sum)/d(layer-2 sum), before rn2
        }
        float vo, dvo;
        act_d(R.act[2], ((o[0] + o[1]) + (o[2] + o[3]) + w3[kRW]) * R.rn[2], vo, dvo);
        out = vo;
        if (!do_forces) return out;
        // delta2 = dE/d(layer-2 sum) rn2 beside the layer-1 values in the buffer
        const float g2 = R.rn[2] * dvo * rn2;
        float *hd = hb + kRW * bs;
#pragma unroll
        for (int n = 0; n < kRW; ++n) hd[n * bs] = z[n] * g2;
#pragma unroll
        for (int p = 0; p < kRW; ++p) d1[p] = 0.f;
        rowmv<kRW>(d1, w2 + kRW * kRW + kRW, hd);  // sum_n W2[p][n] delta2[n]
        const uint8_t a1 = R.act[0];
#pragma unroll
        for (int p = 0; p < kRW; ++p) {
            z[p] = hb[p * bs];
            d1[p] *= rn1;
        }
        act_dv_layer(a1, z, d1);
    } else {
        const float *w2 = wb + (nin + 1) * kRW;
        float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int n = 0; n < kRW; ++n) o[n & 3] = fmaf(w2[n], z[n], o[n & 3]);
        float vo, dvo;
        act_d(R.act[1], ((o[0] + o[1]) + (o[2] + o[3]) + w2[kRW]) * R.rn[1], vo, dvo);
        out = vo;
        if (!do_forces) return out;
        const float g1 = R.rn[1] * dvo * rn1;
#pragma unroll
        for (int p = 0; p < kRW; ++p) d1[p] = w2[p] * g1;
        act_dv_layer(R.act[0], z, d1);
    }
    // dE/dG_q = dscal_q sum_p W1[q][p] d1[p]
    const float *ds = S.dscal + ei * nin;
#pragma unroll 2
    for (int q = 0; q < nin; ++q) {
        const float4 *row = reinterpret_cast<const float4 *>(wb + q * kRW);
        float a[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int p4 = 0; p4 < kRW / 4; ++p4) {
            const float4 w = row[p4];
            a[p4 & 3] = fmaf(w.x, d1[4 * p4], a[p4 & 3]);
            a[p4 & 3] = fmaf(w.y, d1[4 * p4 + 1], a[p4 & 3]);
            a[p4 & 3] = fmaf(w.z, d1[4 * p4 + 2], a[p4 & 3]);
            a[p4 & 3] = fmaf(w.w, d1[4 * p4 + 3], a[p4 & 3]);
        }
        hb[q * bs] = ((a[0] + a[1]) + (a[2] + a[3])) * ds[q];
    }
    return out;
}

// ---- one force evaluation of the atom: descriptors, (network,) forces --------------------
// BLA / BLB: block length of the shifted-Gaussian recurrence of group 0 / 1 (0: one 2^x
// per function).  Descriptors: the scaled symmetry functions in the padded grouped order,
// the trajectory's out-of-range flag, the neighbour-list overflow and the nearest
// neighbour entry (rmin2) with its atom (near: the first entry of the walk at that
// distance).
template <int KA, int KB, int BLA, int BLB, int UNR>
__device__ __forceinline__ void nnr_descr(const RadialNN &R, const NNScratch &X, const SmemR &S, const AtomR &A,
                                          const unsigned *sk, int cnt, int *flag, float &rmin2, int &near,
                                          float (&xs)[KA + KB]) {
    constexpr int KT = KA + KB;
    float G[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) G[k] = 0.f;
    int nn = 0;
    for_neighbours<false, UNR>(R, S, A, sk, cnt, [&](auto gc, int js, float dx, float dy, float dz, float r2) {
        constexpr int g = decltype(gc)::value;
        constexpr int K = g == 0 ? KA : KB, off = g == 0 ? 0 : KA, BL = g == 0 ? BLA : BLB;
        const bool inside = r2 < R.rc2;
        nn += inside ? 1 : 0;
        near = r2 < rmin2 ? js : near;
        rmin2 = fminf(rmin2, r2);
        const float r = r2 * rsqrtf(r2);
        const float fc = inside ? fc_of_s(r2 * R.inv_rc2) : 0.f;
        if constexpr (BL > 0) {
            // e_(k+1) = e_k q_k, q_(k+1) = q_k gamma; a fresh 2^x at every block start
#pragma unroll
            for (int b = 0; b < K; b += BL) {
                const float u = r - R.rs[g][b];
                float e = ex2a(u * R.c[g][b] * u);
                float q = ex2a(fmaf(R.gq[g], u, R.gc[g]));
#pragma unroll
                for (int m = 0; m < BL && b + m < K; ++m) {
                    G[off + b + m] = fmaf(e, fc, G[off + b + m]);
                    if (m + 1 < BL && b + m + 1 < K) {
                        e *= q;
                        q *= R.gam[g];
                    }
                }
            }
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float u = r - R.rs[g][k];
                const float t = u * R.c[g][k];
                G[off + k] = fmaf(ex2a(t * u), fc, G[off + k]);
            }
        }
    });
    if (nn > R.maxnb) X.nnstatus[S.tr_t[A.s]] = 1;
    // scaling and range test (padded grouped order)
    {
        const float4 *sc = S.scal + A.ei * KT;
        bool out = false;
#pragma unroll
        for (int q = 0; q < KT; ++q) {
            const float4 c = sc[q];
            out |= G[q] < c.z || G[q] > c.w;
            xs[q] = fmaf(c.x, G[q], c.y);
        }
        if (out) flag[A.s] = 1;
    }
}

// Forces of the atom from dE/dG (raw descriptors, padded grouped order) in reverse mode: the
// centre's share returned in fix/fiy/fiz, the neighbours' by red.shared.
template <int KA, int KB, int BLA, int BLB, int UNR>
__device__ __forceinline__ void nnr_forces(const RadialNN &R, const SmemR &S, const AtomR &A, const unsigned *sk,
                                           int cnt, const float (&dG)[KA + KB], float &fix, float &fiy,
                                           float &fiz) {
    constexpr int bs = kRS;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for_neighbours<true, UNR>(R, S, A, sk, cnt, [&](auto gc, int js, float dx, float dy, float dz, float r2) {
        constexpr int g = decltype(gc)::value;
        constexpr int K = g == 0 ? KA : KB, off = g == 0 ? 0 : KA, BL = g == 0 ? BLA : BLB;
        const float ri = rsqrtf(r2);
        const float r = r2 * ri;
        float fc, dfds;
        fc_of_s_d(fminf(r2 * R.inv_rc2, 1.f), fc, dfds);
        if (!(r2 < R.rc2)) {
            fc = 0.f;
            dfds = 0.f;
        }
        float s0 = 0.f, s1 = 0.f, dEdr;
        if constexpr (BL > 0) {
            // s1 = sum_k w_k u_k, u_k = u_b - (k - b) delta within a block; dE/dr needs c s1
#pragma unroll
            for (int b = 0; b < K; b += BL) {
                const float u = r - R.rs[g][b];
                float e = ex2a(u * R.c[g][b] * u);
                float q = ex2a(fmaf(R.gq[g], u, R.gc[g]));
                float sb = 0.f, sm = 0.f;
#pragma unroll
                for (int m = 0; m < BL && b + m < K; ++m) {
                    const float w = dG[off + b + m] * e;
                    sb += w;
                    sm = fmaf(w, (float)m, sm);
                    if (m + 1 < BL && b + m + 1 < K) {
                        e *= q;
                        q *= R.gam[g];
                    }
                }
                s0 += sb;
                s1 = fmaf(u, sb, s1);
                s1 = fmaf(-R.dl[g], sm, s1);
            }
            dEdr = fmaf(fc * (2.f * kLn2F) * R.c[g][0], s1, (2.f * R.inv_rc2) * r * dfds * s0);
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const float u = r - R.rs[g][k];
                const float t = u * R.c[g][k];
                const float w = dG[off + k] * ex2a(t * u);
                s0 += w;
                s1 = fmaf(w, t, s1);
            }
            // dE/dr = fc sum_k dG_k de_k/dr + dfc/dr sum_k dG_k e_k, de_k/dr = 2 ln2 t_k e_k
            dEdr = fmaf(fc * (2.f * kLn2F), s1, (2.f * R.inv_rc2) * r * dfds * s0);
        }
        const float f = dEdr * ri;
        fx = fmaf(f, dx, fx);
        fy = fmaf(f, dy, fy);
        fz = fmaf(f, dz, fz);
        red_shared(&S.f3[js], -f * dx);
        red_shared(&S.f3[bs + js], -f * dy);
        red_shared(&S.f3[2 * bs + js], -f * dz);
    });
    fix = fx;
    fiy = fy;
    fiz = fz;
}


// Scaling tables of both elements in the padded grouped order (both network variants)
template <int NIN>
__device__ void load_scaling_r(const RadialNN &R, const SmemR &S) {
    const int tid = threadIdx.x, bs = blockDim.x, nin = NIN;
    for (int e = 0; e < R.nelem; ++e)
        for (int q = tid; q < nin; q += bs) {
            const int s = R.qsrc[e][q];
            S.scal[e * nin + q] =
                s >= 0 ? R.fscal[e * R.maxsf + s] : make_float4(1.f, 0.f, -INFINITY, INFINITY);
            S.dscal[e * nin + q] = s >= 0 ? R.fdscal[e * R.maxsf + s] : 0.f;
        }
}

// Weight blocks and scaling tables in shared memory from the model's current FP32 weights
// (calconenn.f90 layout: layer l of element e is an n_(l-1) x n_l row-major matrix plus
// n_l biases at woff[e][l]); hidden layers padded to 32 nodes with zeros, inputs in the
// padded grouped order.
template <int NIN, int NH>
__device__ void load_weights_r(const RadialNN &R, const SmemR &S) {
    const int tid = threadIdx.x, bs = blockDim.x, nin = NIN;
    for (int e = 0; e < R.nelem; ++e) {
        const float *src = R.wf + (size_t)e * R.maxweights;
        float *dst = S.w + (e == 0 ? 0 : nnr_wofs1(NIN, NH));
        const int n1 = R.nodes[e][1];
        const float *l1 = src + R.woff[e][1];
        for (int k = tid; k < (nin + 1) * kRW; k += bs) {
            const int q = k / kRW, n = k % kRW;
            float v = 0.f;
            if (n < n1) {
                if (q < nin) {
                    const int s = R.qsrc[e][q];
                    if (s >= 0) v = l1[s * n1 + n];
                } else {
                    v = l1[R.nodes[e][0] * n1 + n];
                }
            }
            dst[k] = v;
        }
        const int o2 = (nin + 1) * kRW;
        const float *l2 = src + R.woff[e][2];
        if (NH == 2) {
            const int n2 = R.nodes[e][2];
            const float *l3 = src + R.woff[e][3];
            for (int k = tid; k < kRW * kRW; k += bs) {
                const int p = k / kRW, n = k % kRW;
                const float v = (p < n1 && n < n2) ? l2[p * n2 + n] : 0.f;
                dst[o2 + k] = v;                                  // W2 [p][n]
                dst[o2 + kRW * kRW + kRW + n * kRW + p] = v;      // W2T [n][p]
            }
            for (int n = tid; n < kRW; n += bs) {
                dst[o2 + kRW * kRW + n] = n < n2 ? l2[n1 * n2 + n] : 0.f;          // b2
                dst[o2 + 2 * kRW * kRW + kRW + n] = n < n2 ? l3[n] : 0.f;          // w3
            }
            if (tid < 4) dst[o2 + 2 * kRW * kRW + 2 * kRW + tid] = tid == 0 ? l3[n2] : 0.f;  // b3
        } else {
            for (int n = tid; n < kRW; n += bs) dst[o2 + n] = n < n1 ? l2[n] : 0.f;       // w2
            if (tid < 4) dst[o2 + kRW + tid] = tid == 0 ? l2[n1] : 0.f;                  // b2
        }
    }
    load_scaling_r<NIN>(R, S);
}

// ---- tensor-core network (BF16 operands, FP32 accumulation in TMEM) ----------------------
// The same network as nnr_network, organised as GEMMs over 128-atom tiles: thread k of the
// CTA is row k % 128 of tile k / 128 and the four warps of a tile reach TMEM lanes
// 32 (w % 4) .. +31, i.e. exactly their own rows.  Per tile and layer: every thread writes its
// operand row (bf16) to shared memory, the tile's threads meet at a named barrier, one thread
// issues the MMAs for both elements' weights (D_e = A B_e^T, M = 128, K-steps of 16) and
// commits them to the tile's mbarrier, every thread waits for it and reads its row of the
// accumulator of its own element from TMEM.  Activations, biases, the output node and the
// scaling stay FP32 in registers; the layer-1 values wait in TMEM (spill columns) for the
// backward pass.  Four GEMMs per force evaluation: x W1, v1 W2, delta2 W2^T, delta1 W1^T.
struct TcCtx {
    uint32_t tmem;  // TMEM base of the CTA
    uint64_t *bar;  // one mbarrier per tile
    int *err;       // set when a GEMM did not complete within the wait limit
};

// A GEMM round takes microseconds; a wait that runs out of polls marks the error word, and
// after that no thread waits again (the kernel finishes with wrong numbers instead of
// stalling, and the host reports the error).
constexpr uint32_t kTcMaxPolls = 1u << 18;

// One GEMM round of the tile group: D_e (TMEM columns d0, d1) = A (K x 128 rows at a_s) x B_e^T
// (N rows at b0_s / b1_s); all threads of the tile call it, returns with the result visible.
// SPLIT: A = A_hi + A_lo and B = B_hi + B_lo (each a BF16 operand; the low parts at a_lo
// bytes after the high A tile and b_lo bytes after the high B operands) and
// D = A_hi B_hi + A_lo B_hi + A_hi B_lo: three MMAs per K step, about 16 significant bits.
template <int KK, int NN, bool SPLIT>
__device__ __forceinline__ void tc_round(const TcCtx &C, int g, int nthr, uint32_t a_s, uint32_t b0_s, uint32_t b1_s,
                                         bool two, uint32_t d0, uint32_t d1, uint32_t &phase, uint32_t a_lo = 0,
                                         uint32_t b_lo = 0) {
    fence_async_smem();
    tc_fence_before();
    named_barrier(1 + g, nthr);
    if ((threadIdx.x & 127) == 0) {
        tc_fence_after();
        constexpr uint32_t idesc = tc_idesc_bf16(128, NN);
#pragma unroll
        for (int ks = 0; ks < KK / 16; ++ks) {
            const uint32_t ao = a_s + 256 * ks, bo0 = b0_s + 256 * ks, bo1 = b1_s + 256 * ks;
            const uint64_t ad = tc_desc(ao, 128, 16 * KK);
            tc_mma_bf16(C.tmem + d0, ad, tc_desc(bo0, 128, 16 * KK), idesc, ks > 0);
            if (two) tc_mma_bf16(C.tmem + d1, ad, tc_desc(bo1, 128, 16 * KK), idesc, ks > 0);
            if constexpr (SPLIT) {
                const uint64_t al = tc_desc(ao + a_lo, 128, 16 * KK);
                tc_mma_bf16(C.tmem + d0, al, tc_desc(bo0, 128, 16 * KK), idesc, true);
                tc_mma_bf16(C.tmem + d0, ad, tc_desc(bo0 + b_lo, 128, 16 * KK), idesc, true);
                if (two) {
                    tc_mma_bf16(C.tmem + d1, al, tc_desc(bo1, 128, 16 * KK), idesc, true);
                    tc_mma_bf16(C.tmem + d1, ad, tc_desc(bo1 + b_lo, 128, 16 * KK), idesc, true);
                }
            }
        }
        tc_commit(&C.bar[g]);
    }
    if (!*(volatile int *)C.err && !mbar_wait_bounded(&C.bar[g], phase, kTcMaxPolls)) atomicExch(C.err, 1);
    phase ^= 1u;
    tc_fence_after();
}

// eight FP32 values as one 16-byte chunk of BF16 operand row; with SPLIT also the rounding
// residuals (x - bf16(x)) as the chunk of the low part, `lo` bytes further on
__device__ __forceinline__ float bf16_value(float x) { return __uint_as_float(pack_bf16x2(x, 0.f) << 16); }
template <bool SPLIT>
__device__ __forceinline__ void st_row8(unsigned char *chunk, size_t lo, const float *v) {
    st_bf16x8(chunk, v);
    if constexpr (SPLIT) {
        float r[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = v[j] - bf16_value(v[j]);
        st_bf16x8(chunk + lo, r);
    }
}

// 16 accumulator columns of the thread's row, from element 1's block when e1
__device__ __forceinline__ void tc_ld_row(uint32_t t0, uint32_t t1, bool two, bool e1, float (&v)[16]) {
    tmem_ld16(t0, v);
    if (two) {
        float w[16];
        tmem_ld16(t1, w);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = e1 ? w[j] : v[j];
    } else {
        tmem_wait_ld();
    }
}

template <int N> __device__ __forceinline__ void act_vals(uint8_t a, float (&z)[N]) {
    if (a == 'p') {
#pragma unroll
        for (int n = 0; n < N; ++n) z[n] = act_v<'p'>(z[n]);
    } else if (a == 't') {
#pragma unroll
        for (int n = 0; n < N; ++n) z[n] = act_v<'t'>(z[n]);
    } else if (a == 's') {
#pragma unroll
        for (int n = 0; n < N; ++n) z[n] = act_v<'s'>(z[n]);
    }
}
template <int N> __device__ __forceinline__ void act_dvals(uint8_t a, const float (&v)[N], float (&d)[N]) {
    if (a == 'p') {
#pragma unroll
        for (int n = 0; n < N; ++n) d[n] *= act_dv<'p'>(v[n]);
    } else if (a == 't') {
#pragma unroll
        for (int n = 0; n < N; ++n) d[n] *= act_dv<'t'>(v[n]);
    } else if (a == 's') {
#pragma unroll
        for (int n = 0; n < N; ++n) d[n] *= act_dv<'s'>(v[n]);
    }
}

// B operands and FP32 vectors of both elements from the model's FP32 weights (calconenn.f90
// layout, as load_weights_r reads it).  B1[n][q] = W1[q][n] (32 x KP), B2[n][p] = W2[p][n],
// B3[p][n] = W2[p][n] (32 x 32), B4[q][p] = W1[q][p] (KP x 32); vectors: b1, then b2, w3, b3
// (two hidden layers) or w2, b2 (one).
template <int NIN, int NH, bool SPLIT>
__device__ void load_weights_tc(const RadialNN &R, const SmemR &S) {
    constexpr int KP = nnr_kp(NIN), BEL = nnr_tc_bel(NIN);
    constexpr int oB2 = 32 * KP * 2, oB3 = oB2 + 2048, oB4 = oB3 + 2048;
    const int tid = threadIdx.x, bs = blockDim.x;
    for (int e = 0; e < R.nelem; ++e) {
        const float *src = R.wf + (size_t)e * R.maxweights;
        const int n1 = R.nodes[e][1], n2 = NH == 2 ? R.nodes[e][2] : 0;
        const float *l1 = src + R.woff[e][1];
        const float *l2 = src + R.woff[e][2];
        auto w1 = [&](int q, int n) -> float {  // W1[q][n] in the padded grouped order
            if (q >= NIN || n >= n1) return 0.f;
            const int sidx = R.qsrc[e][q];
            return sidx >= 0 ? l1[sidx * n1 + n] : 0.f;
        };
        auto w2 = [&](int p, int n) -> float { return (NH == 2 && p < n1 && n < n2) ? l2[p * n2 + n] : 0.f; };
        unsigned char *wb = S.wb + (size_t)e * BEL;
        const size_t lo = 2 * (size_t)BEL;  // low parts of the split operands
        // one 8-wide chunk per item: rows x (K / 8) chunks per matrix
        for (int it = tid; it < 32 * (KP / 8); it += bs) {  // B1: row n, chunk k0 over q
            const int n = it / (KP / 8), k0 = 8 * (it % (KP / 8));
            float v[8];
            for (int j = 0; j < 8; ++j) v[j] = w1(k0 + j, n);
            st_row8<SPLIT>(wb + tc_offset(n, k0, KP), lo, v);
        }
        for (int it = tid; it < 32 * 4; it += bs) {  // B2, B3
            const int n = it / 4, k0 = 8 * (it % 4);
            float v[8], u[8];
            for (int j = 0; j < 8; ++j) {
                v[j] = w2(k0 + j, n);  // B2[n][p] = W2[p][n]
                u[j] = w2(n, k0 + j);  // B3[p][n] = W2[p][n], row p = n here
            }
            st_row8<SPLIT>(wb + oB2 + tc_offset(n, k0, 32), lo, v);
            st_row8<SPLIT>(wb + oB3 + tc_offset(n, k0, 32), lo, u);
        }
        for (int it = tid; it < KP * 4; it += bs) {  // B4: row q, chunk over p
            const int q = it / 4, k0 = 8 * (it % 4);
            float v[8];
            for (int j = 0; j < 8; ++j) v[j] = w1(q, k0 + j);
            st_row8<SPLIT>(wb + oB4 + tc_offset(q, k0, 32), lo, v);
        }
        float *vec = S.wv + e * kTcVec;
        for (int n = tid; n < 32; n += bs) {
            vec[n] = n < n1 ? l1[R.nodes[e][0] * n1 + n] : 0.f;                      // b1
            if (NH == 2) {
                const float *l3 = src + R.woff[e][3];
                vec[32 + n] = n < n2 ? l2[n1 * n2 + n] : 0.f;                          // b2
                vec[64 + n] = n < n2 ? l3[n] : 0.f;                                    // w3
                if (n == 0) vec[96] = l3[n2];                                          // b3
            } else {
                vec[32 + n] = n < n1 ? l2[n] : 0.f;                                    // w2
                if (n == 0) vec[64] = l2[n1];                                          // b2
            }
        }
    }
    load_scaling_r<NIN>(R, S);
}

// The network of this thread's atom on the tensor cores.  Every thread of the CTA calls it
// (rows without an atom carry zeros).  Returns the atomic energy (output node, Ha); with
// do_forces, dG receives dE/dG for the raw descriptors (padded grouped order).
template <int NIN, int NH, bool SPLIT>
__device__ __forceinline__ float nnr_network_tc(const RadialNN &R, const SmemR &S, const TcCtx &C, int ei,
                                                const float (&xs)[NIN], bool do_forces, float (&dG)[NIN],
                                                uint32_t &phase) {
    constexpr int KP = nnr_kp(NIN), TW = nnr_tw(NIN), CPT = nnr_tc_cpt(NIN), BEL = nnr_tc_bel(NIN);
    constexpr int oB2 = 32 * KP * 2, oB3 = oB2 + 2048, oB4 = oB3 + 2048;
    const int tid = threadIdx.x, g = tid >> 7, row = tid & 127;
    const int nthr = min(128, (int)blockDim.x - 128 * g);
    unsigned char *at = S.at + (size_t)g * 128 * TW * 2;
    const uint32_t a_s = smem_u32(at), b_s = smem_u32(S.wb);
    constexpr size_t ALO = (size_t)kTcTiles * 128 * TW * 2;  // low A parts after all high tiles
    constexpr uint32_t BLO = 2 * BEL;                          // low B parts after both elements
    const uint32_t lane = ((uint32_t)((tid >> 5) & 3) * 32u) << 16;
    const uint32_t c0 = (uint32_t)(g * CPT), c1 = c0 + TW, cs = c0 + 2 * TW;
    const bool two = R.nelem > 1, e1 = ei == 1;
    const float *vec = S.wv + ei * kTcVec;
    const float rn1 = R.rn[0];
    const uint8_t a1 = R.act[0];
    // ---- layer 1: x W1 -------------------------------------------------------------------
#pragma unroll
    for (int k0 = 0; k0 < KP; k0 += 8) {
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (k0 + j < NIN) ? xs[k0 + j] : 0.f;
        st_row8<SPLIT>(at + tc_offset(row, k0, KP), ALO, v);
    }
    tc_round<KP, 32, SPLIT>(C, g, nthr, a_s, b_s, b_s + BEL, two, c0, c1, phase, ALO, BLO);
    float o = 0.f;  // output-node sum (one hidden layer)
#pragma unroll
    for (int h = 0; h < 32; h += 16) {
        float z[16];
        tc_ld_row(C.tmem + lane + c0 + h, C.tmem + lane + c1 + h, two, e1, z);
#pragma unroll
        for (int j = 0; j < 16; ++j) z[j] = (z[j] + vec[h + j]) * rn1;
        act_vals<16>(a1, z);
        tmem_st16(C.tmem + lane + cs + h, z);  // layer-1 values for the backward pass
        if (NH == 2) {
            st_row8<SPLIT>(at + tc_offset(row, h, 32), ALO, z);
            st_row8<SPLIT>(at + tc_offset(row, h + 8, 32), ALO, z + 8);
        } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) o = fmaf(vec[32 + h + j], z[j], o);
        }
    }
    tmem_wait_st();
    float out, g1;
    if (NH == 2) {
        // ---- layer 2: v1 W2; output node -------------------------------------------------
        tc_round<32, 32, SPLIT>(C, g, nthr, a_s, b_s + oB2, b_s + BEL + oB2, two, c0, c1, phase, ALO, BLO);
        const float rn2 = R.rn[1];
        const uint8_t a2 = R.act[1];
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
            float z[16];
            tc_ld_row(C.tmem + lane + c0 + h, C.tmem + lane + c1 + h, two, e1, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float v, dv;
                act_d(a2, (z[j] + vec[32 + h + j]) * rn2, v, dv);
                o = fmaf(vec[64 + h + j], v, o);
            }
        }
        float vo, dvo;
        act_d(R.act[2], (o + vec[96]) * R.rn[2], vo, dvo);
        out = vo;
        if (!do_forces) return out;
        // delta2 = w3 f'(layer-2 sum) g2, from the accumulator still in TMEM
        const float g2 = R.rn[2] * dvo * rn2;
#pragma unroll
        for (int h = 0; h < 32; h += 16) {
            float z[16];
            tc_ld_row(C.tmem + lane + c0 + h, C.tmem + lane + c1 + h, two, e1, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float v, dv;
                act_d(a2, (z[j] + vec[32 + h + j]) * rn2, v, dv);
                z[j] = vec[64 + h + j] * dv * g2;
            }
            st_row8<SPLIT>(at + tc_offset(row, h, 32), ALO, z);
            st_row8<SPLIT>(at + tc_offset(row, h + 8, 32), ALO, z + 8);
        }
        // ---- delta1 = (delta2 W2^T) rn1 f'(v1) -------------------------------------------
        tc_round<32, 32, SPLIT>(C, g, nthr, a_s, b_s + oB3, b_s + BEL + oB3, two, c0, c1, phase, ALO, BLO);
        g1 = rn1;
    } else {
        float vo, dvo;
        act_d(R.act[1], (o + vec[64]) * R.rn[1], vo, dvo);
        out = vo;
        if (!do_forces) return out;
        g1 = R.rn[1] * dvo * rn1;
    }
#pragma unroll
    for (int h = 0; h < 32; h += 16) {
        float d[16], v1[16];
        if (NH == 2) {
            tc_ld_row(C.tmem + lane + c0 + h, C.tmem + lane + c1 + h, two, e1, d);
        } else {
#pragma unroll
            for (int j = 0; j < 16; ++j) d[j] = vec[32 + h + j];
        }
        tmem_ld16(C.tmem + lane + cs + h, v1);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 16; ++j) d[j] *= g1;
        act_dvals<16>(a1, v1, d);
        st_row8<SPLIT>(at + tc_offset(row, h, 32), ALO, d);
        st_row8<SPLIT>(at + tc_offset(row, h + 8, 32), ALO, d + 8);
    }
    // ---- dE/dG_q = dscal_q (delta1 W1^T)_q ---------------------------------------------
    tc_round<32, KP, SPLIT>(C, g, nthr, a_s, b_s + oB4, b_s + BEL + oB4, two, c0, c1, phase, ALO, BLO);
    const float *ds = S.dscal + ei * NIN;
#pragma unroll
    for (int q0 = 0; q0 < KP; q0 += 16) {
        float z[16];
        tc_ld_row(C.tmem + lane + c0 + q0, C.tmem + lane + c1 + q0, two, e1, z);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (q0 + j < NIN) dG[q0 + j] = z[j] * ds[q0 + j];
    }
    return out;
}

// Propagators of the fused step for single-bead atoms.  The constant-friction Langevin
// coefficients (langevin_coef of md_algo.f90:165-198 / 253-285: exp, sqrt and divisions in
// FP64, the slowest pipe of the GPU) depend only on the atom, so they are formed once per
// pack by the same FP64 expressions as langevin_1 / langevin_2 and the per-step updates
// apply them exactly as those functions do.
enum { kLcC0, kLcC1, kLcC2S, kLcC1mC2, kLcSr, kLcSvr, kLcC2, kLcSv2, kLcN };

__device__ __forceinline__ void lc_setup(const Batch &B, const PropParams &P, const TrajView &T, int i, double *lc,
                                         int stride) {
    const int ty = B.type[T.aoff + i];
    const double temp = kBoltz * T.nb * temp_of(B, P, ty) / B.mass[T.aoff + i];
    const bool all_big = all_xidt_big(B, P, T, i, kPropLangevinConst);
    LangCoef a, b;
    langevin_coef(P.gamma_const, P.step, temp, all_big, false, a);
    langevin_coef(P.gamma_const, P.step, temp, all_big, true, b);
    lc[kLcC0 * stride] = a.c0;
    lc[kLcC1 * stride] = a.c1;
    lc[kLcC2S * stride] = a.c2 * P.step;
    lc[kLcC1mC2 * stride] = a.c1 - a.c2;
    lc[kLcSr * stride] = a.sigma_r;
    lc[kLcSvr * stride] = a.sigma_v * a.c_rv;
    lc[kLcC2 * stride] = b.c2;
    lc[kLcSv2 * stride] = b.sigma_v * sqrt(1 - b.c_rv * b.c_rv);
}

// langevin_1 (md_algo.f90:146-232) for one single-bead atom with its coefficients
__device__ __forceinline__ void lc_half1(const Batch &B, const PropParams &P, const TrajView &T, int i, int step,
                                         const double *lc, int stride) {
    const int64_t k = T.base + i;
    const uint8_t fx = B.fixed[k];
    const double c0 = lc[kLcC0 * stride], c1 = lc[kLcC1 * stride], c2s = lc[kLcC2S * stride],
                 c1mc2 = lc[kLcC1mC2 * stride], sr = lc[kLcSr * stride], svr = lc[kLcSvr * stride];
    for (int d = 0; d < 3; ++d) {
        double &v = comp(B.vx, B.vy, B.vz, d, k);
        if (!(fx >> d & 1)) {
            const double rnd = rand_normal(P, T, step, 0, i, d, kStreamLangevin, P.randy);
            const double a = comp(B.ax, B.ay, B.az, d, k);
            comp(B.rx, B.ry, B.rz, d, k) += c1 * v + c2s * a + sr * rnd;
            v = c0 * v + c1mc2 * a + svr * rnd;
        } else {
            v = 0.0;
        }
    }
}

// langevin_2 (md_algo.f90:236-300) for one single-bead atom with its coefficients
__device__ __forceinline__ void lc_half2(const Batch &B, const PropParams &P, const TrajView &T, int i, int step,
                                         const double *lc, int stride) {
    const int64_t k = T.base + i;
    const uint8_t fx = B.fixed[k];
    const double c2 = lc[kLcC2 * stride], sv = lc[kLcSv2 * stride];
    for (int d = 0; d < 3; ++d) {
        double &v = comp(B.vx, B.vy, B.vz, d, k);
        if (!(fx >> d & 1)) {
            const double rnd = rand_normal(P, T, step, 0, i, d, kStreamLangevin, P.randy);
            v = v + c2 * comp(B.ax, B.ay, B.az, d, k) + sv * rnd;
        } else {
            v = 0.0;
        }
    }
}

// mode 0: forces, 1: energies only, 2: nsteps fused MD steps (propagate_1, forces,
// propagate_2, exit test), as the other network kernels.
template <int KA, int KB, int NH, int BLA, int BLB, int TC>
__global__ void __launch_bounds__(kRBlockMax, 1)
    nnr_kernel(Batch B, RadialNN R, EmtConst E, NNScratch X, PropParams P, const int2 *packs, const int *ptraj, int npack,
               int *counter, int nsteps, int mode) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int KT = KA + KB, bs = kRS;
    const int tid = threadIdx.x;
    const SmemR S = carve_r<KT, NH, TC>(smem_raw);
    SmemEmt<double> SE = carve_smem<double>(S.emt, B.max_atoms, B.max_beads);
    SE.red = S.red;
    SE.cjk = S.red;  // single-bead trajectories only: the ring-polymer table is never read
    TcCtx C{0u, S.tcbar, X.tcerr};
    uint32_t phase = 0;  // parity of this thread's tile mbarrier
    if constexpr (TC) {
        load_weights_tc<KT, NH, TC == 2>(R, S);
        if (tid < 32) {
            tmem_alloc(S.tslot, kTcCols);
            tmem_relinquish();
        }
        if (tid == 0) {
            for (int g = 0; g < kTcTiles; ++g) mbar_init(&S.tcbar[g], 1);
            fence_mbar_init();
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        C.tmem = *S.tslot;
    } else {
        load_weights_r<KT, NH>(R, S);
    }
    __syncthreads();
    const bool do_forces = mode != 1;
    for (;;) {
        __syncthreads();
        if (tid == 0) S.misc[0] = atomicAdd(counter, 1);
        __syncthreads();
        const int pk = S.misc[0];
        if (pk >= npack) break;
        const int2 pd = packs[pk];
        if (tid < pd.y) {
            const int t = ptraj[pd.x + tid];
            S.tr_t[tid] = t;
            S.tr_n[tid] = B.natoms[t];
            const int run = (mode != 2 || B.status[t] == kStatusRunning) ? 1 : 0;
            for (int b = 0; b < 2; ++b) {
                S.tr_over[b * kRMaxTraj + tid] = 0;
                S.tr_flag[b * kRMaxTraj + tid] = 0;
                S.tr_d2[b * kRMaxTraj + tid] = 0;
                S.tr_bad[b * kRMaxTraj + tid] = 0;
            }
            for (int b = 0; b < 3; ++b) S.tr_stat[b * kRMaxTraj + tid] = run;
            double lat[18];
            acsf_lattice(B.box + 9 * t, lat);
            float *T = S.tr_lat + 24 * tid;
            for (int k = 0; k < 18; ++k) T[k] = (float)lat[k];
            for (int d = 0; d < 3; ++d) {
                const double *I = lat + 9 + 3 * d;
                const double bn = sqrt(I[0] * I[0] + I[1] * I[1] + I[2] * I[2]);
                T[18 + d] = (float)(R.rcs * bn * (1.0 + 1e-4) + 1e-4);
                T[21 + d] = (float)(bn * (1.0 + 1e-4));
            }
        }
        __syncthreads();
        if (tid == 0) {
            int st = 0;
            for (int s = 0; s < pd.y; ++s) {
                S.tr_st[s] = st;
                st += S.tr_n[s];
            }
        }
        __syncthreads();
        AtomR A;
        A.s = -1;
        for (int s = 0; s < pd.y; ++s)
            if (tid >= S.tr_st[s] && tid < S.tr_st[s] + S.tr_n[s]) A.s = s;
        TrajView T{};
        if (A.s >= 0) {
            const int t = S.tr_t[A.s];
            T = traj_view(B, t);
            A.st = S.tr_st[A.s];
            A.N = T.N;
            A.i = tid - A.st;
            A.base = T.base;
            A.ei = R.elem_of_type[B.type[T.aoff + A.i]];
            S.elem[tid] = (int8_t)A.ei;
            const float *TL = S.tr_lat + 24 * A.s;
#pragma unroll
            for (int k = 0; k < 9; ++k) A.L[k] = TL[k];
            const int ty = B.type[T.aoff + A.i];
            A.algo = B.algo[ty];
            S.im[tid] = 1.0 / B.mass[T.aoff + A.i];
            if (mode == 2 && A.algo == kPropLangevinConst) {
                const double *src = X.lcoef + kLcN * (A.base + A.i);
#pragma unroll
                for (int q = 0; q < kLcN; ++q) S.lc[q * bs + tid] = src[q];
            }
        }
        const int steps0 = A.s >= 0 ? B.steps_done[T.t] : 0;
        __syncthreads();  // pack set-up read before any thread of the pack writes state
        // Two CTA barriers per MD step: (A) positions and this step's flags written, before
        // neighbours read them; (B) forces accumulated, before they are read.  The exit test
        // needs only the positions after the first half-step, so the projectile's thread
        // decides whether its trajectory runs the next step before (A).
        const int steps = mode == 2 ? nsteps : 1;
        int last = -1;  // last step run by the pack
        for (int step_i = 0; step_i < steps; ++step_i) {
            const int cur = step_i & 1, nxt = cur ^ 1;
            const int *stat = S.tr_stat + (step_i % 3) * kRMaxTraj;
            bool any = false;
            for (int s = 0; s < pd.y; ++s) any |= stat[s] != 0;
            if (!any) break;  // every trajectory of the pack has stopped (uniform: flags are stable)
            last = step_i;
            const bool active = A.s >= 0 && stat[A.s] != 0;
            const int step = steps0 + step_i + 1;
            int *flag = S.tr_flag + cur * kRMaxTraj;
            int *d2 = S.tr_d2 + cur * kRMaxTraj;
            int *over = S.tr_over + cur * kRMaxTraj;
            // ---- first half-step, positions, exit decision ------------------------------
            if (active) {
                if (mode == 2) {
                    if (A.algo == kPropVerlet) verlet_half(B, P, T, A.i, true);
                    else lc_half1(B, P, T, A.i, step, S.lc + tid, bs);
                }
                const int64_t k = A.base + A.i;
                const double rx = B.rx[k], ry = B.ry[k], rz = B.rz[k];
                const double x = rx * kAng2BohrD, y = ry * kAng2BohrD, z = rz * kAng2BohrD;
                A.xhi = (float)x;
                A.yhi = (float)y;
                A.zhi = (float)z;
                A.xli = (float)(x - (double)A.xhi);
                A.yli = (float)(y - (double)A.yhi);
                A.zli = (float)(z - (double)A.zhi);
                S.ph[tid] = make_float4(A.xhi, A.yhi, A.zhi, 0.f);
                S.pl[tid] = make_float4(A.xli, A.yli, A.zli, 0.f);
                if (mode == 2 && !isfinite((rx + ry) + (rz + B.vx[k]) + (B.vy[k] + B.vz[k])))
                    S.tr_bad[cur * kRMaxTraj + A.s] = 1;
                if (R.skin > 0.f) {
                    const double *r0 = X.skref + 3 * k;
                    const float ddx = (float)(rx - r0[0]), ddy = (float)(ry - r0[1]), ddz = (float)(rz - r0[2]);
                    atomicMax(&d2[A.s], __float_as_int(ddx * ddx + ddy * ddy + ddz * ddz));
                }
            }
            if (A.s >= 0 && A.i == 0) {
                // the exit test of md_tian2.f90:88-92 on the projectile (atom 0); positions do
                // not change in the second half-step
                int run_next = active ? 1 : 0;
                if (active && mode == 2) {
                    B.steps_done[T.t] = step;
                    // a bead-atom of the trajectory was not finite after the previous step's
                    // first half-step: this step is its last
                    if (S.tr_bad[nxt * kRMaxTraj + A.s]) {
                        B.status[T.t] = kStatusErrNonFinite;
                        run_next = 0;
                    } else if (P.use_exit && B.is_proj[B.type[T.aoff]]) {
                        const double z = B.rz[T.base];
                        if (z > P.pul) {
                            B.status[T.t] = kStatusExitUpper;
                            run_next = 0;
                        } else if (z < P.pll) {
                            B.status[T.t] = kStatusExitLower;
                            run_next = 0;
                        }
                    }
                    if (run_next && P.max_steps > 0 && step >= P.max_steps) {
                        B.status[T.t] = kStatusStepLimit;
                        run_next = 0;
                    }
                }
                S.tr_stat[((step_i + 1) % 3) * kRMaxTraj + A.s] = run_next;
            }
            S.f3[tid] = 0.f;
            S.f3[bs + tid] = 0.f;
            S.f3[2 * bs + tid] = 0.f;
            __syncthreads();  // (A)
            if (tid < pd.y) {
                S.tr_flag[nxt * kRMaxTraj + tid] = 0;
                S.tr_d2[nxt * kRMaxTraj + tid] = 0;
                S.tr_over[nxt * kRMaxTraj + tid] = 0;
                S.tr_bad[nxt * kRMaxTraj + tid] = 0;
            }
            // ---- forces; skin lists rebuilt when invalid or when some atom of the
            // trajectory moved more than half the skin (displacements in A, skin in bohr) ----
            const float half = 0.5f * R.skin * (float)kBohr2Ang;
            float fix = 0.f, fiy = 0.f, fiz = 0.f;
            float rmin2 = INFINITY;  // nearest neighbour entry (bohr^2): the closest approach of atom 0
            int near_js = -1;        // its atom (slot of the pack)
            const unsigned *sk = reinterpret_cast<const unsigned *>(X.skw) + A.base * X.skcap;
            int cnt = -1;
            float xs[KT], dG[KT];
#pragma unroll
            for (int q = 0; q < KT; ++q) xs[q] = 0.f;
            if (active) {
                const int64_t k = A.base + A.i;
                const int bead = B.bead_off[T.t];
                if (R.skin > 0.f && (X.skok[bead] == 0 || __int_as_float(d2[A.s]) > half * half)) {
                    const int c = build_skin(R, S, A, reinterpret_cast<unsigned *>(X.skw) + A.base * X.skcap, X.skcap);
                    X.skcnt[k] = c;
                    if (c < 0) over[A.s] = 1;
                    double *r0 = X.skref + 3 * k;
                    r0[0] = B.rx[k];
                    r0[1] = B.ry[k];
                    r0[2] = B.rz[k];
                }
                cnt = R.skin > 0.f ? X.skcnt[k] : -1;
                nnr_descr<KA, KB, BLA, BLB, TC ? 1 : 3>(R, X, S, A, sk, cnt, flag, rmin2, near_js, xs);
            }
            float e_at = 0.f;
            if constexpr (TC) {
                // every thread of the CTA: the GEMMs are per 128-row tile
                e_at = nnr_network_tc<KT, NH, TC == 2>(R, S, C, active ? A.ei : 0, xs, do_forces, dG, phase);
            } else if (active) {
#pragma unroll
                for (int q = 0; q < KT; ++q) S.hb[q * bs + tid] = xs[q];
                e_at = nnr_network<KT, NH>(R, S, A.ei, tid, do_forces);
#pragma unroll
                for (int q = 0; q < KT; ++q) dG[q] = S.hb[q * bs + tid];
            }
            if (active) {
                S.ea[tid] = (double)e_at + R.atom_energy[A.ei];
                if (do_forces) nnr_forces<KA, KB, BLA, BLB, TC ? 1 : 3>(R, S, A, sk, cnt, dG, fix, fiy, fiz);
            }
            __syncthreads();  // (B)
            // per-trajectory energy and skin-list state: one warp per trajectory, strided FP64
            // partial sums and a butterfly (fixed order)
            {
                const int warp = tid >> 5, lane = tid & 31, nw = blockDim.x >> 5;
                for (int s = warp; s < pd.y; s += nw) {
                    if (!stat[s]) continue;
                    const int t = S.tr_t[s];
                    double e = 0.0;
                    for (int k = lane; k < S.tr_n[s]; k += 32) e += S.ea[S.tr_st[s] + k];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
                    if (lane == 0) {
                        const int bead = B.bead_off[t];
                        if (R.skin > 0.f && (X.skok[bead] == 0 || __int_as_float(d2[s]) > half * half))
                            X.skok[bead] = over[s] ? 0 : 1;
                        B.epot[bead] = (R.surrogate && flag[s]) ? 0.0 : e * kHa2eVR;
                    }
                }
            }
            if (active) {
                const int64_t k = A.base + A.i;
                const bool fb = R.surrogate && flag[A.s];
                const double c = kHa2eVR * kAng2BohrD;
                double fx = 0.0, fy = 0.0, fz = 0.0;
                if (do_forces && !fb) {
                    fx = (double)(S.f3[tid] + fix) * c;
                    fy = (double)(S.f3[bs + tid] + fiy) * c;
                    fz = (double)(S.f3[2 * bs + tid] + fiz) * c;
                }
                B.fx[k] = fx;
                B.fy[k] = fy;
                B.fz[k] = fz;
                const double im = S.im[tid];
                const uint8_t fxd = B.fixed[k];
                B.ax[k] = (do_forces && !(fxd & 1)) ? fx * im : 0.0;
                B.ay[k] = (do_forces && !(fxd & 2)) ? fy * im : 0.0;
                B.az[k] = (do_forces && !(fxd & 4)) ? fz * im : 0.0;
            }
            // ---- EMT for the trajectories whose descriptors left the training range ----------
            if (R.surrogate) {
                bool anyfb = false;
                for (int s = 0; s < pd.y; ++s) anyfb |= stat[s] && flag[s];
                if (anyfb) {  // uniform over the CTA
                    __syncthreads();
                    for (int s = 0; s < pd.y; ++s) {
                        if (!stat[s] || !flag[s]) continue;
                        const int t = S.tr_t[s];
                        __syncthreads();
                        emt_bead<double>(B, E, SE, t, 0, do_forces);
                        if (tid == 0) X.fallback[t] += 1;
                        if (A.s == s && do_forces) {
                            const int64_t k = A.base + A.i;
                            const double m = B.mass[T.aoff + A.i];
                            const uint8_t fxd = B.fixed[k];
                            if (!(fxd & 1)) B.ax[k] = B.fx[k] / m;
                            if (!(fxd & 2)) B.ay[k] = B.fy[k] / m;
                            if (!(fxd & 4)) B.az[k] = B.fz[k] / m;
                        }
                        __syncthreads();
                    }
                }
            }
            // ---- second half-step ------------------------------------------------------------
            if (active && mode == 2) {
                if (A.algo == kPropVerlet) verlet_half(B, P, T, A.i, false);
                else lc_half2(B, P, T, A.i, step, S.lc + tid, bs);
                // trajectory observables by the projectile's thread; the closest approach is
                // the nearest entry of its skin list (every image within the cutoff + skin)
                if (A.i == 0) {
                    // the bounce partner: the atom of the nearest entry, found by the descriptor
                    // walk; its displacement is the minimum image of the unwrapped difference
                    // (the nearest atom lies far inside half a cell).  Should that image not
                    // reproduce the entry's distance (a cell too skewed for rounding fractional
                    // coordinates), the step has no partner and the bounce segment goes on.
                    int near = -1;
                    float nx = 0.f, ny = 0.f, nz = 0.f;
                    if (rmin2 < INFINITY && near_js >= 0) {
                        float dx, dy, dz;
                        rel_pos(S, A, near_js, dx, dy, dz);
                        const float *TL = S.tr_lat + 24 * A.s;
                        float f[3];
#pragma unroll
                        for (int d = 0; d < 3; ++d)
                            f[d] = rintf(TL[9 + 3 * d] * dx + TL[9 + 3 * d + 1] * dy + TL[9 + 3 * d + 2] * dz);
                        dx -= fmaf(f[0], A.L[0], fmaf(f[1], A.L[3], f[2] * A.L[6]));
                        dy -= fmaf(f[0], A.L[1], fmaf(f[1], A.L[4], f[2] * A.L[7]));
                        dz -= fmaf(f[0], A.L[2], fmaf(f[1], A.L[5], f[2] * A.L[8]));
                        if (fabsf(dx * dx + dy * dy + dz * dz - rmin2) <= 1e-4f * rmin2) {
                            near = near_js - A.st;
                            nx = dx;
                            ny = dy;
                            nz = dz;
                        }
                    }
                    // single bead: the centroid is atom 0 itself, its state in this thread's slot
                    const int64_t k = A.base;
                    const double fx0 = B.fx[k], fy0 = B.fy[k], fz0 = B.fz[k];
                    observe_core(B, P, T.t, step,
                                 rmin2 < INFINITY ? (double)sqrtf(rmin2) * kBohr2Ang : kDefaultReal, near, nx, ny,
                                 nz, B.rx[k], B.ry[k], B.rz[k], B.vx[k], B.vy[k], B.vz[k], fx0, fy0, fz0,
                                 fx0 != 0.0 || fy0 != 0.0 || fz0 != 0.0);
                }
            }
        }
        // a state that stopped being finite in the launch's last step retires the trajectory too
        if (mode == 2 && last >= 0 && A.s >= 0 && A.i == 0 && S.tr_bad[(last & 1) * kRMaxTraj + A.s] &&
            B.status[T.t] == kStatusRunning)
            B.status[T.t] = kStatusErrNonFinite;
    }
    if constexpr (TC) {
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid < 32) tmem_dealloc(C.tmem, kTcCols);
    }
}

template <int KA, int KB, int NH, int BLA, int BLB, int TC>
cudaError_t nnr_launch_t(const LaunchCfg &c, const Batch &B, const RadialNN &R, const EmtConst &E,
                         const NNScratch &X, const PropParams &P, const int2 *packs, const int *ptraj, int npack,
                         size_t sm, int nsteps, int mode) {
    cudaError_t e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(nnr_kernel<KA, KB, NH, BLA, BLB, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    nnr_kernel<KA, KB, NH, BLA, BLB, TC><<<c.grid, R.block, sm, c.stream>>>(B, R, E, X, P, packs, ptraj, npack,
                                                                            c.counter, nsteps, mode);
    return cudaGetLastError();
}

template <int KA, int KB, int NH, int BLA, int BLB, int TC>
int nnr_occupancy_t(int block, size_t sm) {
    int n = 0;
    cudaFuncSetAttribute(nnr_kernel<KA, KB, NH, BLA, BLB, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, nnr_kernel<KA, KB, NH, BLA, BLB, TC>, block, sm);
    // a CTA of the tensor-core kernels holds all 512 TMEM columns of its SM
    return TC ? (n > 0 ? 1 : 0) : n;  // (tensor-core variants: one CTA per SM)
}

}  // namespace

// Instantiated shapes (functions over neighbour element 0 and 1, hidden layers, recurrence
// block lengths): exact sizes for the shipped H/Au surrogate layout (4 + 20 shifted
// Gaussians, recurrences of 4 and 5), and padded kernels with one 2^x per function for any
// other radial model within the limits (unused slots carry zero weights).
#define MDT_NNR_SHAPES(X) X(4, 20, 2, 4, 5) X(24, 24, 2, 0, 0) X(24, 24, 1, 0, 0)

bool nnr_shape(int cnt0, int cnt1, int nh, const int *maxbl, RadialNN &R) {
    bool found = false;
#define MDT_TRY(A_, B_, H_, LA_, LB_)                                                                   \
    if (!found && nh == H_ && cnt0 <= A_ && cnt1 <= B_ && (LA_ == 0 || (cnt0 == A_ && LA_ <= maxbl[0])) && \
        (LB_ == 0 || (cnt1 == B_ && LB_ <= maxbl[1]))) {                                                 \
        R.ka = A_;                                                                                      \
        R.kb = B_;                                                                                      \
        R.bla = LA_;                                                                                    \
        R.blb = LB_;                                                                                    \
        found = true;                                                                                   \
    }
    MDT_NNR_SHAPES(MDT_TRY)
#undef MDT_TRY
    return found;
}

size_t nnr_smem(const RadialNN &R) { return smem_r(R.nin, R.nh, R.tc); }

size_t nnr_hb_bytes(const RadialNN &R) { return hb_bytes(R.nin, R.nh, R.tc); }

size_t nnr_emt_smem(int max_atoms) { return smem_bytes(max_atoms, 1, 8); }

int nnr_resident_ctas(const RadialNN &R) {
    const size_t sm = nnr_smem(R);
#define MDT_OCC(A_, B_, H_, LA_, LB_)                                                   \
    if (R.ka == A_ && R.kb == B_ && R.nh == H_ && R.bla == LA_ && R.blb == LB_) \
        return R.tc == 2 ? nnr_occupancy_t<A_, B_, H_, LA_, LB_, 2>(R.block, sm)       \
               : R.tc == 1 ? nnr_occupancy_t<A_, B_, H_, LA_, LB_, 1>(R.block, sm)     \
                           : nnr_occupancy_t<A_, B_, H_, LA_, LB_, 0>(R.block, sm);
    MDT_NNR_SHAPES(MDT_OCC)
#undef MDT_OCC
    return 0;
}

cudaError_t launch_nnr(const LaunchCfg &c, const Batch &B, const RadialNN &R, const EmtConst &E, const NNScratch &X,
                       const PropParams &P, const int2 *packs, const int *ptraj, int npack, int nsteps, int mode) {
    const size_t sm = nnr_smem(R);
#define MDT_LAUNCH(A_, B_, H_, LA_, LB_)                                                                      \
    if (R.ka == A_ && R.kb == B_ && R.nh == H_ && R.bla == LA_ && R.blb == LB_)                       \
        return R.tc == 2 ? nnr_launch_t<A_, B_, H_, LA_, LB_, 2>(c, B, R, E, X, P, packs, ptraj, npack, sm, nsteps, mode) \
               : R.tc == 1 ? nnr_launch_t<A_, B_, H_, LA_, LB_, 1>(c, B, R, E, X, P, packs, ptraj, npack, sm, nsteps, mode) \
                           : nnr_launch_t<A_, B_, H_, LA_, LB_, 0>(c, B, R, E, X, P, packs, ptraj, npack, sm, nsteps, mode);
    MDT_NNR_SHAPES(MDT_LAUNCH)
#undef MDT_LAUNCH
    return cudaErrorInvalidValue;
}

// The network of a generic model on the tensor cores, as a pass of its own: every bead-atom
// of the batch is a row of a 128-row tile (four tiles per CTA, persistent over the batch);
// its scaled descriptors come from the raw symmetry functions G [ba][maxsf] of a descriptor
// pass, and the atomic energy (Ha) and dE/dG go to eat / dg for a forces pass (the
// descriptor VJP of the generic kernels).  R holds the network's tables with the model's
// own descriptor order (qsrc the identity up to nsf).
template <int NIN, int NH, int TC>
__global__ void __launch_bounds__(kRBlockMax, 1)
    nn_tc_kernel(Batch B, RadialNN R, const double *G, const int *ba_traj, int64_t total_ba, float *dg, double *eat,
                 int *err, int do_forces) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const SmemR S = carve_r<NIN, NH, TC>(smem_raw);
    const int tid = threadIdx.x;
    TcCtx C{0u, S.tcbar, err};
    uint32_t phase = 0;
    load_weights_tc<NIN, NH, TC == 2>(R, S);
    if (tid < 32) {
        tmem_alloc(S.tslot, kTcCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        for (int g = 0; g < kTcTiles; ++g) mbar_init(&S.tcbar[g], 1);
        fence_mbar_init();
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    C.tmem = *S.tslot;
    // uniform over the CTA: every thread takes part in every tile's GEMMs
    for (int64_t k0 = (int64_t)blockIdx.x * kRBlockMax; k0 < total_ba; k0 += (int64_t)gridDim.x * kRBlockMax) {
        const int64_t k = k0 + tid;
        int ei = -1;
        float xs[NIN];
#pragma unroll
        for (int q = 0; q < NIN; ++q) xs[q] = 0.f;
        if (k < total_ba) {
            const TrajView T = traj_view(B, ba_traj[k]);
            const int i = (int)((k - T.base) % T.N);
            ei = R.elem_of_type[B.type[T.aoff + i]];
            if (ei >= 0) {
                const float4 *sc = S.scal + ei * NIN;
                const double *g = G + k * R.maxsf;
#pragma unroll
                for (int q = 0; q < NIN; ++q) {
                    const int s = R.qsrc[ei][q];
                    if (s >= 0) xs[q] = fmaf(sc[q].x, (float)g[s], sc[q].y);
                }
            }
        }
        float dgv[NIN];
        const float e = nnr_network_tc<NIN, NH, TC == 2>(R, S, C, ei >= 0 ? ei : 0, xs, do_forces != 0, dgv, phase);
        if (ei >= 0) {
            eat[k] = (double)e;
            if (do_forces)
#pragma unroll
                for (int q = 0; q < NIN; ++q) {
                    const int s = R.qsrc[ei][q];
                    if (s >= 0) dg[k * R.maxsf + s] = dgv[q];
                }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_dealloc(C.tmem, kTcCols);
}

template <int NIN, int NH, int TC>
cudaError_t nn_tc_launch_t(cudaStream_t s, int grid, const Batch &B, const RadialNN &R, const double *G,
                           const int *ba_traj, int64_t total_ba, float *dg, double *eat, int *err, int do_forces) {
    const size_t sm = smem_r(NIN, NH, TC);
    cudaError_t e = cudaFuncSetAttribute(nn_tc_kernel<NIN, NH, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    nn_tc_kernel<NIN, NH, TC><<<grid, kRBlockMax, sm, s>>>(B, R, G, ba_traj, total_ba, dg, eat, err, do_forces);
    return cudaGetLastError();
}

size_t nn_tc_smem(int nin, int nh, int tc) { return smem_r(nin, nh, tc); }

cudaError_t launch_nn_tc(cudaStream_t s, int grid, const Batch &B, const RadialNN &R, const double *G,
                         const int *ba_traj, int64_t total_ba, float *dg, double *eat, int *err, int do_forces) {
#define MDT_NNTC(NIN_, NH_)                                                                                  \
    if (R.nin == NIN_ && R.nh == NH_)                                                                        \
        return R.tc == 2 ? nn_tc_launch_t<NIN_, NH_, 2>(s, grid, B, R, G, ba_traj, total_ba, dg, eat, err, do_forces) \
                         : nn_tc_launch_t<NIN_, NH_, 1>(s, grid, B, R, G, ba_traj, total_ba, dg, eat, err, do_forces);
    MDT_NNTC(24, 2) MDT_NNTC(24, 1) MDT_NNTC(48, 2) MDT_NNTC(48, 1)
#undef MDT_NNTC
    return cudaErrorInvalidValue;
}

__global__ void lcoef_kernel(Batch B, PropParams P, const int *ba_traj, int64_t total_ba, double *lcoef) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total_ba; k += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[k];
        const TrajView T = traj_view(B, t);
        const int i = (int)(k - T.base);
        if (T.nb == 1 && B.algo[B.type[T.aoff + i]] == kPropLangevinConst) lc_setup(B, P, T, i, lcoef + kLcN * k, 1);
    }
}

cudaError_t launch_nnr_lcoef(cudaStream_t s, const Batch &B, const PropParams &P, const int *ba_traj,
                             int64_t total_ba, double *lcoef) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    lcoef_kernel<<<std::max(grid, 1), 256, 0, s>>>(B, P, ba_traj, total_ba, lcoef);
    return cudaGetLastError();
}

// The tensor-core network's wait, exercised alone: every thread waits (max_polls tries, as a
// GEMM round does) on an mbarrier of one arrival; with arrive the CTA's thread 0 arrives
// first, without it nothing ever completes the phase and every wait must give up and set
// the error word.
__global__ void wait_check_kernel(uint32_t max_polls, int arrive, int *err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (arrive && threadIdx.x == 0) mbar_arrive(&bar);
    if (!mbar_wait_bounded(&bar, 0u, max_polls)) atomicExch(err, 1);
}

}  // namespace mdt

extern "C" int32_t mdt_wait_check(int32_t max_polls, int32_t arrive, int32_t *timed_out, double *ms) {
    if (!timed_out || max_polls < 0) return MDT_ERR_ARG;
    const uint32_t polls = max_polls == 0 ? mdt::kTcMaxPolls : (uint32_t)max_polls;
    int *err = nullptr;
    if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return MDT_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaMemset(err, 0, sizeof(int));
    cudaEventRecord(e0);
    if (e == cudaSuccess) mdt::wait_check_kernel<<<1, 128>>>(polls, arrive ? 1 : 0, err);
    cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
    float t = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(err);
    if (e != cudaSuccess) return MDT_ERR_CUDA;
    *timed_out = h;
    if (ms) *ms = t;
    return MDT_OK;
}
