// mdt_emt.cuh -- EMT energy/force for one bead inside a CTA (device code shared by
// the EMT kernels and the surrogate's EMT fallback).
#pragma once
#include "mdt_common.cuh"

namespace mdt {

constexpr int kBlock = 128;  // threads per CTA (one trajectory per CTA)

// ---------------------------------------------------------------------------
// Arithmetic helpers.  On GB300 an FP64 instruction costs as much issue bandwidth as
// ~64 FP32 ones, so the FP64 kernels keep every FP64 operation that is not needed
// for 1e-10 eV/A parity off the FP64 pipe:
//  * reciprocal and reciprocal square root start from the hardware approximations
//    (rcp/rsqrt.approx.ftz.f64) and are refined by two Newton-Raphson steps, which is
//    accurate to ~1 ulp (the approximations are good to ~2^-23; each step squares the
//    relative error);
//  * the minimum-image shift (an integer per cell direction) is found in FP32 and
//    applied in FP64; when FP32 cannot decide the rounding (fractional part within
//    1e-4 of 1/2) the fractional coordinate is recomputed in FP64.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ double rcp_nr(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

static __device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = 0.5 * x;
    double t = y * y;
    y = fma(y, fma(-h, t, 0.5), y);
    t = y * y;
    return fma(y, fma(-h, t, 0.5), y);
}

// FP64 exp by the table-driven method of Tang (ACM TOMS 15(2), 1989): x = (64 n_hi + j)
// ln2/64 + r with |r| <= ln2/128, exp(x) = 2^n_hi 2^(j/64) (1 + p(r)), p the Taylor series
// of exp(r) - 1 to r^5 (truncation below 2^-54).  The 64 entries 2^(j/64) come from exp2
// (e2t, filled per call); ln2/64 enters in two parts (its double, then the remainder) so
// that r is exact to ~2^-100, and n = round(64 x / ln2) comes from adding 1.5 * 2^52.
// About 12 FP64 instructions against ~19 for exp(), within 1 ulp of exp() on [-700, 700]
// (measured on GB300); outside that range, and for NaN, exp() itself.
static __device__ __forceinline__ double exp_t64(double x, const double *e2t) {
    if (!(fabs(x) <= 700.0)) return exp(x);
    const double shifter = 6755399441055744.0;
    const double t = fma(x, 92.332482616893657, shifter);
    const int n = __double2loint(t);
    const double nd = t - shifter;
    double r = fma(-nd, 0x1.62e42fefa39efp-7, x);
    r = fma(-nd, 0x1.abc9e3b39803fp-62, r);
    double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
    q = fma(r, q, 1.0 / 6.0);
    q = fma(r, q, 0.5);
    const double pr = fma(r * r, q, r);
    const double tj = e2t[n & 63];
    const double y = fma(tj, pr, tj);
    return __hiloint2double(__double2hiint(y) + (n >> 6) * (1 << 20), __double2loint(y));
}

template <typename R> struct M;
template <> struct M<double> {
    static __device__ __forceinline__ double ex(double x) { return exp(x); }
    static __device__ __forceinline__ double ex(double x, const double *e2t) { return exp_t64(x, e2t); }
    static __device__ __forceinline__ double rcp(double x) { return rcp_nr(x); }
    static __device__ __forceinline__ double rsq(double x) { return rsqrt_nr(x); }
};
template <> struct M<float> {
    static __device__ __forceinline__ float ex(float x) { return __expf(x); }
    static __device__ __forceinline__ float ex(float x, const double *) { return __expf(x); }
    static __device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
    static __device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }
};

struct Cell;

template <typename R> struct SmemEmt {
    double *px, *py, *pz;  // staged bead positions
    float *xh, *yh, *zh, *xl, *yl, *zl;  // FP32 forces (R = float): their FP32 hi/lo split
    R *sig, *A, *fx, *fy, *fz;
    Cell *cell;
    int8_t *slot;          // EMT species slot per atom (-1: none)
    int8_t *typ;           // universe type per atom
    double *red;           // 64 doubles for block reductions
    double *e2t;           // 2^(j/64), j < 64 (exp_t64: the pair loop in FP64, the per-atom epilogue)
    double *cjk;           // the trajectory's normal-mode table, then its per-type, per-mode
                           // propagator tables (rp_cells doubles in all)
};

// doubles of the normal-mode area: the nb x nb table and 5 per-type, per-mode tables
__host__ __device__ constexpr size_t rp_cells(int max_beads) {
    return (size_t)max_beads * max_beads + 5 * (size_t)kMaxTypes * max_beads;
}

template <typename R>
static __device__ SmemEmt<R> carve_smem(unsigned char *base, int max_atoms, int max_beads) {
    SmemEmt<R> s;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += (bytes + 15) & ~size_t(15);
        return p;
    };
    s.px = (double *)take(sizeof(double) * max_atoms);
    s.py = (double *)take(sizeof(double) * max_atoms);
    s.pz = (double *)take(sizeof(double) * max_atoms);
    const size_t nf = sizeof(R) == 4 ? sizeof(float) * max_atoms : 0;
    s.xh = (float *)take(nf);
    s.yh = (float *)take(nf);
    s.zh = (float *)take(nf);
    s.xl = (float *)take(nf);
    s.yl = (float *)take(nf);
    s.zl = (float *)take(nf);
    s.red = (double *)take(sizeof(double) * 64);
    s.e2t = (double *)take(sizeof(double) * 64);
    s.cjk = (double *)take(sizeof(double) * rp_cells(max_beads));
    s.sig = (R *)take(sizeof(R) * max_atoms);
    s.A = (R *)take(sizeof(R) * max_atoms);
    s.fx = (R *)take(sizeof(R) * max_atoms);
    s.fy = (R *)take(sizeof(R) * max_atoms);
    s.fz = (R *)take(sizeof(R) * max_atoms);
    s.cell = (Cell *)take(256);
    s.slot = (int8_t *)take(max_atoms);
    s.typ = (int8_t *)take(max_atoms);
    return s;
}

inline size_t smem_bytes(int max_atoms, int max_beads, size_t rsize) {
    auto r16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    return 3 * r16(8 * max_atoms) + (rsize == 4 ? 6 * r16(4 * max_atoms) : 0) + 2 * r16(8 * 64) +
           r16(8 * rp_cells(max_beads)) + 5 * r16(rsize * max_atoms) +
           256 + 2 * r16(max_atoms);
}

// Block-wide sum of a double; every thread gets the result.
static __device__ __noinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[w];
    __syncthreads();
    return t;
}

// Block-wide minimum of a double; every thread gets the result.
static __device__ __noinline__ double block_min(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double m = red[0];
    for (int w = 1; w < nw; ++w) m = fmin(m, red[w]);
    __syncthreads();
    return m;
}

// Cell of one trajectory: FP64 matrix for applying image shifts, FP32 inverse for
// choosing them.  Column major (cell vectors as columns).
struct Cell {
    double h[9], hi[9];
    float hif[9], hf[9];  // FP32 inverse and (FP32 bead forces) FP32 matrix
    unsigned nz;  // bit k set when h[k] != 0
};
static_assert(sizeof(Cell) <= 256, "the shared-memory carve reserves 256 bytes for the cell");

static __device__ __forceinline__ void load_cell(const Batch &B, int t, Cell &c) {
    unsigned nz = 0;
    for (int k = 0; k < 9; ++k) {
        c.h[k] = B.box[9 * t + k];
        c.hi[k] = B.ibox[9 * t + k];
        c.hif[k] = (float)c.hi[k];
        c.hf[k] = (float)c.h[k];
        if (c.h[k] != 0.0) nz |= 1u << k;
    }
    c.nz = nz;
}

// image index n = anint(w) for one fractional coordinate (Fortran anint: half away
// from zero).  FP32 decides unless it is within 1e-4 of a tie; then the fractional
// coordinate is recomputed in FP64 with the oracle's operation order and no fused
// multiply-add, so that exact ties (pairs half a cell apart on a perfect lattice) pick
// the same image on both sides.
static __device__ __forceinline__ double image_shift(float wf, const double *hi_row3, double ex, double ey, double ez,
                                                     int row) {
    const float n = roundf(wf);
    if (fabsf(fabsf(wf - n) - 0.5f) > 1e-4f) return (double)n;
    const double w = __dadd_rn(__dadd_rn(__dmul_rn(hi_row3[row], ex), __dmul_rn(hi_row3[row + 3], ey)),
                               __dmul_rn(hi_row3[row + 6], ez));
    return round(w);
}

// FP32 bead forces: the minimum image of r_i - r_j from the FP32 hi/lo split of the
// positions, with the image chosen as min_image chooses it (FP32, exact ties in FP64)
// and applied in FP32: no FP64 instruction per pair unless a pair sits on a tie.
template <typename S_>
static __device__ __forceinline__ void min_image_f(const Cell &c, const S_ &S, int i, int j, float &dx, float &dy,
                                            float &dz) {
    const float ex = (S.xh[i] - S.xh[j]) + (S.xl[i] - S.xl[j]);
    const float ey = (S.yh[i] - S.yh[j]) + (S.yl[i] - S.yl[j]);
    const float ez = (S.zh[i] - S.zh[j]) + (S.zl[i] - S.zl[j]);
    float n[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float w = c.hif[r] * ex + c.hif[r + 3] * ey + c.hif[r + 6] * ez;
        n[r] = roundf(w);
        if (!(fabsf(fabsf(w - n[r]) - 0.5f) > 1e-4f))
            n[r] = (float)image_shift(w, c.hi, S.px[i] - S.px[j], S.py[i] - S.py[j], S.pz[i] - S.pz[j], r);
    }
    dx = ex - (c.hf[0] * n[0] + c.hf[3] * n[1] + c.hf[6] * n[2]);
    dy = ey - (c.hf[1] * n[0] + c.hf[4] * n[1] + c.hf[7] * n[2]);
    dz = ez - (c.hf[2] * n[0] + c.hf[5] * n[1] + c.hf[8] * n[2]);
}

// minimum image of e = r_i - r_j, src/universe_mod.f90:411-428
static __device__ __forceinline__ void min_image(const Cell &c, double ex, double ey, double ez, double &dx, double &dy,
                                          double &dz) {
    const float fx = (float)ex, fy = (float)ey, fz = (float)ez;
    const float w0 = c.hif[0] * fx + c.hif[3] * fy + c.hif[6] * fz;
    const float w1 = c.hif[1] * fx + c.hif[4] * fy + c.hif[7] * fz;
    const float w2 = c.hif[2] * fx + c.hif[5] * fy + c.hif[8] * fz;
    const double n0 = image_shift(w0, c.hi, ex, ey, ez, 0);
    const double n1 = image_shift(w1, c.hi, ex, ey, ez, 1);
    const double n2 = image_shift(w2, c.hi, ex, ey, ez, 2);
    dx = ex;
    dy = ey;
    dz = ez;
    if (n0 != 0.0) {
        if (c.nz & 1u) dx = fma(-c.h[0], n0, dx);
        if (c.nz & 2u) dy = fma(-c.h[1], n0, dy);
        if (c.nz & 4u) dz = fma(-c.h[2], n0, dz);
    }
    if (n1 != 0.0) {
        if (c.nz & 8u) dx = fma(-c.h[3], n1, dx);
        if (c.nz & 16u) dy = fma(-c.h[4], n1, dy);
        if (c.nz & 32u) dz = fma(-c.h[5], n1, dz);
    }
    if (n2 != 0.0) {
        if (c.nz & 64u) dx = fma(-c.h[6], n2, dx);
        if (c.nz & 128u) dy = fma(-c.h[7], n2, dy);
        if (c.nz & 256u) dz = fma(-c.h[8], n2, dz);
    }
}

// ---------------------------------------------------------------------------
// EMT for one bead of one trajectory.  Adds forces into B.f*, sets dens, adds the
// bead's energy into B.epot.  Must be called by all threads of the CTA.
//
// Pair layout: pair (i, j = (i+k) mod N), k = 1..N/2, lives in scratch slot
// p = (k-1)*N + i (the k = N/2 row holds only i < N/2 when N is even).  Each slot
// keeps d = r_i - r_j, the density-derivative scalars Q_ij, Q_ji and the pair-
// potential force scalar F_V.  Pass 1 walks rows: thread i owns atom i and visits its
// pairs k = 1..N/2 in lockstep with its warp, so lanes touch distinct atoms j (no
// shared-memory atomic conflicts) and write consecutive scratch slots.  Pass 2 is a
// gather: thread i reads the slots where it is the first atom and those where it is
// the second, so forces need no atomics at all.
// ---------------------------------------------------------------------------
template <typename R>
static __device__ void emt_bead(const Batch &B, const EmtConst &E, const SmemEmt<R> &S, int t, int b,
                         bool do_forces) {
    const int N = B.natoms[t];
    const int64_t base = B.ba_off[t] + (int64_t)b * N;
    const int aoff = B.atom_off[t];
    const int tid = threadIdx.x, nt = blockDim.x;

    for (int i = tid; i < N; i += nt) {
        S.px[i] = B.rx[base + i];
        S.py[i] = B.ry[base + i];
        S.pz[i] = B.rz[base + i];
        if constexpr (sizeof(R) == 4) {
            const double x = S.px[i], y = S.py[i], z = S.pz[i];
            S.xh[i] = (float)x;
            S.yh[i] = (float)y;
            S.zh[i] = (float)z;
            S.xl[i] = (float)(x - (double)S.xh[i]);
            S.yl[i] = (float)(y - (double)S.yh[i]);
            S.zl[i] = (float)(z - (double)S.zh[i]);
        }
        const int ty = B.type[aoff + i];
        S.typ[i] = (int8_t)ty;
        S.slot[i] = (int8_t)E.slot_of_type[ty];
        S.sig[i] = R(0);
        S.fx[i] = R(0);
        S.fy[i] = R(0);
        S.fz[i] = R(0);
    }
    for (int k = tid; k < 64; k += nt) S.e2t[k] = exp2((double)k * (1.0 / 64.0));
    if (tid == 0) load_cell(B, t, *S.cell);
    __syncthreads();
    const Cell &cell = *S.cell;

    const int K = N / 2, NK = N * K;
    R *scr = (R *)B.pair_scratch + 6 * (B.pair_off[t] + (int64_t)b * NK);
    R *s_dx = scr, *s_dy = scr + NK, *s_dz = scr + 2 * NK, *s_qij = scr + 3 * NK, *s_qji = scr + 4 * NK,
      *s_fv = scr + 5 * NK;
    const R cut2 = (R)E.cut2, acut = (R)E.acut, rcut = (R)E.rcut;
    double e_pair = 0.0;

    // ---- pass 1 (pair-parallel; consecutive threads take consecutive atoms i of one
    // k row, so their shared-memory atomics hit distinct atoms) --------------------
    for (int p = tid; p < NK; p += nt) {
        const int k = p / N + 1, i = p - (k - 1) * N;
        int j = i + k;
        if (j >= N) j -= N;
        const int ti = S.typ[i], tj = S.typ[j];
        R q_ij = R(0), q_ji = R(0), fv = R(0), rx = R(0), ry = R(0), rz = R(0);
        if (!(2 * k == N && i >= K) && ((E.pair_mask >> (ti * kMaxTypes + tj)) & 1u)) {
            if constexpr (sizeof(R) == 4) {
                min_image_f(cell, S, i, j, rx, ry, rz);
            } else {
                double dx, dy, dz;
                min_image(cell, S.px[i] - S.px[j], S.py[i] - S.py[j], S.pz[i] - S.pz[j], dx, dy, dz);
                rx = (R)dx;
                ry = (R)dy;
                rz = (R)dz;
            }
            const R r2 = rx * rx + ry * ry + rz * rz;
            // skipped only beyond the cutoff, like the reference's `if (r > cutoff*rcut) cycle`
            // (pes_emt_mod.f90:660): a distance that is not a number enters the sums
            if (!(r2 > cut2)) {
                const R ir = M<R>::rsq(r2), r = r2 * ir;
                const R e = M<R>::ex(acut * (r - rcut), S.e2t);
                const R theta = M<R>::rcp(R(1) + e);
                const R rt1 = acut * e * theta;
                const int si = S.slot[i], sj = S.slot[j];
                const R phi_j = theta * M<R>::ex(-(R)E.eta2[sj] * (r - (R)E.betas0[sj]), S.e2t);
                const R psi_j = theta * M<R>::ex(-(R)E.kappadbeta[sj] * (r - (R)E.betas0[sj]), S.e2t);
                R phi_i = phi_j, psi_i = psi_j;
                if (si != sj) {
                    phi_i = theta * M<R>::ex(-(R)E.eta2[si] * (r - (R)E.betas0[si]), S.e2t);
                    psi_i = theta * M<R>::ex(-(R)E.kappadbeta[si] * (r - (R)E.betas0[si]), S.e2t);
                }
                const R gij = (R)(E.igamma1[si] * E.chi[si][sj]);
                const R gji = (R)(E.igamma1[sj] * E.chi[sj][si]);
                atomicAdd(&S.sig[i], gij * phi_j);
                atomicAdd(&S.sig[j], gji * phi_i);
                const R cij = (R)(E.g2v0[si] * E.chi[si][sj]);
                const R cji = (R)(E.g2v0[sj] * E.chi[sj][si]);
                e_pair -= 0.5 * (double)(cij * psi_j + cji * psi_i);
                fv = -R(0.5) * (cij * ((R)E.kappadbeta[sj] + rt1) * psi_j +
                                cji * ((R)E.kappadbeta[si] + rt1) * psi_i) * ir;
                R eta_j = (R)E.eta2[sj], eta_i = (R)E.eta2[si];
                // QUIRK kept from pes_emt_mod.f90:705: the type1-type1 density
                // derivative uses eta2 of type2.
                if (E.hh_quirk && si == 0 && sj == 0) eta_j = eta_i = (R)E.eta2[1];
                q_ij = gij * (eta_j + rt1) * phi_j * ir;
                q_ji = gji * (eta_i + rt1) * phi_i * ir;
            }
        }
        if (do_forces) {
            s_dx[p] = rx;
            s_dy[p] = ry;
            s_dz[p] = rz;
            s_qij[p] = q_ij;
            s_qji[p] = q_ji;
            s_fv[p] = fv;
        }
    }
    __syncthreads();

    // ---- per-atom epilogue ---------------------------------------------------
    double e_atom = 0.0;
    for (int i = tid; i < N; i += nt) {
        const int s = S.slot[i];
        if (s < 0) {
            S.A[i] = R(0);
            continue;
        }
        const double sc = fmax((double)1e-30f, (double)S.sig[i]);  // single-precision 1e-30, pes_emt_mod.f90:793
        const double sa = -log(fmax(kTolerance, sc) * kTwelfth) / E.betaeta2[s];
        const double el = exp_t64(-E.lambda[s] * sa, S.e2t), ek = exp_t64(-E.kappa[s] * sa, S.e2t);
        e_atom += E.e0[s] * ((1.0 + E.lambda[s] * sa) * el - 1.0) + 6.0 * E.v0[s] * ek;
        const double W = E.e0[s] * E.lambda[s] * E.lambda[s] * sa * el + 6.0 * E.v0[s] * E.kappa[s] * ek;
        S.A[i] = (R)(W / (E.betaeta2[s] * sc));
        B.dens[base + i] = E.n0[s] * exp_t64(E.dens_exp[s] * sa, S.e2t);
    }
    const double etot = block_sum(e_pair + e_atom, S.red);  // contains __syncthreads
    if (tid == 0) B.epot[B.bead_off[t] + b] += etot;
    if (!do_forces) return;

    // ---- pass 2 (gather): work item (i, chunk of k); consecutive threads take
    // consecutive atoms, partial forces meet in shared memory ----------------------
    const int C = (N >= nt) ? 1 : min(K > 0 ? K : 1, nt / N);
    const int per = (K + C - 1) / C;
    for (int w = tid; w < N * C; w += nt) {
        const int c = w / N, i = w - c * N;
        const int k0 = 1 + c * per, k1 = min(K, (c + 1) * per);
        const R Ai = S.A[i];
        R fx = R(0), fy = R(0), fz = R(0);
        for (int k = k0; k <= k1; ++k) {
            const bool half = (2 * k == N);
            int j = i + k;
            if (j >= N) j -= N;
            if (!(half && i >= K)) {  // i is the first atom of pair (i, i+k)
                const int p = (k - 1) * N + i;
                const R cc = Ai * s_qij[p] + S.A[j] * s_qji[p] + s_fv[p];
                fx += cc * s_dx[p];
                fy += cc * s_dy[p];
                fz += cc * s_dz[p];
            }
            int m = i - k;
            if (m < 0) m += N;
            if (!(half && m >= K)) {  // i is the second atom of pair (m, m+k)
                const int p = (k - 1) * N + m;
                const R cc = S.A[m] * s_qij[p] + Ai * s_qji[p] + s_fv[p];
                fx -= cc * s_dx[p];
                fy -= cc * s_dy[p];
                fz -= cc * s_dz[p];
            }
        }
        if (C == 1) {
            S.fx[i] = fx;
            S.fy[i] = fy;
            S.fz[i] = fz;
        } else {
            atomicAdd(&S.fx[i], fx);
            atomicAdd(&S.fy[i], fy);
            atomicAdd(&S.fz[i], fz);
        }
    }
    __syncthreads();
    for (int i = tid; i < N; i += nt) {
        B.fx[base + i] += (double)S.fx[i];
        B.fy[base + i] += (double)S.fy[i];
        B.fz[base + i] += (double)S.fz[i];
    }
    __syncthreads();
}

}  // namespace mdt
