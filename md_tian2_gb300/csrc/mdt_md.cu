// mdt_md.cu -- batched EMT force evaluation and propagators for sm_103a.
//
// One CTA owns one trajectory (all its beads) at a time and pulls trajectories from a
// work queue ordered largest-first.  Within a CTA:
//   * the bead being evaluated is staged in shared memory (positions, accumulators);
//   * unordered atom pairs are enumerated in a rectangular N x (N/2) layout (pair
//     (i, (i+k) mod N), k = 1..N/2, the k = N/2 row halved for even N), so every thread
//     gets the same amount of work without a square-root index decode;
//   * EMT is evaluated in two pair passes around a per-atom epilogue: pass 1 builds the
//     neutral-sphere densities and the pair-potential forces and leaves the pair's
//     density-derivative scalars in a global scratch slot; the epilogue turns each
//     atom's density into s_i, its energy, its embedded density and the coefficient
//     A_i = (dE/ds_i) / (beta*eta2*sigma_i); pass 2 scatters (A_i Q_ij + A_j Q_ji) d_ij.
//     This is the O(N^2)-time, O(N)-memory restatement of the reference's dense
//     (3,nb,N,N) derivative tensors (src/pes_emt_mod.f90:483-1027).
// The fused kernel runs propagate_1 -> calc_force -> propagate_2 for many steps
// without leaving the CTA (md_tian2.f90:78-92).
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_internal.h"

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
__device__ __forceinline__ double rcp_nr(double x) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = 0.5 * x;
    double t = y * y;
    y = fma(y, fma(-h, t, 0.5), y);
    t = y * y;
    return fma(y, fma(-h, t, 0.5), y);
}

template <typename R> struct M;
template <> struct M<double> {
    static __device__ __forceinline__ double ex(double x) { return exp(x); }
    static __device__ __forceinline__ double rcp(double x) { return rcp_nr(x); }
    static __device__ __forceinline__ double rsq(double x) { return rsqrt_nr(x); }
};
template <> struct M<float> {
    static __device__ __forceinline__ float ex(float x) { return __expf(x); }
    static __device__ __forceinline__ float rcp(float x) { return __frcp_rn(x); }
    static __device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }
};

struct Cell;

template <typename R> struct SmemEmt {
    double *px, *py, *pz;  // staged bead positions
    R *sig, *A, *fx, *fy, *fz;
    Cell *cell;
    int8_t *slot;          // EMT species slot per atom (-1: none)
    int8_t *typ;           // universe type per atom
    double *red;           // 64 doubles for block reductions
    double *cjk;           // max_beads^2 normal-mode table
};

template <typename R>
__device__ SmemEmt<R> carve_smem(unsigned char *base, int max_atoms, int max_beads) {
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
    s.red = (double *)take(sizeof(double) * 64);
    s.cjk = (double *)take(sizeof(double) * max_beads * max_beads);
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

size_t smem_bytes(int max_atoms, int max_beads, size_t rsize) {
    auto r16 = [](size_t b) { return (b + 15) & ~size_t(15); };
    return 3 * r16(8 * max_atoms) + r16(8 * 64) + r16(8 * max_beads * max_beads) + 5 * r16(rsize * max_atoms) +
           256 + 2 * r16(max_atoms);
}

// Block-wide sum of a double; every thread gets the result.
__device__ double block_sum(double v, double *red) {
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

// Cell of one trajectory: FP64 matrix for applying image shifts, FP32 inverse for
// choosing them.  Column major (cell vectors as columns).
struct Cell {
    double h[9], hi[9];
    float hif[9];
    unsigned nz;  // bit k set when h[k] != 0
};

__device__ __forceinline__ void load_cell(const Batch &B, int t, Cell &c) {
    unsigned nz = 0;
    for (int k = 0; k < 9; ++k) {
        c.h[k] = B.box[9 * t + k];
        c.hi[k] = B.ibox[9 * t + k];
        c.hif[k] = (float)c.hi[k];
        if (c.h[k] != 0.0) nz |= 1u << k;
    }
    c.nz = nz;
}

// image index n = anint(w) for one fractional coordinate (Fortran anint: half away
// from zero).  FP32 decides unless it is within 1e-4 of a tie.
__device__ __forceinline__ double image_shift(float wf, const double *hi_row3, double ex, double ey, double ez,
                                              int row) {
    const float n = roundf(wf);
    if (fabsf(fabsf(wf - n) - 0.5f) > 1e-4f) return (double)n;
    const double w = hi_row3[row] * ex + hi_row3[row + 3] * ey + hi_row3[row + 6] * ez;
    return round(w);
}

// minimum image of e = r_i - r_j, src/universe_mod.f90:411-428
__device__ __forceinline__ void min_image(const Cell &c, double ex, double ey, double ez, double &dx, double &dy,
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
__device__ void emt_bead(const Batch &B, const EmtConst &E, const SmemEmt<R> &S, int t, int b,
                         bool do_forces) {
    const int N = B.natoms[t];
    const int64_t base = B.ba_off[t] + (int64_t)b * N;
    const int aoff = B.atom_off[t];
    const int tid = threadIdx.x, nt = blockDim.x;

    for (int i = tid; i < N; i += nt) {
        S.px[i] = B.rx[base + i];
        S.py[i] = B.ry[base + i];
        S.pz[i] = B.rz[base + i];
        const int ty = B.type[aoff + i];
        S.typ[i] = (int8_t)ty;
        S.slot[i] = (int8_t)E.slot_of_type[ty];
        S.sig[i] = R(0);
        S.fx[i] = R(0);
        S.fy[i] = R(0);
        S.fz[i] = R(0);
    }
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
            double dx, dy, dz;
            min_image(cell, S.px[i] - S.px[j], S.py[i] - S.py[j], S.pz[i] - S.pz[j], dx, dy, dz);
            rx = (R)dx;
            ry = (R)dy;
            rz = (R)dz;
            const R r2 = rx * rx + ry * ry + rz * rz;
            if (r2 <= cut2) {
                const R ir = M<R>::rsq(r2), r = r2 * ir;
                const R e = M<R>::ex(acut * (r - rcut));
                const R theta = M<R>::rcp(R(1) + e);
                const R rt1 = acut * e * theta;
                const int si = S.slot[i], sj = S.slot[j];
                const R phi_j = theta * M<R>::ex(-(R)E.eta2[sj] * (r - (R)E.betas0[sj]));
                const R psi_j = theta * M<R>::ex(-(R)E.kappadbeta[sj] * (r - (R)E.betas0[sj]));
                R phi_i = phi_j, psi_i = psi_j;
                if (si != sj) {
                    phi_i = theta * M<R>::ex(-(R)E.eta2[si] * (r - (R)E.betas0[si]));
                    psi_i = theta * M<R>::ex(-(R)E.kappadbeta[si] * (r - (R)E.betas0[si]));
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
        const double el = exp(-E.lambda[s] * sa), ek = exp(-E.kappa[s] * sa);
        e_atom += E.e0[s] * ((1.0 + E.lambda[s] * sa) * el - 1.0) + 6.0 * E.v0[s] * ek;
        const double W = E.e0[s] * E.lambda[s] * E.lambda[s] * sa * el + 6.0 * E.v0[s] * E.kappa[s] * ek;
        S.A[i] = (R)(W / (E.betaeta2[s] * sc));
        B.dens[base + i] = E.n0[s] * exp(E.dens_exp[s] * sa);
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

// ---------------------------------------------------------------------------
// Propagators (src/md_algo.f90).  Thread per atom, all beads of the atom.
// ---------------------------------------------------------------------------
struct TrajView {
    int t, N, nb, aoff;
    int64_t base;
};

__device__ __forceinline__ TrajView traj_view(const Batch &B, int t) {
    return TrajView{t, B.natoms[t], B.nbeads[t], B.atom_off[t], B.ba_off[t]};
}

__device__ __forceinline__ double temp_of(const Batch &B, const PropParams &P, int ty) {
    return B.is_proj[ty] ? P.Tproj : P.Tsurf;
}

// Deviate for (bead b, atom i, dimension d).  Host-provided arrays use the reference's
// Fortran order (3, nb, N) per trajectory, concatenated.
__device__ __forceinline__ double rand_normal(const PropParams &P, const TrajView &T, int step, int b, int i,
                                              int d, uint32_t stream, const double *injected) {
    if (P.rng_mode == 1) return injected[(T.base + (int64_t)i * T.nb + b) * 3 + d];
    return normal_deviate(P.seed, (uint32_t)T.t, (uint32_t)step, (uint32_t)((b * T.N + i) * 3 + d), stream);
}

__device__ __forceinline__ double &comp(double *x, double *y, double *z, int d, int64_t k) {
    return d == 0 ? x[k] : (d == 1 ? y[k] : z[k]);
}

// verlet_1 / verlet_2, md_algo.f90:110-142
__device__ void verlet_half(const Batch &B, const PropParams &P, const TrajView &T, int i, bool move_r) {
    for (int b = 0; b < T.nb; ++b) {
        const int64_t k = T.base + (int64_t)b * T.N + i;
        const uint8_t fx = B.fixed[k];
        for (int d = 0; d < 3; ++d) {
            double &v = comp(B.vx, B.vy, B.vz, d, k);
            if (!(fx >> d & 1)) v = v + 0.5 * P.step * comp(B.ax, B.ay, B.az, d, k);
            else v = 0.0;
        }
    }
    if (move_r && T.nb == 1) {
        const int64_t k = T.base + i;
        const uint8_t fx = B.fixed[k];
        for (int d = 0; d < 3; ++d)
            if (!(fx >> d & 1)) comp(B.rx, B.ry, B.rz, d, k) += P.step * comp(B.vx, B.vy, B.vz, d, k);
    }
}

struct LangCoef { double c0, c1, c2, sigma_r, sigma_v, c_rv; };

// md_algo.f90:165-198 (first half) and 253-285 (second half)
__device__ void langevin_coef(double xi, double step, double temp, bool all_big, bool second, LangCoef &c) {
    const double xidt = xi * step, xidt2 = xidt * xidt, ixidt = step / xidt;
    if (all_big && temp > kTolerance) {
        c.c0 = exp(-xidt);
        c.c1 = (1 - c.c0) * ixidt;
        c.c2 = (1 - c.c1 / step) * ixidt;
        c.sigma_r = ixidt * sqrt(temp * (2 * xidt - 3 + 4 * c.c0 - c.c0 * c.c0));
        c.sigma_v = sqrt(temp * (1 - c.c0 * c.c0));
        c.c_rv = ixidt * temp * (1 - c.c0) * (1 - c.c0) / (c.sigma_r * c.sigma_v);
    } else {
        c.c0 = 1 - xidt + 0.5 * xidt2;
        c.c1 = (1 - 0.5 * xidt + 2 * kTwelfth * xidt2) * step;
        c.c2 = (0.5 - 2 * kTwelfth * xidt + 0.5 * kTwelfth * xidt2) * step;
        c.sigma_r = second ? 0.0 : step * sqrt(temp * (8 * kTwelfth * xidt - 0.5 * xidt2));
        c.sigma_v = sqrt(2 * temp * xidt * (1 - xidt));
        c.c_rv = 0.5 * kSqrt3 * (1 - 0.125 * xidt);
    }
}

__device__ __forceinline__ double friction(const Batch &B, const PropParams &P, int algo, int64_t k) {
    return algo == kPropLangevinConst ? P.gamma_const : B.dens[k];
}

__device__ bool all_xidt_big(const Batch &B, const PropParams &P, const TrajView &T, int i, int algo) {
    bool all_big = true;
    for (int b = 0; b < T.nb; ++b)
        if (!(friction(B, P, algo, T.base + (int64_t)b * T.N + i) * P.step > (double)1e-2f)) all_big = false;
    return all_big;
}

// langevin_1, md_algo.f90:146-232
__device__ void langevin_1(const Batch &B, const PropParams &P, const TrajView &T, int i, int step, int algo) {
    const int ty = B.type[T.aoff + i];
    const double temp = kBoltz * T.nb * temp_of(B, P, ty) / B.mass[T.aoff + i];
    const bool all_big = all_xidt_big(B, P, T, i, algo);
    for (int b = 0; b < T.nb; ++b) {
        const int slot = b * T.N + i;
        const int64_t k = T.base + slot;
        LangCoef c;
        langevin_coef(friction(B, P, algo, k), P.step, temp, all_big, false, c);
        const uint8_t fx = B.fixed[k];
        for (int d = 0; d < 3; ++d) {
            double &v = comp(B.vx, B.vy, B.vz, d, k);
            if (!(fx >> d & 1)) {
                const double rnd = rand_normal(P, T, step, b, i, d, kStreamLangevin, P.randy);
                const double a = comp(B.ax, B.ay, B.az, d, k);
                comp(B.rx, B.ry, B.rz, d, k) += c.c1 * v + c.c2 * P.step * a + c.sigma_r * rnd;
                v = c.c0 * v + (c.c1 - c.c2) * a + c.sigma_v * c.c_rv * rnd;
            } else {
                v = 0.0;
            }
        }
    }
}

// ldfa, md_algo.f90:506-570 -- dens(:,i) becomes the friction coefficient in place
__device__ bool ldfa(const Batch &B, const TrajView &T, int i) {
    const double coefs[12] = {0.0802484, -1.12851, 9.28508, 2.10064, -843.419, 8.85354e3, -4.89023e4,
                              1.6741e5, -3.67098e5, 5.03476e5, -3.9426e5, 1.34763e5};
    const double convert = 1.00794 * kAmu2Mass;
    const double m = B.mass[T.aoff + i];
    bool ok = true;
    for (int b = 0; b < T.nb; ++b) {
        const int64_t k = T.base + (int64_t)b * T.N + i;
        const double d0 = B.dens[k];
        double fric;
        if ((double)-1e-12f <= d0 && d0 <= (double)0.36f) {
            fric = 0.0;
            double temp = d0;
            for (int j = 0; j < 12; ++j) {
                fric = fric + coefs[j] * temp;
                temp = temp * d0;
            }
        } else if (d0 > (double)0.36f) {
            fric = 0.001 * (4.7131 - exp(-4.41305 * d0));
        } else {
            ok = false;
            fric = 0.0;
        }
        B.dens[k] = fric * convert / kHbar / m;
    }
    return ok;
}

// langevin_2, md_algo.f90:236-300
__device__ void langevin_2(const Batch &B, const PropParams &P, const TrajView &T, int i, int step, int algo) {
    const int ty = B.type[T.aoff + i];
    const double temp = kBoltz * T.nb * temp_of(B, P, ty) / B.mass[T.aoff + i];
    const bool all_big = all_xidt_big(B, P, T, i, algo);
    for (int b = 0; b < T.nb; ++b) {
        const int slot = b * T.N + i;
        const int64_t k = T.base + slot;
        LangCoef c;
        langevin_coef(friction(B, P, algo, k), P.step, temp, all_big, true, c);
        const uint8_t fx = B.fixed[k];
        const double sv = c.sigma_v * sqrt(1 - c.c_rv * c.c_rv);
        for (int d = 0; d < 3; ++d) {
            double &v = comp(B.vx, B.vy, B.vz, d, k);
            if (!(fx >> d & 1)) {
                const double rnd = rand_normal(P, T, step, b, i, d, kStreamLangevin, P.randy);
                v = v + c.c2 * comp(B.ax, B.ay, B.az, d, k) + sv * rnd;
            } else {
                v = 0.0;
            }
        }
    }
}

// andersen, md_algo.f90:402-432
__device__ void andersen(const Batch &B, const PropParams &P, const TrajView &T, int i, int step) {
    const int ty = B.type[T.aoff + i];
    const double ibetaN = T.nb * kBoltz * temp_of(B, P, ty);
    const double sd = sqrt(ibetaN / B.mass[T.aoff + i]);
    const double thr = P.step / P.andersen_time;
    for (int b = 0; b < T.nb; ++b) {
        const int slot = b * T.N + i;
        const int64_t k = T.base + slot;
        const double u = P.rng_mode == 1 ? P.andersen_u[T.base + (int64_t)i * T.nb + b]
                                         : uniform_deviate(P.seed, (uint32_t)T.t, (uint32_t)step, (uint32_t)slot,
                                                           kStreamAndersenU);
        if (u < thr) {
            const uint8_t fx = B.fixed[k];
            for (int d = 0; d < 3; ++d)
                if (!(fx >> d & 1))
                    comp(B.vx, B.vy, B.vz, d, k) =
                        rand_normal(P, T, step, b, i, d, kStreamAndersenV, P.andersen_v) * sd;
        }
    }
}

// pile_thermostat, md_algo.f90:440-502 (one thread per atom, all three dimensions)
__device__ void pile(const Batch &B, const PropParams &P, const TrajView &T, const double *cjk, int i, int step) {
    const int nb = T.nb;
    const int ty = B.type[T.aoff + i];
    const double m = B.mass[T.aoff + i];
    const double betaN = 1.0 / (kBoltz * temp_of(B, P, ty) * nb);
    const double sq = sqrt(m / betaN);
    for (int d = 0; d < 3; ++d) {
        double newP[32], atomP[32];
        for (int b = 0; b < nb; ++b) atomP[b] = m * comp(B.vx, B.vy, B.vz, d, T.base + (int64_t)b * T.N + i);
        for (int b = 0; b < nb; ++b) {
            double s = 0.0;
            for (int k = 0; k < nb; ++k) s = s + atomP[k] * cjk[b * nb + k];  // cjk(k,b)
            newP[b] = s;
        }
        for (int kk = 0; kk < nb; ++kk) {
            double gam;
            if (kk == 0) gam = 1 / P.pile_tau;
            else gam = 2 * (2 * (1 / betaN / kHbar) * sin(kk * kPi / nb));
            const double c1 = exp(-0.5 * P.step * gam), c2 = sqrt(1 - c1 * c1);
            const double z = rand_normal(P, T, step, kk, i, d, kStreamPile, P.zeta);
            newP[kk] = c1 * newP[kk] + sq * c2 * z;
        }
        for (int b = 0; b < nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            double s = 0.0;
            if (!(B.fixed[k] >> d & 1))
                for (int kk = 0; kk < nb; ++kk) s = s + newP[kk] * cjk[kk * nb + b];  // cjk(b,kk)
            comp(B.vx, B.vy, B.vz, d, k) = s / m;
        }
    }
}

// remove_com_velocity, universe_mod.f90:222-241.  Its 1000 subtraction sweeps have the
// closed form v -= v_cm0 * N * (1 - (1 - 1/N)^1000), applied to every bead-atom.
__device__ void remove_com(const Batch &B, const TrajView &T, double *red) {
    double sx = 0, sy = 0, sz = 0, ms = 0;
    for (int i = threadIdx.x; i < T.N; i += blockDim.x) {
        const double m = B.mass[T.aoff + i];
        double ax = 0, ay = 0, az = 0;
        for (int b = 0; b < T.nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            ax += B.vx[k];
            ay += B.vy[k];
            az += B.vz[k];
        }
        sx += ax * m;
        sy += ay * m;
        sz += az * m;
        ms += m;
    }
    sx = block_sum(sx, red);
    sy = block_sum(sy, red);
    sz = block_sum(sz, red);
    ms = block_sum(ms, red);
    const double n = (double)T.N;
    const double fac = n * (1.0 - pow(1.0 - 1.0 / n, 1000.0));
    const double cx = sx / ms / T.nb / n * fac, cy = sy / ms / T.nb / n * fac, cz = sz / ms / T.nb / n * fac;
    const int tot = T.N * T.nb;
    for (int s = threadIdx.x; s < tot; s += blockDim.x) {
        const int64_t k = T.base + s;
        B.vx[k] -= cx;
        B.vy[k] -= cy;
        B.vz[k] -= cz;
    }
    __syncthreads();
}

__device__ bool traj_has_algo(const Batch &B, int id) {
    for (int ty = 0; ty < B.ntypes; ++ty)
        if (B.algo[ty] == id) return true;
    return false;
}

// propagate_1, md_algo.f90:37-76
__device__ void propagate_1(const Batch &B, const PropParams &P, const TrajView &T, const double *cjk, int step,
                            double *red) {
    for (int i = threadIdx.x; i < T.N; i += blockDim.x) {
        const int algo = B.algo[B.type[T.aoff + i]];
        switch (algo) {
            case kPropVerlet: verlet_half(B, P, T, i, true); break;
            case kPropAndersen:
                verlet_half(B, P, T, i, true);
                andersen(B, P, T, i, step);
                break;
            case kPropPile:
                pile(B, P, T, cjk, i, step);
                verlet_half(B, P, T, i, true);
                break;
            case kPropLangevin:
            case kPropLangevinConst: langevin_1(B, P, T, i, step, algo); break;
            default: break;
        }
    }
    __syncthreads();
    if (traj_has_algo(B, kPropAndersen) || traj_has_algo(B, kPropPile)) remove_com(B, T, red);
}

// propagate_2, md_algo.f90:80-106
__device__ void propagate_2(const Batch &B, const PropParams &P, const TrajView &T, int step) {
    bool bad = false;
    for (int i = threadIdx.x; i < T.N; i += blockDim.x) {
        const int algo = B.algo[B.type[T.aoff + i]];
        if (algo == kPropLangevin) {
            if (!ldfa(B, T, i)) bad = true;
            langevin_2(B, P, T, i, step, algo);
        } else if (algo == kPropLangevinConst) {
            langevin_2(B, P, T, i, step, algo);
        } else {
            verlet_half(B, P, T, i, false);
        }
    }
    if (bad) B.status[T.t] = kStatusErrDensity;
    __syncthreads();
}

// do_ring_polymer_step, rpmd.f90:309-452.  Thread per (atom, dimension).
__device__ void ring_polymer_step(const Batch &B, const PropParams &P, const TrajView &T, const double *cjk) {
    const int nb = T.nb;
    const double prefactor = -1 * B.mass[T.aoff] * pow(kBoltz * P.Tproj * nb / kHbar, 2.0);
    const double piN = kPi / nb;
    for (int w = threadIdx.x; w < 3 * T.N; w += blockDim.x) {
        const int i = w / 3, d = w - 3 * (w / 3);
        const int ty = B.type[T.aoff + i];
        const double m = B.mass[T.aoff + i];
        double p[32], q[32], np[32], nq[32];
        for (int b = 0; b < nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            p[b] = m * comp(B.vx, B.vy, B.vz, d, k);
            q[b] = comp(B.rx, B.ry, B.rz, d, k);
        }
        for (int b = 0; b < nb; ++b) {
            double sp = 0.0, sq = 0.0;
            for (int k = 0; k < nb; ++k) {
                sp = sp + p[k] * cjk[b * nb + k];
                sq = sq + q[k] * cjk[b * nb + k];
            }
            np[b] = sp;
            nq[b] = sq;
        }
        const double betaN = 1.0 / (kBoltz * temp_of(B, P, ty) * nb);
        const double twown = 2.0 / betaN / kHbar;
        for (int b = 0; b < nb; ++b) {
            double c0 = 1.0, c1 = 0.0, c2 = P.step / m, c3 = 1.0;
            if (nb > 1 && b > 0) {
                const int bb = (b <= nb / 2) ? b : nb - b;
                const double wk = twown * sin(bb * piN), wt = wk * P.step, wm = wk * m;
                const double cw = cos(wt), sw = sin(wt);
                c0 = cw; c1 = -wm * sw; c2 = sw / wm; c3 = cw;
            }
            const double pn = np[b] * c0 + nq[b] * c1;
            nq[b] = np[b] * c2 + nq[b] * c3;
            np[b] = pn;
        }
        const int algo = B.algo[ty];
        const bool revert = (algo == kPropLangevin || algo == kPropLangevinConst);
        for (int b = 0; b < nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            if (revert) continue;
            if (B.fixed[k] >> d & 1) continue;
            double sr = 0.0, sv = 0.0;
            for (int kk = 0; kk < nb; ++kk) {
                sr = sr + nq[kk] * cjk[kk * nb + b];
                sv = sv + np[kk] * cjk[kk * nb + b] / m;
            }
            comp(B.rx, B.ry, B.rz, d, k) = sr;
            comp(B.vx, B.vy, B.vz, d, k) = sv;
        }
        if (revert) {
            // rpmd.f90:418-435: positions/velocities kept, spring force set instead
            for (int b = 0; b < nb; ++b) {
                const int prev = (b == 0) ? nb - 1 : b - 1, next = (b == nb - 1) ? 0 : b + 1;
                const int64_t k = T.base + (int64_t)b * T.N + i;
                const double rb = q[b], rp = q[prev], rn = q[next];
                comp(B.fx, B.fy, B.fz, d, k) = prefactor * (2 * rb - rp - rn);
            }
        }
    }
    __syncthreads();
}

__device__ void load_cjk(const Batch &B, int t, double *cjk_s) {
    const int nb = B.nbeads[t];
    if (nb <= 1) return;
    const double *src = B.cjk + B.cjk_off[t];
    for (int k = threadIdx.x; k < nb * nb; k += blockDim.x) cjk_s[k] = src[k];
    __syncthreads();
}

// calc_force, force.f90:40-86, for trajectory t
template <typename R>
__device__ void calc_force(const Batch &B, const EmtConst &E, const PropParams &P, const SmemEmt<R> &S,
                           const TrajView &T, bool do_forces) {
    const int tot = T.N * T.nb;
    for (int s = threadIdx.x; s < tot; s += blockDim.x) {
        const int64_t k = T.base + s;
        B.fx[k] = 0.0; B.fy[k] = 0.0; B.fz[k] = 0.0;
        B.ax[k] = 0.0; B.ay[k] = 0.0; B.az[k] = 0.0;
    }
    for (int b = threadIdx.x; b < T.nb; b += blockDim.x) B.epot[B.bead_off[T.t] + b] = 0.0;
    __syncthreads();
    if (T.nb > 1) ring_polymer_step(B, P, T, S.cjk);
    for (int b = 0; b < T.nb; ++b) emt_bead<R>(B, E, S, T.t, b, do_forces);
    if (do_forces) {
        // set_acceleration, force.f90:89-98
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

__device__ __forceinline__ int next_work(int *counter, int *shared_slot) {
    if (threadIdx.x == 0) *shared_slot = atomicAdd(counter, 1);
    __syncthreads();
    const int w = *shared_slot;
    __syncthreads();
    return w;
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kBlock, 4) phase_kernel(Batch B, EmtConst E, PropParams P, const int *order,
                                                    int *counter, int phase) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    SmemEmt<R> S = carve_smem<R>(smem_raw, B.max_atoms, B.max_beads);
    for (;;) {
        const int w = next_work(counter, &work_slot);
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, S.cjk);
        const int step = B.steps_done[t] + 1;
        if (phase == kPhaseForce || phase == kPhaseEnergyOnly)
            calc_force<R>(B, E, P, S, T, phase == kPhaseForce);
        else if (phase == kPhaseProp1)
            propagate_1(B, P, T, S.cjk, step, S.red);
        else {
            propagate_2(B, P, T, step);
            if (threadIdx.x == 0) B.steps_done[t] = step;
            __syncthreads();
        }
    }
}

// Fused propagate_1 -> calc_force -> propagate_2 for nsteps steps per trajectory.
template <typename R>
__global__ void __launch_bounds__(kBlock, 4) md_steps_kernel(Batch B, EmtConst E, PropParams P, const int *order,
                                                       int *counter, int nsteps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    SmemEmt<R> S = carve_smem<R>(smem_raw, B.max_atoms, B.max_beads);
    for (;;) {
        const int w = next_work(counter, &work_slot);
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, S.cjk);
        const int ty0 = B.type[T.aoff];
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, S.cjk, step, S.red);
            calc_force<R>(B, E, P, S, T, true);
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

// Fortran-order host layout (3, nb, N) per trajectory <-> SoA device layout.
__global__ void unpack_kernel(Batch B, const double *src, double *x, double *y, double *z, int64_t total_ba,
                              const int *ba_traj) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total_ba;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[s];
        const int N = B.natoms[t];
        const int64_t loc = s - B.ba_off[t];
        const int b = (int)(loc / N), i = (int)(loc - (int64_t)b * N);
        const int64_t f = (B.ba_off[t] + (int64_t)i * B.nbeads[t] + b) * 3;
        x[s] = src[f];
        y[s] = src[f + 1];
        z[s] = src[f + 2];
    }
}

__global__ void pack_kernel(Batch B, double *dst, const double *x, const double *y, const double *z,
                            int64_t total_ba, const int *ba_traj) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total_ba;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[s];
        const int N = B.natoms[t];
        const int64_t loc = s - B.ba_off[t];
        const int b = (int)(loc / N), i = (int)(loc - (int64_t)b * N);
        const int64_t f = (B.ba_off[t] + (int64_t)i * B.nbeads[t] + b) * 3;
        dst[f] = x[s];
        dst[f + 1] = y[s];
        dst[f + 2] = z[s];
    }
}

// scalar per bead-atom (dens) in Fortran (nb, N) order
__global__ void pack_scalar_kernel(Batch B, double *dst, const double *x, int64_t total_ba, const int *ba_traj) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total_ba;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[s];
        const int N = B.natoms[t];
        const int64_t loc = s - B.ba_off[t];
        const int b = (int)(loc / N), i = (int)(loc - (int64_t)b * N);
        dst[B.ba_off[t] + (int64_t)i * B.nbeads[t] + b] = x[s];
    }
}

// Per-trajectory observables: mean bead epot, atom_ekin (universe_mod.f90:433-458) and
// the ring-polymer spring energy calc_bead_epot (rpmd.f90:244-267).  out: 5 per traj.
__global__ void summary_kernel(Batch B, PropParams P, double *out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double *red = (double *)smem_raw;
    for (int t = blockIdx.x; t < B.ntraj; t += gridDim.x) {
        const TrajView T = traj_view(B, t);
        double ep = 0.0, el = 0.0, eb = 0.0;
        for (int i = threadIdx.x; i < T.N; i += blockDim.x) {
            const int ty = B.type[T.aoff + i];
            const double m = B.mass[T.aoff + i];
            double sx = 0, sy = 0, sz = 0, spring = 0;
            for (int b = 0; b < T.nb; ++b) {
                const int64_t k = T.base + (int64_t)b * T.N + i;
                sx += B.vx[k];
                sy += B.vy[k];
                sz += B.vz[k];
                const int64_t k2 = T.base + (int64_t)((b + 1) % T.nb) * T.N + i;
                const double dx = B.rx[k] - B.rx[k2], dy = B.ry[k] - B.ry[k2], dz = B.rz[k] - B.rz[k2];
                spring += dx * dx + dy * dy + dz * dz;
            }
            const double nrg = m * (sx * sx + sy * sy + sz * sz);
            if (B.is_proj[ty]) ep += nrg; else el += nrg;
            if (T.nb > 1) {
                const double wn = kBoltz * temp_of(B, P, ty) * T.nb / kHbar;
                eb += m * spring * wn * wn;
            }
        }
        ep = block_sum(ep, red);
        el = block_sum(el, red);
        eb = block_sum(eb, red);
        double epot = 0.0;
        for (int b = 0; b < T.nb; ++b) epot += B.epot[B.bead_off[t] + b];
        if (threadIdx.x == 0) {
            out[5 * t + 0] = epot / T.nb;
            out[5 * t + 1] = 0.5 * ep / T.nb / T.nb;
            out[5 * t + 2] = 0.5 * el / T.nb / T.nb;
            out[5 * t + 3] = 0.5 * eb / T.nb;
            out[5 * t + 4] = (double)B.steps_done[t];
        }
        __syncthreads();
    }
}

cudaError_t launch_summary(cudaStream_t s, const Batch &B, const PropParams &P, double *out5) {
    const int grid = B.ntraj < 4096 ? (B.ntraj > 0 ? B.ntraj : 1) : 4096;
    summary_kernel<<<grid, 128, 64 * sizeof(double), s>>>(B, P, out5);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <typename R>
static cudaError_t launch_phase_t(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P,
                                  int phase) {
    const size_t sm = smem_bytes(B.max_atoms, B.max_beads, sizeof(R));
    cudaError_t e = cudaFuncSetAttribute(phase_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    phase_kernel<R><<<c.grid, kBlock, sm, c.stream>>>(B, E, P, c.order, c.counter, phase);
    return cudaGetLastError();
}

cudaError_t launch_phase(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P, int phase,
                         int precision) {
    return precision == 1 ? launch_phase_t<float>(c, B, E, P, phase) : launch_phase_t<double>(c, B, E, P, phase);
}

template <typename R>
static cudaError_t launch_md_t(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P,
                               int nsteps) {
    const size_t sm = smem_bytes(B.max_atoms, B.max_beads, sizeof(R));
    cudaError_t e = cudaFuncSetAttribute(md_steps_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    md_steps_kernel<R><<<c.grid, kBlock, sm, c.stream>>>(B, E, P, c.order, c.counter, nsteps);
    return cudaGetLastError();
}

cudaError_t launch_md_steps(const LaunchCfg &c, const Batch &B, const EmtConst &E, const PropParams &P, int nsteps,
                            int precision) {
    return precision == 1 ? launch_md_t<float>(c, B, E, P, nsteps) : launch_md_t<double>(c, B, E, P, nsteps);
}

cudaError_t launch_unpack(cudaStream_t s, const Batch &B, const double *src, double *x, double *y, double *z,
                          int64_t total_ba, const int *ba_traj) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    unpack_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(B, src, x, y, z, total_ba, ba_traj);
    return cudaGetLastError();
}

cudaError_t launch_pack(cudaStream_t s, const Batch &B, double *dst, const double *x, const double *y,
                        const double *z, int64_t total_ba, const int *ba_traj) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    pack_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(B, dst, x, y, z, total_ba, ba_traj);
    return cudaGetLastError();
}

cudaError_t launch_pack_scalar(cudaStream_t s, const Batch &B, double *dst, const double *x, int64_t total_ba,
                               const int *ba_traj) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    pack_scalar_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(B, dst, x, total_ba, ba_traj);
    return cudaGetLastError();
}

int max_resident_ctas(int max_atoms, int max_beads, int precision) {
    const size_t sm = smem_bytes(max_atoms, max_beads, precision == 1 ? 4 : 8);
    int n = 0;
    if (precision == 1) {
        cudaFuncSetAttribute(md_steps_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, md_steps_kernel<float>, kBlock, sm);
    } else {
        cudaFuncSetAttribute(md_steps_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, md_steps_kernel<double>, kBlock, sm);
    }
    return n > 0 ? n : 1;
}

}  // namespace mdt
