// mdt_acsf.cuh -- atom-centred symmetry functions as CTA/warp device functions, shared by
// the HDNNP/surrogate force kernels (mdt_nn.cu) and the training kernels (mdt_train.cu).
//
// One warp owns one central atom i.  Its neighbour cache (per neighbour q: the vector
// d_q = x_q - x_i, r_q, fc(r_q), dfc/dr(r_q) and exp(-eta r_q^2) for every distinct G3 eta
// of the element) lives in the warp's shared memory.  Triplets (j<k) are walked with a
// lane-strided flat index over the upper triangle.  Three walks exist:
//   forward  G_s                         (atomsymfunction2.f90:80-170, atomsymfunction3Andi.f90:90-257)
//   VJP      F -= sum_s c_s dG_s/dx       (forces from c_s = dE/dG_s)
//   JVP      v_s = sum_k u_k . (-dG_s/dx_k) (the force-loss adjoint for training)
// The G3 derivative factors p1, p2, p3 are those of atomsymfunction3Andi.f90:209-222.
// For the VJP they are summed over functions in factored form: with
// u_s = c_s 2^(1-zeta) (1+lambda cos)^(zeta-1) exp(-eta sum r^2),
//   P1 = pfc (1/(r_ij r_ik) - cos/r_ij^2) A1 - 2 pfc A2 + fc_ik fc_jk dfc_ij/r_ij A3
//   P2 = pfc (1/(r_ij r_ik) - cos/r_ik^2) A1 - 2 pfc A2 + fc_ij fc_jk dfc_ik/r_ik A3
//   P3 = pfc/(r_ij r_ik) A1 + 2 pfc A2 - fc_ij fc_ik dfc_jk/r_jk A3
// where A1 = sum u_s zeta_s lambda_s, A2 = sum u_s eta_s (1+lambda_s cos), A3 = sum u_s (1+lambda_s cos):
// three multiply-adds per function and triplet instead of three full derivative factors.
#pragma once
#include "mdt_common.cuh"
#include "mdt_nn.cuh"

namespace mdt {

constexpr int kMaxG3 = 24;  // G3 functions per element held in lane registers
constexpr double kAng2BohrD = 1.0 / kBohr2Ang;

template <typename R> struct WarpCache {
    R *nb;          // [q][stride]
    R *slotf;       // [q][3]
    int *nbatom;    // [q]
    int8_t *nbelem; // [q]
    int st;
};

template <typename R> __device__ __forceinline__ R warp_sum(R v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Triangle walk over neighbour pairs (q3 < q4): lane-strided flat index, advanced by 32
// pairs per iteration without a square-root decode.
struct TriWalk {
    int q3, q4, n;
    bool valid;
    __device__ __forceinline__ void init(int cnt, int lane) {
        n = cnt;
        q3 = 0;
        q4 = 1 + lane;
        normalize();
    }
    __device__ __forceinline__ void normalize() {
        while (q3 < n - 1 && q4 >= n) {
            const int over = q4 - n;
            ++q3;
            q4 = q3 + 1 + over;
        }
        valid = q3 < n - 1 && q4 < n;
    }
    __device__ __forceinline__ void next() {
        q4 += 32;
        normalize();
    }
};

// Balanced row walk over the same triangle: lane L owns the row pairs (r, nrows-1-r)
// for r = L, L+32, ...; each pair holds cnt pairs (q3, q4) in total, so every lane runs
// the same number of iterations, and because a lane keeps its row q3 for many
// iterations, the q3 side of a triplet can be accumulated in registers (flushed when
// the row changes) while the q4 sides of the 32 lanes are distinct atoms.
struct RowWalk {
    int cnt, nrows, p, it, len0, q3, q4;
    bool valid, row_end;  // row_end: q3 changes after this triplet
    __device__ __forceinline__ void init(int c, int lane) {
        cnt = c;
        nrows = c - 1;
        p = lane;
        start();
    }
    __device__ __forceinline__ void start() {
        it = 0;
        const int npairs = (nrows + 1) / 2;
        valid = p < npairs;
        if (!valid) return;
        len0 = nrows - p;  // row p holds q4 = p+1 .. cnt-1
        set();
    }
    __device__ __forceinline__ int total() const { return (nrows - 1 - p == p) ? len0 : cnt; }
    __device__ __forceinline__ void set() {
        if (it < len0) {
            q3 = p;
            q4 = p + 1 + it;
        } else {
            q3 = nrows - 1 - p;
            q4 = q3 + 1 + (it - len0);
        }
        row_end = (it == len0 - 1) || (it == total() - 1);
    }
    __device__ __forceinline__ void next() {
        ++it;
        if (it >= total()) {
            p += 32;
            start();
            return;
        }
        set();
    }
};

__device__ __forceinline__ int pack_nb(int j, int n1, int n2, int n3) {
    return j | ((n1 + 8) << 16) | ((n2 + 8) << 20) | ((n3 + 8) << 24);
}

// lattice rows (bohr) and the inverse of the column matrix, without fused operations so
// that the cell folding matches the oracle bit for bit.  box: 9 doubles column major (A).
static __device__ void acsf_lattice(const double *bx, double *lat) {
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) lat[3 * i + k] = __dmul_rn(bx[3 * i + k], kAng2BohrD);
    double A[9];
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) A[k * 3 + i] = lat[3 * i + k];
    double *I = lat + 9;
    auto m = [](double a, double b2) { return __dmul_rn(a, b2); };
    auto sb = [](double a, double b2) { return __dsub_rn(a, b2); };
    const double det = __dadd_rn(__dsub_rn(m(A[0], sb(m(A[4], A[8]), m(A[5], A[7]))),
                                            m(A[1], sb(m(A[3], A[8]), m(A[5], A[6])))),
                                 m(A[2], sb(m(A[3], A[7]), m(A[4], A[6]))));
    I[0] = __ddiv_rn(sb(m(A[4], A[8]), m(A[5], A[7])), det);
    I[1] = __ddiv_rn(sb(m(A[2], A[7]), m(A[1], A[8])), det);
    I[2] = __ddiv_rn(sb(m(A[1], A[5]), m(A[2], A[4])), det);
    I[3] = __ddiv_rn(sb(m(A[5], A[6]), m(A[3], A[8])), det);
    I[4] = __ddiv_rn(sb(m(A[0], A[8]), m(A[2], A[6])), det);
    I[5] = __ddiv_rn(sb(m(A[2], A[3]), m(A[0], A[5])), det);
    I[6] = __ddiv_rn(sb(m(A[3], A[7]), m(A[4], A[6])), det);
    I[7] = __ddiv_rn(sb(m(A[1], A[6]), m(A[0], A[7])), det);
    I[8] = __ddiv_rn(sb(m(A[0], A[4]), m(A[1], A[3])), det);
}

// positions A -> bohr, folded into the cell (RuNNer_src/translate.f90)
static __device__ __forceinline__ void acsf_wrap_one(double xa, double ya, double za, const double *lat, double &x,
                                                     double &y, double &z) {
    x = __dmul_rn(xa, kAng2BohrD);
    y = __dmul_rn(ya, kAng2BohrD);
    z = __dmul_rn(za, kAng2BohrD);
    const double *I = lat + 9;
    double f[3];
    for (int d = 0; d < 3; ++d)
        f[d] = __dadd_rn(__dadd_rn(__dmul_rn(I[3 * d], x), __dmul_rn(I[3 * d + 1], y)), __dmul_rn(I[3 * d + 2], z));
    for (int d = 0; d < 3; ++d) {
        const double s = floor(f[d]);
        if (s != 0.0) {
            x = __dsub_rn(x, __dmul_rn(s, lat[3 * d]));
            y = __dsub_rn(y, __dmul_rn(s, lat[3 * d + 1]));
            z = __dsub_rn(z, __dmul_rn(s, lat[3 * d + 2]));
        }
    }
}

// neighbour list of atom i in RuNNer's order (neighbor_para_short.f90:117-163).
// Returns the count (may exceed maxnb: the caller flags the overflow).
static __device__ int acsf_neighbors_one(const NNDev &M, int i, int N, const double *px, const double *py,
                                         const double *pz, const double *L, int na, int nbi, int nc, int *out) {
    const double cut2 = __dmul_rn(M.maxcut, M.maxcut);
    const float cut2f_hi = (float)cut2 * 1.0001f, cut2f_lo = (float)cut2 * 0.9999f;
    int cnt = 0;
    const double xi = px[i], yi = py[i], zi = pz[i];
    for (int j = 0; j < N; ++j) {
        const double xj = px[j], yj = py[j], zj = pz[j];
        for (int n1 = -na; n1 <= na; ++n1)
            for (int n2 = -nbi; n2 <= nbi; ++n2)
                for (int n3 = -nc; n3 <= nc; ++n3) {
                    if (n1 == 0 && n2 == 0 && n3 == 0 && i == j) continue;
                    const double d1n = n1, d2n = n2, d3n = n3;
                    // FP32 screen; the exact FP64 test (the oracle's operation order, no
                    // fused multiply-add) only within 1e-4 (relative) of the cutoff
                    const float fx = (float)(xj - xi) + (float)d1n * (float)L[0] + (float)d2n * (float)L[3] +
                                     (float)d3n * (float)L[6];
                    const float fy = (float)(yj - yi) + (float)d1n * (float)L[1] + (float)d2n * (float)L[4] +
                                     (float)d3n * (float)L[7];
                    const float fz = (float)(zj - zi) + (float)d1n * (float)L[2] + (float)d2n * (float)L[5] +
                                     (float)d3n * (float)L[8];
                    const float rf = fx * fx + fy * fy + fz * fz;
                    if (rf > cut2f_hi) continue;
                    if (rf < cut2f_lo) {
                        if (cnt < M.maxnb) out[cnt] = pack_nb(j, n1, n2, n3);
                        ++cnt;
                        continue;
                    }
                    const double xt = __dadd_rn(__dadd_rn(__dadd_rn(xj, __dmul_rn(d1n, L[0])), __dmul_rn(d2n, L[3])),
                                                __dmul_rn(d3n, L[6]));
                    const double yt = __dadd_rn(__dadd_rn(__dadd_rn(yj, __dmul_rn(d1n, L[1])), __dmul_rn(d2n, L[4])),
                                                __dmul_rn(d3n, L[7]));
                    const double zt = __dadd_rn(__dadd_rn(__dadd_rn(zj, __dmul_rn(d1n, L[2])), __dmul_rn(d2n, L[5])),
                                                __dmul_rn(d3n, L[8]));
                    const double e1 = __dsub_rn(xt, xi), e2 = __dsub_rn(yt, yi), e3 = __dsub_rn(zt, zi);
                    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(e1, e1), __dmul_rn(e2, e2)), __dmul_rn(e3, e3));
                    if (rr <= cut2) {
                        if (cnt < M.maxnb) out[cnt] = pack_nb(j, n1, n2, n3);
                        ++cnt;
                    }
                }
    }
    return cnt;
}

// neighbour cache of central atom i for its warp
template <typename R>
__device__ void acsf_cache(const NNDev &M, const WarpCache<R> &C, int i, int ei, int cnt, const int *words,
                           const double *px, const double *py, const double *pz, const int8_t *elem, const double *L) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const int ng = M.ng3eta[ei];
    for (int q = lane; q < cnt; q += 32) {
        const int w = words[q];
        const int j = w & 0xFFFF;
        const double n1 = ((w >> 16) & 15) - 8, n2 = ((w >> 20) & 15) - 8, n3 = ((w >> 24) & 15) - 8;
        const double dx = px[j] + n1 * L[0] + n2 * L[3] + n3 * L[6] - px[i];
        const double dy = py[j] + n1 * L[1] + n2 * L[4] + n3 * L[7] - py[i];
        const double dz = pz[j] + n1 * L[2] + n2 * L[5] + n3 * L[8] - pz[i];
        const R r = (R)sqrt(dx * dx + dy * dy + dz * dz);
        R *e = C.nb + q * C.st;
        e[0] = (R)dx;
        e[1] = (R)dy;
        e[2] = (R)dz;
        e[3] = r;
        R fc = R(0), dfc = R(0);
        if (r <= rc) cutoff_fn<R>(M, rc, r, fc, dfc);
        e[4] = fc;
        e[5] = dfc;
        for (int m = 0; m < ng; ++m) e[6 + m] = NM<R>::ex(-(R)M.g3eta[ei][m] * r * r);
        C.nbatom[q] = j;
        C.nbelem[q] = elem[j];
        C.slotf[3 * q] = R(0);
        C.slotf[3 * q + 1] = R(0);
        C.slotf[3 * q + 2] = R(0);
    }
    __syncwarp();
}

// G3 functions of an element, in SF order
struct G3List {
    int n;
    int idx[kMaxG3];
};

__device__ __forceinline__ G3List g3_list(const NNDev &M, int ei) {
    G3List g;
    g.n = 0;
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    for (int s = 0; s < nsf && g.n < kMaxG3; ++s)
        if (M.sftype[sfb + s] == 3) g.idx[g.n++] = s;
    return g;
}

// Per-triplet geometry shared by the three walks.
template <typename R> struct Triplet {
    const R *a, *c;  // cache rows of j and k
    R jx, jy, jz;    // d_j - d_k = x_j - x_k
    R rjk2, rjk, fcjk, dfcjk, rinv0, cost0, pfc;
    R ejk[kMaxEta];
};

template <typename R>
__device__ __forceinline__ bool triplet_setup(const NNDev &M, const WarpCache<R> &C, int ei, int q3, int q4, R rc,
                                              Triplet<R> &T) {
    T.a = C.nb + q3 * C.st;
    T.c = C.nb + q4 * C.st;
    if (!(T.a[3] <= rc && T.c[3] <= rc)) return false;
    T.jx = T.a[0] - T.c[0];
    T.jy = T.a[1] - T.c[1];
    T.jz = T.a[2] - T.c[2];
    T.rjk2 = T.jx * T.jx + T.jy * T.jy + T.jz * T.jz;
    if (!(T.rjk2 <= rc * rc)) return false;
    T.rjk = NM<R>::sq(T.rjk2);
    cutoff_fn<R>(M, rc, T.rjk, T.fcjk, T.dfcjk);
    T.rinv0 = R(1) / (T.a[3] * T.c[3]);
    T.cost0 = (T.a[0] * T.c[0] + T.a[1] * T.c[1] + T.a[2] * T.c[2]) * T.rinv0;
    T.pfc = T.a[4] * T.c[4] * T.fcjk;
    const int ng = M.ng3eta[ei];
    for (int m = 0; m < ng; ++m) T.ejk[m] = NM<R>::ex(-(R)M.g3eta[ei][m] * T.rjk2);
    return true;
}

__device__ __forceinline__ bool g3_match(const NNDev &M, int k, int ej, int ek) {
    const int e1 = M.e1[k], e2 = M.e2[k];
    return (e1 == ej && e2 == ek) || (e2 == ej && e1 == ek);
}

// (1 + lambda cos)^(zeta-1) exp(-eta sum r^2) 2^(1-zeta); returns false when 1+lambda cos <= 0
template <typename R>
__device__ __forceinline__ bool g3_term(const NNDev &M, int k, const Triplet<R> &T, R &plam, R &fgn) {
    plam = R(1) + (R)M.lam[k] * T.cost0;
    if (plam <= R(0)) return false;
    const int m = M.etaslot[k];
    const R pexp = T.a[6 + m] * T.c[6 + m] * T.ejk[m];
    const int iz = M.izeta[k];
    fgn = (iz >= 0 ? ipow<R>(plam, iz) : NM<R>::pw(plam, (R)M.zeta[k] - R(1))) * pexp * (R)M.pnorm[k];
    return true;
}

// grid-form G3 walks, defined at the end of this file
template <typename R> __device__ void acsf_g3_forward_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt,
                                                           R *G);
template <typename R>
__device__ void acsf_g3_vjp_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, const R *c, R &fix, R &fiy,
                                 R &fiz);
template <typename R>
__device__ void acsf_g3_jvp_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, int i, const R *ux,
                                 const R *uy, const R *uz, R *v);

// ---- forward ------------------------------------------------------------------------
template <typename R> __device__ void acsf_forward(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, R *G) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    for (int s = 0; s < nsf; ++s) {
        if (M.sftype[sfb + s] != 2) continue;
        const R eta = (R)M.eta[sfb + s], rs = (R)M.rs[sfb + s];
        const int e1 = M.e1[sfb + s];
        R acc = R(0);
        for (int q = lane; q < cnt; q += 32) {
            const R *e = C.nb + q * C.st;
            if (C.nbelem[q] != e1 || !(e[3] <= rc)) continue;
            acc += NM<R>::ex(-eta * (e[3] - rs) * (e[3] - rs)) * e[4];
        }
        acc = warp_sum(acc);
        if (lane == 0) G[s] = acc;
    }
    if (M.g3fast[ei]) {
        acsf_g3_forward_fast<R>(M, C, ei, cnt, G);
        return;
    }
    const G3List g3 = g3_list(M, ei);
    R acc[kMaxG3];
#pragma unroll
    for (int u = 0; u < kMaxG3; ++u) acc[u] = R(0);
    TriWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (triplet_setup<R>(M, C, ei, tw.q3, tw.q4, rc, T)) {
            const int ej = C.nbelem[tw.q3], ek = C.nbelem[tw.q4];
#pragma unroll
            for (int u = 0; u < kMaxG3; ++u) {
                if (u >= g3.n) break;
                const int k = sfb + g3.idx[u];
                if (!g3_match(M, k, ej, ek)) continue;
                R plam, fgn;
                if (g3_term<R>(M, k, T, plam, fgn)) acc[u] += fgn * plam * T.pfc;
            }
        }
        tw.next();
    }
#pragma unroll
    for (int u = 0; u < kMaxG3; ++u) {
        if (u >= g3.n) break;
        const R v = warp_sum(acc[u]);
        if (lane == 0) G[g3.idx[u]] = v;
    }
    __syncwarp();
}

// ---- VJP: slot forces -= c . dG/dx; returns the central atom's force (all lanes) --------
template <typename R>
__device__ void acsf_vjp(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, const R *c, R &fix, R &fiy,
                         R &fiz) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    fix = fiy = fiz = R(0);
    for (int q = lane; q < cnt; q += 32) {
        const R *e = C.nb + q * C.st;
        if (!(e[3] <= rc)) continue;
        R dsum = R(0);
        for (int s = 0; s < nsf; ++s) {
            if (M.sftype[sfb + s] != 2 || C.nbelem[q] != M.e1[sfb + s]) continue;
            const R eta = (R)M.eta[sfb + s], rs = (R)M.rs[sfb + s];
            const R ex = NM<R>::ex(-eta * (e[3] - rs) * (e[3] - rs));
            dsum += c[s] * (R(-2) * eta * (e[3] - rs) * ex * e[4] + ex * e[5]);
        }
        const R fr = dsum / e[3];
        C.slotf[3 * q] -= fr * e[0];
        C.slotf[3 * q + 1] -= fr * e[1];
        C.slotf[3 * q + 2] -= fr * e[2];
        fix += fr * e[0];
        fiy += fr * e[1];
        fiz += fr * e[2];
    }
    __syncwarp();
    if (M.g3fast[ei]) {
        acsf_g3_vjp_fast<R>(M, C, ei, cnt, c, fix, fiy, fiz);
        __syncwarp();
        fix = warp_sum(fix);
        fiy = warp_sum(fiy);
        fiz = warp_sum(fiz);
        return;
    }
    const G3List g3 = g3_list(M, ei);
    TriWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (triplet_setup<R>(M, C, ei, tw.q3, tw.q4, rc, T)) {
            const int ej = C.nbelem[tw.q3], ek = C.nbelem[tw.q4];
            R A1 = R(0), A2 = R(0), A3 = R(0);
            for (int u = 0; u < g3.n; ++u) {
                const int s = g3.idx[u], k = sfb + s;
                if (!g3_match(M, k, ej, ek)) continue;
                R plam, fgn;
                if (!g3_term<R>(M, k, T, plam, fgn)) continue;
                const R us = c[s] * fgn;
                A1 += us * (R)(M.zeta[k] * M.lam[k]);
                A2 += us * (R)M.eta[k] * plam;
                A3 += us * plam;
            }
            const R rij = T.a[3], rik = T.c[3];
            const R P1 = T.pfc * (T.rinv0 - T.cost0 / (rij * rij)) * A1 - R(2) * T.pfc * A2 +
                         T.c[4] * T.fcjk * T.a[5] / rij * A3;
            const R P2 = T.pfc * (T.rinv0 - T.cost0 / (rik * rik)) * A1 - R(2) * T.pfc * A2 +
                         T.a[4] * T.fcjk * T.c[5] / rik * A3;
            const R P3 = T.pfc * T.rinv0 * A1 + R(2) * T.pfc * A2 - T.a[4] * T.c[4] * T.dfcjk / T.rjk * A3;
            // dxij = -a, dxik = -c, dxjk = a - c (atomsymfunction3Andi.f90:225-244):
            // F_i -= dxij P1 + dxik P2 ; F_j -= -dxij P1 - dxjk P3 ; F_k -= -dxik P2 + dxjk P3
            fix += T.a[0] * P1 + T.c[0] * P2;
            fiy += T.a[1] * P1 + T.c[1] * P2;
            fiz += T.a[2] * P1 + T.c[2] * P2;
            atomicAdd(&C.slotf[3 * tw.q3], -T.a[0] * P1 + T.jx * P3);
            atomicAdd(&C.slotf[3 * tw.q3 + 1], -T.a[1] * P1 + T.jy * P3);
            atomicAdd(&C.slotf[3 * tw.q3 + 2], -T.a[2] * P1 + T.jz * P3);
            atomicAdd(&C.slotf[3 * tw.q4], -T.c[0] * P2 - T.jx * P3);
            atomicAdd(&C.slotf[3 * tw.q4 + 1], -T.c[1] * P2 - T.jy * P3);
            atomicAdd(&C.slotf[3 * tw.q4 + 2], -T.c[2] * P2 - T.jz * P3);
        }
        tw.next();
    }
    __syncwarp();
    fix = warp_sum(fix);
    fiy = warp_sum(fiy);
    fiz = warp_sum(fiz);
}

// ---- JVP: v_s = sum_k u_k . (-dG_s/dx_k); lane 0 writes v[s] -------------------------
template <typename R>
__device__ void acsf_jvp(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, int i, const R *ux, const R *uy,
                         const R *uz, R *v) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
    const R uix = ux[i], uiy = uy[i], uiz = uz[i];
    // G2: -dG/dx_i = (d/r) T', -dG/dx_j = -(d/r) T'  ->  v += T'/r d.(u_i - u_j)
    for (int s = 0; s < nsf; ++s) {
        if (M.sftype[sfb + s] != 2) continue;
        const R eta = (R)M.eta[sfb + s], rs = (R)M.rs[sfb + s];
        const int e1 = M.e1[sfb + s];
        R acc = R(0);
        for (int q = lane; q < cnt; q += 32) {
            const R *e = C.nb + q * C.st;
            if (C.nbelem[q] != e1 || !(e[3] <= rc)) continue;
            const int j = C.nbatom[q];
            const R ex = NM<R>::ex(-eta * (e[3] - rs) * (e[3] - rs));
            const R dt = R(-2) * eta * (e[3] - rs) * ex * e[4] + ex * e[5];
            acc += dt / e[3] * (e[0] * (uix - ux[j]) + e[1] * (uiy - uy[j]) + e[2] * (uiz - uz[j]));
        }
        acc = warp_sum(acc);
        if (lane == 0) v[s] = acc;
    }
    if (M.g3fast[ei]) {
        acsf_g3_jvp_fast<R>(M, C, ei, cnt, i, ux, uy, uz, v);
        return;
    }
    const G3List g3 = g3_list(M, ei);
    R acc[kMaxG3];
#pragma unroll
    for (int u = 0; u < kMaxG3; ++u) acc[u] = R(0);
    TriWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (triplet_setup<R>(M, C, ei, tw.q3, tw.q4, rc, T)) {
            const int ej = C.nbelem[tw.q3], ek = C.nbelem[tw.q4];
            const int j = C.nbatom[tw.q3], kk = C.nbatom[tw.q4];
            // q1 = dxij.(u_i-u_j), q2 = dxik.(u_i-u_k), q3 = dxjk.(u_k-u_j)
            const R q1 = -(T.a[0] * (uix - ux[j]) + T.a[1] * (uiy - uy[j]) + T.a[2] * (uiz - uz[j]));
            const R q2 = -(T.c[0] * (uix - ux[kk]) + T.c[1] * (uiy - uy[kk]) + T.c[2] * (uiz - uz[kk]));
            const R q3 = T.jx * (ux[kk] - ux[j]) + T.jy * (uy[kk] - uy[j]) + T.jz * (uz[kk] - uz[j]);
            const R rij = T.a[3], rik = T.c[3];
            const R b1 = T.pfc * (T.rinv0 - T.cost0 / (rij * rij)), b2 = T.pfc * (T.rinv0 - T.cost0 / (rik * rik));
            const R d1 = T.c[4] * T.fcjk * T.a[5] / rij, d2 = T.a[4] * T.fcjk * T.c[5] / rik;
            const R d3 = T.a[4] * T.c[4] * T.dfcjk / T.rjk;
#pragma unroll
            for (int u = 0; u < kMaxG3; ++u) {
                if (u >= g3.n) break;
                const int k = sfb + g3.idx[u];
                if (!g3_match(M, k, ej, ek)) continue;
                R plam, fgn;
                if (!g3_term<R>(M, k, T, plam, fgn)) continue;
                const R zl = (R)(M.zeta[k] * M.lam[k]), e2 = R(2) * (R)M.eta[k] * plam * T.pfc;
                const R p1 = fgn * (b1 * zl - e2 + d1 * plam);
                const R p2 = fgn * (b2 * zl - e2 + d2 * plam);
                const R p3 = fgn * (T.pfc * T.rinv0 * zl + e2 - d3 * plam);
                acc[u] -= p1 * q1 + p2 * q2 + p3 * q3;
            }
        }
        tw.next();
    }
#pragma unroll
    for (int u = 0; u < kMaxG3; ++u) {
        if (u >= g3.n) break;
        const R val = warp_sum(acc[u]);
        if (lane == 0) v[g3.idx[u]] = val;
    }
    __syncwarp();
}

// ---------------------------------------------------------------------------
// Grid form of the G3 functions (NNDev::g3fast): cells (eta slot m, (lambda, zeta)
// slot q) share one neighbour pair; per triplet the ng exponentials and nlz angular
// powers meet in an outer product accumulated in registers.
// ---------------------------------------------------------------------------
constexpr int kGM = 4, kGQ = 8;

__device__ __forceinline__ bool fast_pair(const NNDev &M, int ei, int ej, int ek) {
    const int p1 = M.g3pair[ei][0], p2 = M.g3pair[ei][1];
    return (p1 == ej && p2 == ek) || (p2 == ej && p1 == ek);
}

// geometry of a triplet without the per-eta exponentials (computed by the caller)
template <typename R>
__device__ __forceinline__ bool triplet_geom(const NNDev &M, const WarpCache<R> &C, int q3, int q4, R rc,
                                             Triplet<R> &T) {
    T.a = C.nb + q3 * C.st;
    T.c = C.nb + q4 * C.st;
    if (!(T.a[3] <= rc && T.c[3] <= rc)) return false;
    T.jx = T.a[0] - T.c[0];
    T.jy = T.a[1] - T.c[1];
    T.jz = T.a[2] - T.c[2];
    T.rjk2 = T.jx * T.jx + T.jy * T.jy + T.jz * T.jz;
    if (!(T.rjk2 <= rc * rc)) return false;
    T.rjk = NM<R>::sq(T.rjk2);
    cutoff_fn<R>(M, rc, T.rjk, T.fcjk, T.dfcjk);
    T.rinv0 = R(1) / (T.a[3] * T.c[3]);
    T.cost0 = (T.a[0] * T.c[0] + T.a[1] * T.c[1] + T.a[2] * T.c[2]) * T.rinv0;
    T.pfc = T.a[4] * T.c[4] * T.fcjk;
    return true;
}

template <typename R> struct GridConst {
    R lam[kGQ], zl[kGQ], pn[kGQ], eta[kGM];
    int zm1[kGQ];
    int lidx[kGQ];   // which distinct lambda (0/1) the cell uses
    R lams[2];
    int ng, nq, nl;
};

// (1 + lambda cos) for the (at most two) distinct lambdas and its squaring ladder
// p, p^2, p^4, p^8, p^16, from which every integer power up to 31 is a product.
template <typename R> struct Ladder {
    R pw[2][5];
    bool pos[2];
};

template <typename R>
__device__ __forceinline__ void ladder_make(const GridConst<R> &g, R cost, Ladder<R> &L) {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        const R p = R(1) + g.lams[l] * cost;
        L.pos[l] = (l < g.nl) && (p > R(0));
        L.pw[l][0] = p;
#pragma unroll
        for (int b = 1; b < 5; ++b) L.pw[l][b] = L.pw[l][b - 1] * L.pw[l][b - 1];
    }
}

template <typename R> __device__ __forceinline__ R ladder_pow(const Ladder<R> &L, int l, int e) {
    R r = R(1);
#pragma unroll
    for (int b = 0; b < 5; ++b) r *= ((e >> b) & 1) ? L.pw[l][b] : R(1);
    return r;
}

template <typename R> __device__ __forceinline__ GridConst<R> grid_const(const NNDev &M, int ei) {
    GridConst<R> g;
    g.ng = M.ng3eta[ei];
    g.nq = M.nlz[ei];
#pragma unroll
    for (int q = 0; q < kGQ; ++q) {
        g.lam[q] = (R)M.lz_lam[ei][q];
        g.zl[q] = (R)M.lz_zl[ei][q];
        g.pn[q] = (R)M.lz_pnorm[ei][q];
        g.zm1[q] = M.lz_zm1[ei][q];
    }
#pragma unroll
    for (int m = 0; m < kGM; ++m) g.eta[m] = (R)(m < g.ng ? M.g3eta[ei][m] : 0.0);
    g.nl = 0;
    g.lams[0] = g.lams[1] = R(0);
#pragma unroll
    for (int q = 0; q < kGQ; ++q) {
        g.lidx[q] = 0;
        if (q >= g.nq) continue;
        if (g.nl > 0 && g.lams[0] == g.lam[q]) g.lidx[q] = 0;
        else if (g.nl > 1 && g.lams[1] == g.lam[q]) g.lidx[q] = 1;
        else if (g.nl < 2) { g.lams[g.nl] = g.lam[q]; g.lidx[q] = g.nl; ++g.nl; }
    }
    return g;
}

// exp(-eta_m (r_ij^2 + r_ik^2 + r_jk^2)) for every eta slot
template <typename R>
__device__ __forceinline__ void grid_pexp(const GridConst<R> &g, const Triplet<R> &T, R *E) {
#pragma unroll
    for (int m = 0; m < kGM; ++m) E[m] = (m < g.ng) ? T.a[6 + m] * T.c[6 + m] * NM<R>::ex(-g.eta[m] * T.rjk2) : R(0);
}

template <typename R> __device__ void acsf_g3_forward_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt,
                                                           R *G) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const GridConst<R> g = grid_const<R>(M, ei);
    R acc[kGM][kGQ];
#pragma unroll
    for (int m = 0; m < kGM; ++m)
#pragma unroll
        for (int q = 0; q < kGQ; ++q) acc[m][q] = R(0);
    RowWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (fast_pair(M, ei, C.nbelem[tw.q3], C.nbelem[tw.q4]) && triplet_geom<R>(M, C, tw.q3, tw.q4, rc, T)) {
            R E[kGM];
            grid_pexp<R>(g, T, E);
#pragma unroll
            for (int m = 0; m < kGM; ++m) E[m] *= T.pfc;
            Ladder<R> L;
            ladder_make<R>(g, T.cost0, L);
#pragma unroll
            for (int q = 0; q < kGQ; ++q) {
                if (q >= g.nq) break;
                const int l = g.lidx[q];
                if (!L.pos[l]) continue;
                const R pw = ladder_pow<R>(L, l, g.zm1[q]) * L.pw[l][0];
#pragma unroll
                for (int m = 0; m < kGM; ++m) acc[m][q] += E[m] * pw;
            }
        }
        tw.next();
    }
#pragma unroll
    for (int m = 0; m < kGM; ++m)
#pragma unroll
        for (int q = 0; q < kGQ; ++q) {
            if (m >= g.ng || q >= g.nq) continue;
            const R v = warp_sum(acc[m][q]);
            const int s = M.sf_of[ei][m][q];
            if (lane == 0 && s >= 0) G[s] = v * g.pn[q];
        }
    __syncwarp();
}

// G3 part of the VJP in grid form; adds into fix/fiy/fiz and the slot forces
template <typename R>
__device__ void acsf_g3_vjp_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, const R *c, R &fix, R &fiy,
                                 R &fiz) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const GridConst<R> g = grid_const<R>(M, ei);
    R Wc[kGM][kGQ];
#pragma unroll
    for (int m = 0; m < kGM; ++m)
#pragma unroll
        for (int q = 0; q < kGQ; ++q) {
            const int s = (m < g.ng && q < g.nq) ? M.sf_of[ei][m][q] : -1;
            Wc[m][q] = s >= 0 ? c[s] * g.pn[q] : R(0);
        }
    R sjx = R(0), sjy = R(0), sjz = R(0);  // force on the current row's neighbour q3
    RowWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (fast_pair(M, ei, C.nbelem[tw.q3], C.nbelem[tw.q4]) && triplet_geom<R>(M, C, tw.q3, tw.q4, rc, T)) {
            R E[kGM];
            grid_pexp<R>(g, T, E);
            Ladder<R> L;
            ladder_make<R>(g, T.cost0, L);
            R A1 = R(0), A2 = R(0), A3 = R(0);
#pragma unroll
            for (int q = 0; q < kGQ; ++q) {
                if (q >= g.nq) break;
                const int l = g.lidx[q];
                if (!L.pos[l]) continue;
                const R plam = L.pw[l][0];
                const R pp = ladder_pow<R>(L, l, g.zm1[q]);
                R S = R(0), Tq = R(0);
#pragma unroll
                for (int m = 0; m < kGM; ++m) {
                    const R w = Wc[m][q] * E[m];
                    S += w;
                    Tq += g.eta[m] * w;
                }
                A1 += g.zl[q] * pp * S;
                A2 += plam * pp * Tq;
                A3 += plam * pp * S;
            }
            const R rij = T.a[3], rik = T.c[3];
            const R P1 = T.pfc * (T.rinv0 - T.cost0 / (rij * rij)) * A1 - R(2) * T.pfc * A2 +
                         T.c[4] * T.fcjk * T.a[5] / rij * A3;
            const R P2 = T.pfc * (T.rinv0 - T.cost0 / (rik * rik)) * A1 - R(2) * T.pfc * A2 +
                         T.a[4] * T.fcjk * T.c[5] / rik * A3;
            const R P3 = T.pfc * T.rinv0 * A1 + R(2) * T.pfc * A2 - T.a[4] * T.c[4] * T.dfcjk / T.rjk * A3;
            fix += T.a[0] * P1 + T.c[0] * P2;
            fiy += T.a[1] * P1 + T.c[1] * P2;
            fiz += T.a[2] * P1 + T.c[2] * P2;
            sjx += -T.a[0] * P1 + T.jx * P3;
            sjy += -T.a[1] * P1 + T.jy * P3;
            sjz += -T.a[2] * P1 + T.jz * P3;
            atomicAdd(&C.slotf[3 * tw.q4], -T.c[0] * P2 - T.jx * P3);
            atomicAdd(&C.slotf[3 * tw.q4 + 1], -T.c[1] * P2 - T.jy * P3);
            atomicAdd(&C.slotf[3 * tw.q4 + 2], -T.c[2] * P2 - T.jz * P3);
        }
        if (tw.row_end) {
            atomicAdd(&C.slotf[3 * tw.q3], sjx);
            atomicAdd(&C.slotf[3 * tw.q3 + 1], sjy);
            atomicAdd(&C.slotf[3 * tw.q3 + 2], sjz);
            sjx = sjy = sjz = R(0);
        }
        tw.next();
    }
}

// G3 part of the JVP in grid form; lane 0 writes v[s]
template <typename R>
__device__ void acsf_g3_jvp_fast(const NNDev &M, const WarpCache<R> &C, int ei, int cnt, int i, const R *ux,
                                 const R *uy, const R *uz, R *v) {
    const int lane = threadIdx.x & 31;
    const R rc = (R)M.rc[ei];
    const GridConst<R> g = grid_const<R>(M, ei);
    const R uix = ux[i], uiy = uy[i], uiz = uz[i];
    R acc[kGM][kGQ];
#pragma unroll
    for (int m = 0; m < kGM; ++m)
#pragma unroll
        for (int q = 0; q < kGQ; ++q) acc[m][q] = R(0);
    RowWalk tw;
    tw.init(cnt, lane);
    while (tw.valid) {
        Triplet<R> T;
        if (fast_pair(M, ei, C.nbelem[tw.q3], C.nbelem[tw.q4]) && triplet_geom<R>(M, C, tw.q3, tw.q4, rc, T)) {
            const int j = C.nbatom[tw.q3], kk = C.nbatom[tw.q4];
            const R q1 = -(T.a[0] * (uix - ux[j]) + T.a[1] * (uiy - uy[j]) + T.a[2] * (uiz - uz[j]));
            const R q2 = -(T.c[0] * (uix - ux[kk]) + T.c[1] * (uiy - uy[kk]) + T.c[2] * (uiz - uz[kk]));
            const R q3 = T.jx * (ux[kk] - ux[j]) + T.jy * (uy[kk] - uy[j]) + T.jz * (uz[kk] - uz[j]);
            const R rij = T.a[3], rik = T.c[3];
            const R b1 = T.pfc * (T.rinv0 - T.cost0 / (rij * rij)), b2 = T.pfc * (T.rinv0 - T.cost0 / (rik * rik));
            const R d1 = T.c[4] * T.fcjk * T.a[5] / rij, d2 = T.a[4] * T.fcjk * T.c[5] / rik;
            const R d3 = T.a[4] * T.c[4] * T.dfcjk / T.rjk;
            const R X1 = b1 * q1 + b2 * q2 + T.pfc * T.rinv0 * q3, X2 = T.pfc * (q1 + q2 - q3),
                    X3 = d1 * q1 + d2 * q2 - d3 * q3;
            R E[kGM];
            grid_pexp<R>(g, T, E);
            Ladder<R> L;
            ladder_make<R>(g, T.cost0, L);
#pragma unroll
            for (int q = 0; q < kGQ; ++q) {
                if (q >= g.nq) break;
                const int l = g.lidx[q];
                if (!L.pos[l]) continue;
                const R plam = L.pw[l][0];
                const R base = ladder_pow<R>(L, l, g.zm1[q]) * g.pn[q];
                const R t1 = g.zl[q] * X1 + plam * X3, t2 = R(2) * plam * X2;
#pragma unroll
                for (int m = 0; m < kGM; ++m) acc[m][q] -= base * E[m] * (t1 - g.eta[m] * t2);
            }
        }
        tw.next();
    }
#pragma unroll
    for (int m = 0; m < kGM; ++m)
#pragma unroll
        for (int q = 0; q < kGQ; ++q) {
            if (m >= g.ng || q >= g.nq) continue;
            const R val = warp_sum(acc[m][q]);
            const int s = M.sf_of[ei][m][q];
            if (lane == 0 && s >= 0) v[s] = val;
        }
    __syncwarp();
}

}  // namespace mdt
