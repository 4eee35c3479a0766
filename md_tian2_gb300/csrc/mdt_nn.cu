// mdt_nn.cu -- HDNNP (RuNNer-style) force evaluation and the NN-surrogate MD step.
// See mdt_nn.cuh for the per-warp descriptor/network design.
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"
#include "mdt_prop.cuh"

namespace mdt {

constexpr int kNNBlock = 32 * kNNWarps;
constexpr int kMaxG3 = 24;   // G3 functions per element held in lane registers
constexpr double kAng2BohrD = 1.0 / kBohr2Ang;
constexpr double kHa2eV = 27.21138602;

template <typename R> struct SmemNN {
    double *px, *py, *pz;  // wrapped positions, bohr
    int8_t *elem;
    R *fx, *fy, *fz;       // force accumulators, Ha/bohr
    double *red, *lat;     // lat: 9 lattice (rows = vectors) + 9 inverse
    R *w;                  // network weights of all elements
    // per warp
    R *nb;                 // [warp][q][stride]
    R *slotf;              // [warp][q][3]
    int *nbatom;           // [warp][q]
    int8_t *nbelem;        // [warp][q]
    R *G, *dEdG;           // [warp][kMaxSF]
    R *hs, *hv;            // [warp][kMaxLayers+1][kMaxNodes] sums / values
    int *flag;             // out-of-range flag for the bead
    int stride;
};

__host__ __device__ inline int nn_stride(int ngeta) { return 6 + ngeta; }

__host__ __device__ inline size_t nn_smem_bytes(int max_atoms, int maxnb, int ngeta, int nelem, int maxweights,
                                                size_t rs) {
    auto r16 = [](size_t b) -> size_t { return (b + 15) & ~size_t(15); };
    size_t s = 3 * r16(8 * max_atoms) + r16(max_atoms) + 3 * r16(rs * max_atoms) + r16(8 * 64) + r16(8 * 18) +
               r16(rs * (size_t)nelem * maxweights);
    s += r16(rs * kNNWarps * maxnb * nn_stride(ngeta)) + r16(rs * kNNWarps * maxnb * 3) +
         r16(4 * kNNWarps * maxnb) + r16(kNNWarps * maxnb) + 2 * r16(rs * kNNWarps * kMaxSF) +
         2 * r16(rs * kNNWarps * (kMaxLayers + 1) * kMaxNodes) + 16;
    return s;
}

template <typename R>
__device__ SmemNN<R> carve_nn(unsigned char *base, const NNDev &M, int max_atoms, int ngeta) {
    SmemNN<R> s;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += (bytes + 15) & ~size_t(15);
        return p;
    };
    s.px = (double *)take(8 * max_atoms);
    s.py = (double *)take(8 * max_atoms);
    s.pz = (double *)take(8 * max_atoms);
    s.elem = (int8_t *)take(max_atoms);
    s.fx = (R *)take(sizeof(R) * max_atoms);
    s.fy = (R *)take(sizeof(R) * max_atoms);
    s.fz = (R *)take(sizeof(R) * max_atoms);
    s.red = (double *)take(8 * 64);
    s.lat = (double *)take(8 * 18);
    s.w = (R *)take(sizeof(R) * M.nelem * M.maxweights);
    s.stride = nn_stride(ngeta);
    s.nb = (R *)take(sizeof(R) * kNNWarps * M.maxnb * s.stride);
    s.slotf = (R *)take(sizeof(R) * kNNWarps * M.maxnb * 3);
    s.nbatom = (int *)take(4 * kNNWarps * M.maxnb);
    s.nbelem = (int8_t *)take(kNNWarps * M.maxnb);
    s.G = (R *)take(sizeof(R) * kNNWarps * kMaxSF);
    s.dEdG = (R *)take(sizeof(R) * kNNWarps * kMaxSF);
    s.hs = (R *)take(sizeof(R) * kNNWarps * (kMaxLayers + 1) * kMaxNodes);
    s.hv = (R *)take(sizeof(R) * kNNWarps * (kMaxLayers + 1) * kMaxNodes);
    s.flag = (int *)take(16);
    return s;
}

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

__device__ __forceinline__ int pack_nb(int j, int n1, int n2, int n3) {
    return j | ((n1 + 8) << 16) | ((n2 + 8) << 20) | ((n3 + 8) << 24);
}

// ---------------------------------------------------------------------------
// One bead: wrapped positions, neighbour lists, descriptors, network, forces.
// Adds eV and eV/A into B.epot / B.f*.  Returns (in S.flag) whether a descriptor left
// the scaling range widened by M.margin.
// ---------------------------------------------------------------------------
template <typename R>
__device__ bool nn_bead(const Batch &B, const NNDev &M, const NNScratch &X, const SmemNN<R> &S, int t, int b,
                        bool do_forces, bool skip_if_flagged) {
    const int N = B.natoms[t];
    const int64_t base = B.ba_off[t] + (int64_t)b * N;
    const int aoff = B.atom_off[t];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int warp = tid >> 5, lane = tid & 31;

    // lattice rows (bohr) and inverse of the column matrix, exactly as the oracle's wrap
    if (tid == 0) {
        const double *bx = B.box + 9 * t;  // column major: column i = vector i
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) S.lat[3 * i + k] = __dmul_rn(bx[3 * i + k], kAng2BohrD);
        double A[9];
        for (int i = 0; i < 3; ++i)
            for (int k = 0; k < 3; ++k) A[k * 3 + i] = S.lat[3 * i + k];
        double *I = S.lat + 9;
        // cofactor inverse without contraction (matches the oracle bit for bit)
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
        *S.flag = 0;
    }
    __syncthreads();
    for (int i = tid; i < N; i += nt) {
        double x = __dmul_rn(B.rx[base + i], kAng2BohrD), y = __dmul_rn(B.ry[base + i], kAng2BohrD),
               z = __dmul_rn(B.rz[base + i], kAng2BohrD);
        const double *I = S.lat + 9;
        double f[3];
        for (int d = 0; d < 3; ++d)
            f[d] = __dadd_rn(__dadd_rn(__dmul_rn(I[3 * d], x), __dmul_rn(I[3 * d + 1], y)), __dmul_rn(I[3 * d + 2], z));
        for (int d = 0; d < 3; ++d) {
            const double s = floor(f[d]);
            if (s != 0.0) {
                x = __dsub_rn(x, __dmul_rn(s, S.lat[3 * d]));
                y = __dsub_rn(y, __dmul_rn(s, S.lat[3 * d + 1]));
                z = __dsub_rn(z, __dmul_rn(s, S.lat[3 * d + 2]));
            }
        }
        S.px[i] = x;
        S.py[i] = y;
        S.pz[i] = z;
        S.elem[i] = (int8_t)M.elem_of_type[B.type[aoff + i]];
        S.fx[i] = R(0);
        S.fy[i] = R(0);
        S.fz[i] = R(0);
    }
    __syncthreads();

    // ---- neighbour lists, RuNNer order (neighbor_para_short.f90:117-163) --------
    const int na = X.img[3 * t], nbi = X.img[3 * t + 1], nc = X.img[3 * t + 2];
    const double cut2 = __dmul_rn(M.maxcut, M.maxcut);
    const double *L = S.lat;
    for (int i = tid; i < N; i += nt) {
        int cnt = 0;
        int *out = X.nbw + (base + i) * (int64_t)M.maxnb;
        const double xi = S.px[i], yi = S.py[i], zi = S.pz[i];
        for (int j = 0; j < N; ++j) {
            const double xj = S.px[j], yj = S.py[j], zj = S.pz[j];
            for (int n1 = -na; n1 <= na; ++n1)
                for (int n2 = -nbi; n2 <= nbi; ++n2)
                    for (int n3 = -nc; n3 <= nc; ++n3) {
                        if (n1 == 0 && n2 == 0 && n3 == 0 && i == j) continue;
                        const double d1n = n1, d2n = n2, d3n = n3;
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
        if (cnt > M.maxnb) {
            X.nnstatus[t] = 1;
            cnt = M.maxnb;
        }
        X.nbcnt[base + i] = cnt;
    }
    __syncthreads();

    const R *W = S.w;
    R *nbw = S.nb + (size_t)warp * M.maxnb * S.stride;
    R *slotf = S.slotf + (size_t)warp * M.maxnb * 3;
    int *nbatom = S.nbatom + warp * M.maxnb;
    int8_t *nbelem = S.nbelem + warp * M.maxnb;
    R *G = S.G + warp * kMaxSF;
    R *dEdG = S.dEdG + warp * kMaxSF;
    R *hs = S.hs + warp * (kMaxLayers + 1) * kMaxNodes;
    R *hv = S.hv + warp * (kMaxLayers + 1) * kMaxNodes;
    const int st = S.stride;
    double e_warp = 0.0;

    for (int i = warp; i < N; i += kNNWarps) {
        const int ei = S.elem[i];
        if (ei < 0) continue;
        const int cnt = X.nbcnt[base + i];
        const int *words = X.nbw + (base + i) * (int64_t)M.maxnb;
        const R rc = (R)M.rc[ei];
        const int ng = M.ng3eta[ei];
        // ---- neighbour cache ----------------------------------------------------
        for (int q = lane; q < cnt; q += 32) {
            const int w = words[q];
            const int j = w & 0xFFFF;
            const double n1 = ((w >> 16) & 15) - 8, n2 = ((w >> 20) & 15) - 8, n3 = ((w >> 24) & 15) - 8;
            const double dx = S.px[j] + n1 * L[0] + n2 * L[3] + n3 * L[6] - S.px[i];
            const double dy = S.py[j] + n1 * L[1] + n2 * L[4] + n3 * L[7] - S.py[i];
            const double dz = S.pz[j] + n1 * L[2] + n2 * L[5] + n3 * L[8] - S.pz[i];
            const R r = (R)sqrt(dx * dx + dy * dy + dz * dz);
            R *e = nbw + q * st;
            e[0] = (R)dx;
            e[1] = (R)dy;
            e[2] = (R)dz;
            e[3] = r;
            R fc = R(0), dfc = R(0);
            if (r <= rc) cutoff_fn<R>(M, rc, r, fc, dfc);
            e[4] = fc;
            e[5] = dfc;
            for (int m = 0; m < ng; ++m) e[6 + m] = NM<R>::ex(-(R)M.g3eta[ei][m] * r * r);
            nbatom[q] = j;
            nbelem[q] = S.elem[j];
            slotf[3 * q] = R(0);
            slotf[3 * q + 1] = R(0);
            slotf[3 * q + 2] = R(0);
        }
        __syncwarp();
        const int nsf = M.nsf[ei];
        const int sfb = ei * M.maxsf;
        // ---- G2 (atomsymfunction2.f90:80-170) -----------------------------------
        for (int s = 0; s < nsf; ++s) {
            if (M.sftype[sfb + s] != 2) continue;
            const R eta = (R)M.eta[sfb + s], rs = (R)M.rs[sfb + s];
            const int e1 = M.e1[sfb + s];
            R acc = R(0);
            for (int q = lane; q < cnt; q += 32) {
                const R *e = nbw + q * st;
                if (nbelem[q] != e1 || !(e[3] <= rc)) continue;
                acc += NM<R>::ex(-eta * (e[3] - rs) * (e[3] - rs)) * e[4];
            }
            acc = warp_sum(acc);
            if (lane == 0) G[s] = acc;
        }
        // ---- G3 (atomsymfunction3Andi.f90:90-257), all G3 of this element at once --
        int g3idx[kMaxG3];
        int ng3 = 0;
        for (int s = 0; s < nsf && ng3 < kMaxG3; ++s)
            if (M.sftype[sfb + s] == 3) g3idx[ng3++] = s;
        {
            R acc[kMaxG3];
#pragma unroll
            for (int u = 0; u < kMaxG3; ++u) acc[u] = R(0);
            const R rc2 = rc * rc;
            TriWalk tw;
            tw.init(cnt, lane);
            while (tw.valid) {
                const R *a = nbw + tw.q3 * st, *c = nbw + tw.q4 * st;
                const int ej = nbelem[tw.q3], ek = nbelem[tw.q4];
                if (a[3] <= rc && c[3] <= rc) {
                    const R jx = a[0] - c[0], jy = a[1] - c[1], jz = a[2] - c[2];
                    const R rjk2 = jx * jx + jy * jy + jz * jz;
                    if (rjk2 <= rc2) {
                        const R rjk = NM<R>::sq(rjk2);
                        R fcjk, dfcjk;
                        cutoff_fn<R>(M, rc, rjk, fcjk, dfcjk);
                        const R cost = (a[0] * c[0] + a[1] * c[1] + a[2] * c[2]) / (a[3] * c[3]);
                        const R pfc = a[4] * c[4] * fcjk;
                        R ejk[kMaxEta];
                        for (int m = 0; m < ng; ++m) ejk[m] = NM<R>::ex(-(R)M.g3eta[ei][m] * rjk2);
#pragma unroll
                        for (int u = 0; u < kMaxG3; ++u) {
                            if (u >= ng3) break;
                            const int s = g3idx[u];
                            const int e1 = M.e1[sfb + s], e2 = M.e2[sfb + s];
                            if (!((e1 == ej && e2 == ek) || (e2 == ej && e1 == ek))) continue;
                            const int m = M.etaslot[sfb + s];
                            const R pexp = a[6 + m] * c[6 + m] * ejk[m];
                            const R plam = R(1) + (R)M.lam[sfb + s] * cost;
                            if (plam <= R(0)) continue;
                            const int iz = M.izeta[sfb + s];
                            const R pz = iz >= 0 ? ipow<R>(plam, iz) : NM<R>::pw(plam, (R)M.zeta[sfb + s] - R(1));
                            acc[u] += pz * pexp * plam * pfc;
                        }
                    }
                }
                tw.next();
            }
#pragma unroll
            for (int u = 0; u < kMaxG3; ++u) {
                if (u >= ng3) break;
                const R v = warp_sum(acc[u]);
                if (lane == 0) G[g3idx[u]] = v * (R)M.pnorm[sfb + g3idx[u]];
            }
        }
        __syncwarp();
        if (X.gout)
            for (int s = lane; s < nsf; s += 32) X.gout[(base + i) * M.maxsf + s] = (double)G[s];
        // ---- scaling (getshortatomic.f90:174-236) and range check ------------------
        for (int s = lane; s < nsf; s += 32) {
            const double mn = M.smin[sfb + s], mx = M.smax[sfb + s], w = mx - mn;
            const double g = (double)G[s];
            if (g < mn - M.margin * w || g > mx + M.margin * w) *S.flag = 1;
            double gs = g;
            if (M.centersym && !M.scalesym) gs = g - M.savg[sfb + s];
            else if (M.scalesym && !M.centersym) gs = (g - mn) / w * (M.scmax - M.scmin) + M.scmin;
            else if (M.scalesym && M.centersym) gs = (g - M.savg[sfb + s]) / w;
            hv[s] = (R)gs;  // layer 0 values
        }
        __syncwarp();
        // ---- network forward (calconenn.f90:83-153) --------------------------------
        const R *we = W + (size_t)ei * M.maxweights;
        for (int l = 1; l <= M.nlayers; ++l) {
            const int nprev = M.nodes[ei][l - 1], ncur = M.nodes[ei][l];
            const R *wl = we + M.woff[ei][l];
            for (int n = lane; n < ncur; n += 32) {
                R z = R(0);
                for (int p = 0; p < nprev; ++p) z += wl[p * ncur + n] * hv[(l - 1) * kMaxNodes + p];
                z += wl[nprev * ncur + n];
                if (M.normnodes) z /= (R)nprev;
                hs[l * kMaxNodes + n] = z;
                hv[l * kMaxNodes + n] = act_fn<R>(M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n], z);
            }
            __syncwarp();
        }
        if (lane == 0) e_warp += (double)hv[M.nlayers * kMaxNodes] + (M.remove_atom_energies ? M.atom_energy[ei] : 0.0);
        if (!do_forces) {
            __syncwarp();
            continue;
        }
        // ---- backward: dE/dG (getdnodes_values.f90 + the chain of getshortatomic.f90:263-291)
        R *delta = hs;  // reuse sums in place as deltas, layer by layer from the top
        for (int l = M.nlayers; l >= 1; --l) {
            const int ncur = M.nodes[ei][l];
            const R norm = M.normnodes ? R(1) / (R)M.nodes[ei][l - 1] : R(1);
            for (int n = lane; n < ncur; n += 32) {
                const uint8_t a = M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n];
                const R dn = norm * act_dfn<R>(a, hs[l * kMaxNodes + n], hv[l * kMaxNodes + n]);
                R up = R(1);
                if (l < M.nlayers) {
                    const int nn = M.nodes[ei][l + 1];
                    const R *wl = we + M.woff[ei][l + 1];
                    up = R(0);
                    for (int m = 0; m < nn; ++m) up += wl[n * nn + m] * delta[(l + 1) * kMaxNodes + m];
                }
                // hs[l] is read only by this lane for node n: safe to overwrite after use
                delta[l * kMaxNodes + n] = dn * up;
            }
            __syncwarp();
        }
        {
            const int n1 = M.nodes[ei][1];
            const R *wl = we + M.woff[ei][1];
            for (int s = lane; s < nsf; s += 32) {
                R v = R(0);
                for (int n = 0; n < n1; ++n) v += wl[s * n1 + n] * delta[1 * kMaxNodes + n];
                if (M.scalesym)
                    v *= (R)((M.scmax - M.scmin) / (M.smax[sfb + s] - M.smin[sfb + s]));
                dEdG[s] = v;
            }
        }
        __syncwarp();
        // ---- forces: G2 --------------------------------------------------------------
        R fix = R(0), fiy = R(0), fiz = R(0);
        for (int q = lane; q < cnt; q += 32) {
            const R *e = nbw + q * st;
            if (!(e[3] <= rc)) continue;
            R dsum = R(0);
            for (int s = 0; s < nsf; ++s) {
                if (M.sftype[sfb + s] != 2 || nbelem[q] != M.e1[sfb + s]) continue;
                const R eta = (R)M.eta[sfb + s], rs = (R)M.rs[sfb + s];
                const R ex = NM<R>::ex(-eta * (e[3] - rs) * (e[3] - rs));
                dsum += dEdG[s] * (R(-2) * eta * (e[3] - rs) * ex * e[4] + ex * e[5]);
            }
            // dG/dx_j = +(d/r) dt/dr ; force = -dE/dG . dG/dx
            const R fr = dsum / e[3];
            slotf[3 * q] -= fr * e[0];
            slotf[3 * q + 1] -= fr * e[1];
            slotf[3 * q + 2] -= fr * e[2];
            fix += fr * e[0];
            fiy += fr * e[1];
            fiz += fr * e[2];
        }
        __syncwarp();
        // ---- forces: G3 ---------------------------------------------------------------
        {
            const R rc2 = rc * rc;
            TriWalk tw;
            tw.init(cnt, lane);
            while (tw.valid) {
                const R *a = nbw + tw.q3 * st, *c = nbw + tw.q4 * st;
                const int ej = nbelem[tw.q3], ek = nbelem[tw.q4];
                if (a[3] <= rc && c[3] <= rc) {
                    const R jx = a[0] - c[0], jy = a[1] - c[1], jz = a[2] - c[2];
                    const R rjk2 = jx * jx + jy * jy + jz * jz;
                    if (rjk2 <= rc2) {
                        const R rij = a[3], rik = c[3];
                        const R rjk = NM<R>::sq(rjk2);
                        R fcjk, dfcjk;
                        cutoff_fn<R>(M, rc, rjk, fcjk, dfcjk);
                        const R rinv0 = R(1) / (rij * rik);
                        const R cost0 = (a[0] * c[0] + a[1] * c[1] + a[2] * c[2]) * rinv0;
                        const R pfc = a[4] * c[4] * fcjk;
                        R ejk[kMaxEta];
                        for (int m = 0; m < ng; ++m) ejk[m] = NM<R>::ex(-(R)M.g3eta[ei][m] * rjk2);
                        R P1 = R(0), P2 = R(0), P3 = R(0);
                        for (int u = 0; u < ng3; ++u) {
                            const int s = g3idx[u];
                            const int e1 = M.e1[sfb + s], e2 = M.e2[sfb + s];
                            if (!((e1 == ej && e2 == ek) || (e2 == ej && e1 == ek))) continue;
                            const int m = M.etaslot[sfb + s];
                            const R lam = (R)M.lam[sfb + s], zeta = (R)M.zeta[sfb + s], eta = (R)M.eta[sfb + s];
                            const R plam = R(1) + lam * cost0;
                            if (plam <= R(0)) continue;
                            const R pexp = a[6 + m] * c[6 + m] * ejk[m];
                            const int iz = M.izeta[sfb + s];
                            const R fg = (iz >= 0 ? ipow<R>(plam, iz) : NM<R>::pw(plam, zeta - R(1))) * pexp *
                                         (R)M.pnorm[sfb + s] * dEdG[s];
                            const R pzl = zeta * lam;
                            const R rinv = rinv0 * pzl, cost = cost0 * pzl, p2el = R(2) * eta * plam;
                            P1 += fg * (pfc * (rinv - cost / (rij * rij) - p2el) + c[4] * fcjk * a[5] * plam / rij);
                            P2 += fg * (pfc * (rinv - cost / (rik * rik) - p2el) + a[4] * fcjk * c[5] * plam / rik);
                            P3 += fg * (pfc * (rinv + p2el) - a[4] * c[4] * dfcjk * plam / rjk);
                        }
                        // dxij = x_i - x_j = -a, dxik = -c, dxjk = x_j - x_k = a - c
                        // F_i -= dxij P1 + dxik P2 ; F_j -= -dxij P1 - dxjk P3 ; F_k -= -dxik P2 + dxjk P3
                        fix += a[0] * P1 + c[0] * P2;
                        fiy += a[1] * P1 + c[1] * P2;
                        fiz += a[2] * P1 + c[2] * P2;
                        atomicAdd(&slotf[3 * tw.q3], -a[0] * P1 + jx * P3);
                        atomicAdd(&slotf[3 * tw.q3 + 1], -a[1] * P1 + jy * P3);
                        atomicAdd(&slotf[3 * tw.q3 + 2], -a[2] * P1 + jz * P3);
                        atomicAdd(&slotf[3 * tw.q4], -c[0] * P2 - jx * P3);
                        atomicAdd(&slotf[3 * tw.q4 + 1], -c[1] * P2 - jy * P3);
                        atomicAdd(&slotf[3 * tw.q4 + 2], -c[2] * P2 - jz * P3);
                    }
                }
                tw.next();
            }
        }
        __syncwarp();
        fix = warp_sum(fix);
        fiy = warp_sum(fiy);
        fiz = warp_sum(fiz);
        if (lane == 0) {
            atomicAdd(&S.fx[i], fix);
            atomicAdd(&S.fy[i], fiy);
            atomicAdd(&S.fz[i], fiz);
        }
        for (int q = lane; q < cnt; q += 32) {
            const int j = nbatom[q];
            atomicAdd(&S.fx[j], slotf[3 * q]);
            atomicAdd(&S.fy[j], slotf[3 * q + 1]);
            atomicAdd(&S.fz[j], slotf[3 * q + 2]);
        }
        __syncwarp();
    }
    const double etot = block_sum(e_warp, S.red);  // contains __syncthreads: flag visible
    const bool flagged = *S.flag != 0;
    if (skip_if_flagged && flagged) {
        __syncthreads();
        return true;
    }
    if (tid == 0) B.epot[B.bead_off[t] + b] += etot * kHa2eV;
    if (do_forces) {
        const double c = kHa2eV * kAng2BohrD;
        for (int i = tid; i < N; i += nt) {
            B.fx[base + i] += (double)S.fx[i] * c;
            B.fy[base + i] += (double)S.fy[i] * c;
            B.fz[base + i] += (double)S.fz[i] * c;
        }
    }
    __syncthreads();
    return flagged;
}

__device__ __forceinline__ void load_weights_nn(const NNDev &M, float *dst) {
    for (int k = threadIdx.x; k < M.nelem * M.maxweights; k += blockDim.x) dst[k] = M.wf[k];
}
__device__ __forceinline__ void load_weights_nn(const NNDev &M, double *dst) {
    for (int k = threadIdx.x; k < M.nelem * M.maxweights; k += blockDim.x) dst[k] = M.wd[k];
}

// calc_force (force.f90:40-86) with the HDNNP: zero, free ring-polymer step, per-bead
// prediction, accelerations.  SURR: beads whose descriptors leave the training range
// are recomputed with plain FP64 EMT (the surrogate's fallback).
template <typename R, bool SURR>
__device__ void nn_calc_force(const Batch &B, const NNDev &M, const EmtConst &E, const NNScratch &X,
                              const PropParams &P, const SmemNN<R> &S, const SmemEmt<double> &SE, const TrajView &T,
                              bool do_forces) {
    const int tot = T.N * T.nb;
    for (int s = threadIdx.x; s < tot; s += blockDim.x) {
        const int64_t k = T.base + s;
        B.fx[k] = 0.0; B.fy[k] = 0.0; B.fz[k] = 0.0;
        B.ax[k] = 0.0; B.ay[k] = 0.0; B.az[k] = 0.0;
    }
    for (int b = threadIdx.x; b < T.nb; b += blockDim.x) B.epot[B.bead_off[T.t] + b] = 0.0;
    __syncthreads();
    if (T.nb > 1) ring_polymer_step(B, P, T, SE.cjk);
    for (int b = 0; b < T.nb; ++b) {
        const bool flagged = nn_bead<R>(B, M, X, S, T.t, b, do_forces, SURR);
        if (SURR && flagged) {
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

struct NNLaunch {
    int max_atoms, ngeta;
};

template <typename R, bool SURR>
__global__ void __launch_bounds__(kNNBlock) nn_force_kernel(Batch B, NNDev M, EmtConst E, NNScratch X, PropParams P,
                                                            NNLaunch LN, const int *order, int *counter, int do_forces) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    SmemNN<R> S = carve_nn<R>(smem_raw, M, LN.max_atoms, LN.ngeta);
    SmemEmt<double> SE = carve_smem<double>(smem_raw + nn_smem_bytes(LN.max_atoms, M.maxnb, LN.ngeta, M.nelem,
                                                                     M.maxweights, sizeof(R)),
                                            B.max_atoms, B.max_beads);
    load_weights_nn(M, S.w);
    for (;;) {
        if (threadIdx.x == 0) work_slot = atomicAdd(counter, 1);
        __syncthreads();
        const int w = work_slot;
        __syncthreads();
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, SE.cjk);
        nn_calc_force<R, SURR>(B, M, E, X, P, S, SE, T, do_forces != 0);
    }
}

template <typename R, bool SURR>
__global__ void __launch_bounds__(kNNBlock) nn_md_steps_kernel(Batch B, NNDev M, EmtConst E, NNScratch X,
                                                               PropParams P, NNLaunch LN, const int *order,
                                                               int *counter, int nsteps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    SmemNN<R> S = carve_nn<R>(smem_raw, M, LN.max_atoms, LN.ngeta);
    SmemEmt<double> SE = carve_smem<double>(smem_raw + nn_smem_bytes(LN.max_atoms, M.maxnb, LN.ngeta, M.nelem,
                                                                     M.maxweights, sizeof(R)),
                                            B.max_atoms, B.max_beads);
    load_weights_nn(M, S.w);
    for (;;) {
        if (threadIdx.x == 0) work_slot = atomicAdd(counter, 1);
        __syncthreads();
        const int w = work_slot;
        __syncthreads();
        if (w >= B.ntraj) break;
        const int t = order[w];
        const TrajView T = traj_view(B, t);
        load_cjk(B, t, SE.cjk);
        const int ty0 = B.type[T.aoff];
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, SE.cjk, step, SE.red);
            nn_calc_force<R, SURR>(B, M, E, X, P, S, SE, T, true);
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

size_t nn_total_smem(const NNDev &M, int max_atoms, int max_beads, int ngeta, int precision) {
    const size_t rs = precision == 1 ? 4 : 8;
    return nn_smem_bytes(max_atoms, M.maxnb, ngeta, M.nelem, M.maxweights, rs) + smem_bytes(max_atoms, max_beads, 8);
}

template <typename R, bool SURR>
static cudaError_t nn_launch_t(const LaunchCfg &c, const Batch &B, const NNDev &M, const EmtConst &E,
                               const NNScratch &X, const PropParams &P, int ngeta, int nsteps, int mode) {
    const size_t sm = nn_total_smem(M, B.max_atoms, B.max_beads, ngeta, sizeof(R) == 4 ? 1 : 0);
    NNLaunch LN{B.max_atoms, ngeta};
    cudaError_t e = cudaMemsetAsync(c.counter, 0, sizeof(int), c.stream);
    if (e != cudaSuccess) return e;
    if (mode == 0 || mode == 1) {
        e = cudaFuncSetAttribute(nn_force_kernel<R, SURR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        nn_force_kernel<R, SURR><<<c.grid, kNNBlock, sm, c.stream>>>(B, M, E, X, P, LN, c.order, c.counter,
                                                                     mode == 0 ? 1 : 0);
    } else {
        e = cudaFuncSetAttribute(nn_md_steps_kernel<R, SURR>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        nn_md_steps_kernel<R, SURR><<<c.grid, kNNBlock, sm, c.stream>>>(B, M, E, X, P, LN, c.order, c.counter,
                                                                        nsteps);
    }
    return cudaGetLastError();
}

cudaError_t launch_nn(const LaunchCfg &c, const Batch &B, const NNDev &M, const EmtConst &E, const NNScratch &X,
                      const PropParams &P, int ngeta, int nsteps, int mode, int precision, bool surrogate) {
    if (precision == 1)
        return surrogate ? nn_launch_t<float, true>(c, B, M, E, X, P, ngeta, nsteps, mode)
                         : nn_launch_t<float, false>(c, B, M, E, X, P, ngeta, nsteps, mode);
    return surrogate ? nn_launch_t<double, true>(c, B, M, E, X, P, ngeta, nsteps, mode)
                     : nn_launch_t<double, false>(c, B, M, E, X, P, ngeta, nsteps, mode);
}

int nn_resident_ctas(const NNDev &M, int max_atoms, int max_beads, int ngeta, int precision, bool surrogate) {
    const size_t sm = nn_total_smem(M, max_atoms, max_beads, ngeta, precision);
    int n = 0;
    if (precision == 1) {
        auto k = surrogate ? nn_md_steps_kernel<float, true> : nn_md_steps_kernel<float, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kNNBlock, sm);
    } else {
        auto k = surrogate ? nn_md_steps_kernel<double, true> : nn_md_steps_kernel<double, false>;
        cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kNNBlock, sm);
    }
    return n > 0 ? n : 1;
}

}  // namespace mdt
