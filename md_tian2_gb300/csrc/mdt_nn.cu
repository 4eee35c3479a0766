// mdt_nn.cu -- HDNNP (RuNNer-style) force evaluation and the NN-surrogate MD step.
// See mdt_nn.cuh for the per-warp descriptor/network design.
#include <cstdio>

#include "mdt_common.cuh"
#include "mdt_emt.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"
#include "mdt_acsf.cuh"
#include "mdt_prop.cuh"

namespace mdt {

constexpr int kNNBlock = 32 * kNNWarps;
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

    if (tid == 0) {
        acsf_lattice(B.box + 9 * t, S.lat);
        *S.flag = 0;
    }
    __syncthreads();
    for (int i = tid; i < N; i += nt) {
        acsf_wrap_one(B.rx[base + i], B.ry[base + i], B.rz[base + i], S.lat, S.px[i], S.py[i], S.pz[i]);
        S.elem[i] = (int8_t)M.elem_of_type[B.type[aoff + i]];
        S.fx[i] = R(0);
        S.fy[i] = R(0);
        S.fz[i] = R(0);
    }
    __syncthreads();
    // ---- neighbour lists ----------------------------------------------------------
    const int na = X.img[3 * t], nbi = X.img[3 * t + 1], nc = X.img[3 * t + 2];
    for (int i = tid; i < N; i += nt) {
        int cnt = acsf_neighbors_one(M, i, N, S.px, S.py, S.pz, S.lat, na, nbi, nc,
                                     X.nbw + (base + i) * (int64_t)M.maxnb);
        if (cnt > M.maxnb) {
            X.nnstatus[t] = 1;
            cnt = M.maxnb;
        }
        X.nbcnt[base + i] = cnt;
    }
    __syncthreads();

    const R *W = S.w;
    WarpCache<R> C{S.nb + (size_t)warp * M.maxnb * S.stride, S.slotf + (size_t)warp * M.maxnb * 3,
                   S.nbatom + warp * M.maxnb, S.nbelem + warp * M.maxnb, S.stride};
    R *G = S.G + warp * kMaxSF;
    R *dEdG = S.dEdG + warp * kMaxSF;
    R *hs = S.hs + warp * (kMaxLayers + 1) * kMaxNodes;
    R *hv = S.hv + warp * (kMaxLayers + 1) * kMaxNodes;
    double e_warp = 0.0;

    for (int i = warp; i < N; i += kNNWarps) {
        const int ei = S.elem[i];
        if (ei < 0) continue;
        const int cnt = X.nbcnt[base + i];
        acsf_cache<R>(M, C, i, ei, cnt, X.nbw + (base + i) * (int64_t)M.maxnb, S.px, S.py, S.pz, S.elem, S.lat);
        const int nsf = M.nsf[ei];
        const int sfb = ei * M.maxsf;
        if (X.dgin) {
            // network on the tensor cores in a prior pass: its atomic energy and dE/dG
            if (lane == 0) e_warp += X.eatin[base + i] + (M.remove_atom_energies ? M.atom_energy[ei] : 0.0);
            if (!do_forces) {
                __syncwarp();
                continue;
            }
            for (int s = lane; s < nsf; s += 32) dEdG[s] = (R)X.dgin[(base + i) * M.maxsf + s];
            __syncwarp();
        } else {
            acsf_forward<R>(M, C, ei, cnt, G);
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
            R *delta = hs;  // sums are overwritten by deltas, layer by layer from the top
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
                    // dG_scaled/dG: (scmax-scmin)/(max-min) whenever scale_symmetry_functions is
                    // set, as getshortatomic.f90:174-190 scales dG/dx
                    if (M.scalesym) v *= (R)((M.scmax - M.scmin) / (M.smax[sfb + s] - M.smin[sfb + s]));
                    dEdG[s] = v;
                }
            }
            __syncwarp();
        }  // descriptors and network in this pass
        R fix, fiy, fiz;
        acsf_vjp<R>(M, C, ei, cnt, dEdG, fix, fiy, fiz);
        if (lane == 0) {
            atomicAdd(&S.fx[i], fix);
            atomicAdd(&S.fy[i], fiy);
            atomicAdd(&S.fz[i], fiz);
        }
        for (int q = lane; q < cnt; q += 32) {
            const int j = C.nbatom[q];
            atomicAdd(&S.fx[j], C.slotf[3 * q]);
            atomicAdd(&S.fy[j], C.slotf[3 * q + 1]);
            atomicAdd(&S.fz[j], C.slotf[3 * q + 2]);
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
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, SE.cjk, step, SE.red);
            nn_calc_force<R, SURR>(B, M, E, X, P, S, SE, T, true);
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
