// mdt_train.cu -- training of the per-element ACSF -> MLP network on energies and forces,
// fused per configuration, and its Adam update.
//
// A training configuration is one trajectory of the context's batch (positions, types
// and cell come from the batch arrays), labelled with a total energy (eV) and atomic
// forces (eV/A).  Raw symmetry functions and neighbour lists are computed once when the
// labels are set (they do not change); each step recomputes what depends on the
// weights.  Per configuration, one CTA:
//   pass A  (warp per atom) network forward + backward -> dE/dG, then the descriptor VJP
//           gives the predicted forces F;  E = sum of atomic energies;
//   loss    L = wE (dE_tot/N)^2 + wF sum|F - F_ref|^2 / (3N),  a = dL/dE,  u_k = dL/dF_k;
//   pass B  (warp per atom) descriptor JVP v_s = sum_k u_k . (-dG_s/dx_k) gives the
//           tangent direction of the network input, and one forward-over-reverse sweep
//           through the network yields dL/dW = a dE/dW + d/dW (v . dE/dg):
//             W_l[p][n] += delta_l[n] (a h_{l-1}[p] + hdot_{l-1}[p]) + delta'_l[n] h_{l-1}[p]
//             delta_{l-1}  = s'(z) (W delta_l),
//             delta'_{l-1} = s'(z) (W delta'_l) + s''(z) zdot (W delta_l).
// The descriptor derivatives are recomputed, never stored.  Gradients meet in warp-
// private shared-memory buffers (no atomics inside the network sweep) and are added to
// the global FP64 gradient once per CTA.
#include <algorithm>
#include <cstdio>

#include "mdt_acsf.cuh"
#include "mdt_emt.cuh"
#include "mdt_common.cuh"
#include "mdt_internal.h"
#include "mdt_nn.cuh"

namespace mdt {

constexpr double kHa2eVt = 27.21138602;

template <typename R> struct TrainCfg {
    static constexpr int warps = sizeof(R) == 4 ? 4 : 2;
};

struct TrainDev {
    const double *E_ref;                    // per configuration, eV
    const double *fx_ref, *fy_ref, *fz_ref; // per slot, eV/A
    const double *G;                        // raw symmetry functions [slot][maxsf]
    const int *conf;                        // configurations of this step
    int nconf;
    double wE, wF;
    const float *theta;                     // live weights [nelem*maxweights]
    double *grad;                           // accumulated gradient
    double *loss;                           // 0: sum (dE/N)^2 eV^2, 1: sum |dF|^2, 2: force components, 3: configs
    const float *dgin;                      // network outside (see TrainArgs): dE/dG per slot
    const double *eatin;                    //   output-node value per slot
    float *xdot;                            //   scaled descriptor tangent per slot (out)
    double *arow;                           //   dL/dE of the slot's configuration (out)
};

template <typename R> struct SmemTrain {
    double *px, *py, *pz, *lat, *red;
    int8_t *elem;
    R *fx, *fy, *fz, *ux, *uy, *uz, *w, *gradw;  // gradw: [warp][nelem*maxweights]
    R *nb, *slotf;
    int *nbatom;
    int8_t *nbelem;
    R *buf;   // per warp: G, c/v, then 6 x (L+1) x kMaxNodes network buffers
    double *scal;  // 0: a (dL/dE in Ha^-1 units)
    int stride;
};

__host__ __device__ inline size_t train_smem_bytes(int max_atoms, int maxnb, int ngeta, int nelem, int maxweights,
                                                   size_t rs, int warps) {
    auto r16 = [](size_t b) -> size_t { return (b + 15) & ~size_t(15); };
    size_t s = 3 * r16(8 * max_atoms) + r16(8 * 18) + r16(8 * 64) + r16(max_atoms) + 6 * r16(rs * max_atoms);
    s += r16(rs * (size_t)nelem * maxweights) * (1 + warps);
    s += r16(rs * warps * maxnb * (6 + ngeta)) + r16(rs * warps * maxnb * 3) + r16(4 * warps * maxnb) +
         r16(warps * maxnb);
    s += r16(rs * warps * (2 * kMaxSF + 6 * (kMaxLayers + 1) * kMaxNodes)) + r16(8 * 4);
    return s;
}

template <typename R>
__device__ SmemTrain<R> carve_train(unsigned char *base, const NNDev &M, int max_atoms, int ngeta) {
    constexpr int W = TrainCfg<R>::warps;
    SmemTrain<R> s;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char *p = base + off;
        off += (bytes + 15) & ~size_t(15);
        return p;
    };
    s.px = (double *)take(8 * max_atoms);
    s.py = (double *)take(8 * max_atoms);
    s.pz = (double *)take(8 * max_atoms);
    s.lat = (double *)take(8 * 18);
    s.red = (double *)take(8 * 64);
    s.elem = (int8_t *)take(max_atoms);
    s.fx = (R *)take(sizeof(R) * max_atoms);
    s.fy = (R *)take(sizeof(R) * max_atoms);
    s.fz = (R *)take(sizeof(R) * max_atoms);
    s.ux = (R *)take(sizeof(R) * max_atoms);
    s.uy = (R *)take(sizeof(R) * max_atoms);
    s.uz = (R *)take(sizeof(R) * max_atoms);
    const size_t nw = (size_t)M.nelem * M.maxweights;
    s.w = (R *)take(sizeof(R) * nw);
    s.gradw = (R *)take(sizeof(R) * nw * W);
    s.stride = 6 + ngeta;
    s.nb = (R *)take(sizeof(R) * W * M.maxnb * s.stride);
    s.slotf = (R *)take(sizeof(R) * W * M.maxnb * 3);
    s.nbatom = (int *)take(4 * W * M.maxnb);
    s.nbelem = (int8_t *)take(W * M.maxnb);
    s.buf = (R *)take(sizeof(R) * W * (2 * kMaxSF + 6 * (kMaxLayers + 1) * kMaxNodes));
    s.scal = (double *)take(8 * 4);
    return s;
}

// network forward (h, z) and optional tangent (hd, zd) for one atom, lanes = nodes
template <typename R>
__device__ void net_forward(const NNDev &M, const R *we, int ei, R *z, R *h, R *zd, R *hd, bool tangent) {
    const int lane = threadIdx.x & 31;
    for (int l = 1; l <= M.nlayers; ++l) {
        const int nprev = M.nodes[ei][l - 1], ncur = M.nodes[ei][l];
        const R *wl = we + M.woff[ei][l];
        for (int n = lane; n < ncur; n += 32) {
            R a = R(0), ad = R(0);
            for (int p = 0; p < nprev; ++p) {
                const R w = wl[p * ncur + n];
                a += w * h[(l - 1) * kMaxNodes + p];
                if (tangent) ad += w * hd[(l - 1) * kMaxNodes + p];
            }
            a += wl[nprev * ncur + n];
            const uint8_t ac = M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n];
            const R v = act_fn<R>(ac, a);
            z[l * kMaxNodes + n] = a;
            h[l * kMaxNodes + n] = v;
            if (tangent) {
                zd[l * kMaxNodes + n] = ad;
                hd[l * kMaxNodes + n] = act_dfn<R>(ac, a, v) * ad;
            }
        }
        __syncwarp();
    }
}

template <typename R>
__global__ void __launch_bounds__(32 * TrainCfg<R>::warps) train_kernel(Batch B, NNDev M, NNScratch X, TrainDev D,
                                                                        int max_atoms, int ngeta, int *counter) {
    constexpr int W = TrainCfg<R>::warps;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int work_slot;
    SmemTrain<R> S = carve_train<R>(smem_raw, M, max_atoms, ngeta);
    const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, lane = tid & 31;
    const size_t nw = (size_t)M.nelem * M.maxweights;
    for (size_t k = tid; k < nw; k += nt) S.w[k] = (R)D.theta[k];
    for (size_t k = tid; k < nw * W; k += nt) S.gradw[k] = R(0);
    WarpCache<R> C{S.nb + (size_t)warp * M.maxnb * S.stride, S.slotf + (size_t)warp * M.maxnb * 3,
                   S.nbatom + warp * M.maxnb, S.nbelem + warp * M.maxnb, S.stride};
    R *wb = S.buf + (size_t)warp * (2 * kMaxSF + 6 * (kMaxLayers + 1) * kMaxNodes);
    R *cv = wb + kMaxSF;
    const int LN = (kMaxLayers + 1) * kMaxNodes;
    R *z = wb + 2 * kMaxSF, *h = z + LN, *zd = h + LN, *hd = zd + LN, *dl = hd + LN, *dp = dl + LN;
    R *gw = S.gradw + nw * warp;
    const R cF = (R)(kHa2eVt / kBohr2Ang);  // Ha/bohr -> eV/A
    for (;;) {
        if (tid == 0) work_slot = atomicAdd(counter, 1);
        __syncthreads();
        const int wk = work_slot;
        __syncthreads();
        if (wk >= D.nconf) break;
        const int t = D.conf[wk];
        const int N = B.natoms[t];
        const int64_t base = B.ba_off[t];
        const int aoff = B.atom_off[t];
        if (tid == 0) acsf_lattice(B.box + 9 * t, S.lat);
        __syncthreads();
        for (int i = tid; i < N; i += nt) {
            acsf_wrap_one(B.rx[base + i], B.ry[base + i], B.rz[base + i], S.lat, S.px[i], S.py[i], S.pz[i]);
            S.elem[i] = (int8_t)M.elem_of_type[B.type[aoff + i]];
            S.fx[i] = R(0);
            S.fy[i] = R(0);
            S.fz[i] = R(0);
        }
        __syncthreads();
        // ---- pass A: energies and forces --------------------------------------------
        double e_warp = 0.0;
        for (int i = warp; i < N; i += W) {
            const int ei = S.elem[i];
            if (ei < 0) continue;
            const int cnt = X.nbcnt[base + i];
            const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
            const R *we = S.w + (size_t)ei * M.maxweights;
            acsf_cache<R>(M, C, i, ei, cnt, X.nbw + (base + i) * (int64_t)M.maxnb, S.px, S.py, S.pz, S.elem, S.lat);
            if (D.dgin) {  // the network ran outside: its output and dE/dG
                if (lane == 0)
                    e_warp += D.eatin[base + i] + (M.remove_atom_energies ? M.atom_energy[ei] : 0.0);
                for (int s = lane; s < nsf; s += 32) cv[s] = (R)D.dgin[(base + i) * M.maxsf + s];
                __syncwarp();
            } else {
                for (int s = lane; s < nsf; s += 32) {
                    const double mn = M.smin[sfb + s], w = M.smax[sfb + s] - mn;
                    h[s] = (R)((D.G[(base + i) * M.maxsf + s] - mn) / w * (M.scmax - M.scmin) + M.scmin);
                }
                __syncwarp();
                net_forward<R>(M, we, ei, z, h, zd, hd, false);
                if (lane == 0) e_warp += (double)h[M.nlayers * kMaxNodes] + (M.remove_atom_energies ? M.atom_energy[ei] : 0.0);
                for (int l = M.nlayers; l >= 1; --l) {
                    const int ncur = M.nodes[ei][l];
                    for (int n = lane; n < ncur; n += 32) {
                        const uint8_t ac = M.act[(ei * kMaxLayers + (l - 1)) * kMaxNodes + n];
                        const R dn = act_dfn<R>(ac, z[l * kMaxNodes + n], h[l * kMaxNodes + n]);
                        R up = R(1);
                        if (l < M.nlayers) {
                            const int nn = M.nodes[ei][l + 1];
                            const R *wl = we + M.woff[ei][l + 1];
                            up = R(0);
                            for (int m = 0; m < nn; ++m) up += wl[n * nn + m] * dl[(l + 1) * kMaxNodes + m];
                        }
                        dl[l * kMaxNodes + n] = dn * up;
                    }
                    __syncwarp();
                }
                {
                    const int n1 = M.nodes[ei][1];
                    const R *wl = we + M.woff[ei][1];
                    for (int s = lane; s < nsf; s += 32) {
                        R v = R(0);
                        for (int n = 0; n < n1; ++n) v += wl[s * n1 + n] * dl[1 * kMaxNodes + n];
                        cv[s] = v * (R)((M.scmax - M.scmin) / (M.smax[sfb + s] - M.smin[sfb + s]));
                    }
                }
                __syncwarp();
            }  // network in this kernel
            R fix, fiy, fiz;
            acsf_vjp<R>(M, C, ei, cnt, cv, fix, fiy, fiz);
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
        const double epred = block_sum(e_warp, S.red) * kHa2eVt;  // eV
        // ---- loss and adjoints ---------------------------------------------------------
        double fsq = 0.0;
        for (int i = tid; i < N; i += nt) {
            const int64_t k = base + i;
            const double dx = (double)(S.fx[i] * cF) - D.fx_ref[k], dy = (double)(S.fy[i] * cF) - D.fy_ref[k],
                         dz = (double)(S.fz[i] * cF) - D.fz_ref[k];
            fsq += dx * dx + dy * dy + dz * dz;
            const double g = 2.0 * D.wF / (3.0 * N) * (double)cF;  // dL/dF in Ha/bohr units
            S.ux[i] = (R)(g * dx);
            S.uy[i] = (R)(g * dy);
            S.uz[i] = (R)(g * dz);
        }
        fsq = block_sum(fsq, S.red);
        if (tid == 0) {
            const double de = (epred - D.E_ref[t]) / N;
            S.scal[0] = 2.0 * D.wE * de / N * kHa2eVt;  // dL/dE_i for every atom (Ha units)
            atomicAdd(&D.loss[0], de * de);
            atomicAdd(&D.loss[1], fsq);
            atomicAdd(&D.loss[2], 3.0 * N);
            atomicAdd(&D.loss[3], 1.0);
        }
        __syncthreads();
        const R a = (R)S.scal[0];
        // ---- pass B: JVP and the forward-over-reverse network sweep ---------------------
        for (int i = warp; i < N; i += W) {
            const int ei = S.elem[i];
            if (ei < 0) continue;
            const int cnt = X.nbcnt[base + i];
            const int nsf = M.nsf[ei], sfb = ei * M.maxsf;
            const R *we = S.w + (size_t)ei * M.maxweights;
            R *gwe = gw + (size_t)ei * M.maxweights;
            acsf_cache<R>(M, C, i, ei, cnt, X.nbw + (base + i) * (int64_t)M.maxnb, S.px, S.py, S.pz, S.elem, S.lat);
            acsf_jvp<R>(M, C, ei, cnt, i, S.ux, S.uy, S.uz, cv);
            if (D.xdot) {  // the network's sweep runs outside: its inputs
                for (int s = lane; s < nsf; s += 32) {
                    const double w = M.smax[sfb + s] - M.smin[sfb + s];
                    D.xdot[(base + i) * M.maxsf + s] = (float)(cv[s] * (R)((M.scmax - M.scmin) / w));
                }
                if (lane == 0) D.arow[base + i] = (double)a;
                __syncwarp();
                continue;
            }
            for (int s = lane; s < nsf; s += 32) {
                const double mn = M.smin[sfb + s], w = M.smax[sfb + s] - mn;
                const R sc = (R)((M.scmax - M.scmin) / w);
                h[s] = (R)((D.G[(base + i) * M.maxsf + s] - mn) / w * (M.scmax - M.scmin) + M.scmin);
                hd[s] = cv[s] * sc;
            }
            __syncwarp();
            net_forward<R>(M, we, ei, z, h, zd, hd, true);
            const int L = M.nlayers;
            if (lane == 0) {
                const uint8_t ac = M.act[(ei * kMaxLayers + (L - 1)) * kMaxNodes];
                dl[L * kMaxNodes] = act_dfn<R>(ac, z[L * kMaxNodes], h[L * kMaxNodes]);
                dp[L * kMaxNodes] = act_ddfn<R>(ac, z[L * kMaxNodes], h[L * kMaxNodes]) * zd[L * kMaxNodes];
            }
            __syncwarp();
            for (int l = L; l >= 1; --l) {
                const int ncur = M.nodes[ei][l], nprev = M.nodes[ei][l - 1];
                const int wo = M.woff[ei][l];
                for (int n = lane; n < ncur; n += 32) {
                    const R d = dl[l * kMaxNodes + n], d2 = dp[l * kMaxNodes + n];
                    for (int p = 0; p < nprev; ++p) {
                        const R hp = h[(l - 1) * kMaxNodes + p];
                        gwe[wo + p * ncur + n] += d * (a * hp + hd[(l - 1) * kMaxNodes + p]) + d2 * hp;
                    }
                    gwe[wo + nprev * ncur + n] += a * d + d2;
                }
                if (l > 1) {
                    const R *wl = we + wo;
                    for (int p = lane; p < nprev; p += 32) {
                        R gd = R(0), gp = R(0);
                        for (int n = 0; n < ncur; ++n) {
                            gd += wl[p * ncur + n] * dl[l * kMaxNodes + n];
                            gp += wl[p * ncur + n] * dp[l * kMaxNodes + n];
                        }
                        const uint8_t ac = M.act[(ei * kMaxLayers + (l - 2)) * kMaxNodes + p];
                        const R zz = z[(l - 1) * kMaxNodes + p], hh = h[(l - 1) * kMaxNodes + p];
                        const R s1 = act_dfn<R>(ac, zz, hh), s2 = act_ddfn<R>(ac, zz, hh);
                        dl[(l - 1) * kMaxNodes + p] = s1 * gd;
                        dp[(l - 1) * kMaxNodes + p] = s1 * gp + s2 * zd[(l - 1) * kMaxNodes + p] * gd;
                    }
                }
                __syncwarp();
            }
        }
        __syncthreads();
    }
    // ---- warp buffers -> global gradient --------------------------------------------
    __syncthreads();
    for (size_t k = tid; k < nw; k += nt) {
        double s = 0.0;
        for (int w2 = 0; w2 < W; ++w2) s += (double)S.gradw[nw * w2 + k];
        if (s != 0.0) atomicAdd(&D.grad[k], s);
    }
}

// Adam (Kingma & Ba, 2015) on the FP32 master weights; grad holds the batch sum.
__global__ void adam_kernel(float *theta, float *m, float *v, const double *grad, int n, double scale, double lr,
                            double b1, double b2, double eps, double bc1, double bc2, const uint8_t *frozen) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        if (frozen && frozen[k]) continue;
        const double g = grad[k] * scale;
        const double mk = b1 * m[k] + (1.0 - b1) * g;
        const double vk = b2 * v[k] + (1.0 - b2) * g * g;
        m[k] = (float)mk;
        v[k] = (float)vk;
        theta[k] = (float)(theta[k] - lr * (mk / bc1) / (sqrt(vk / bc2) + eps));
    }
}

__global__ void weights_to_model(const float *theta, float *wf, double *wd, int n) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        wf[k] = theta[k];
        wd[k] = (double)theta[k];
    }
}

size_t train_total_smem(const NNDev &M, int max_atoms, int ngeta, int precision) {
    return precision == 1 ? train_smem_bytes(max_atoms, M.maxnb, ngeta, M.nelem, M.maxweights, 4, 4)
                          : train_smem_bytes(max_atoms, M.maxnb, ngeta, M.nelem, M.maxweights, 8, 2);
}

cudaError_t launch_train(cudaStream_t s, int num_sms, const Batch &B, const NNDev &M, const NNScratch &X,
                         const TrainArgs &A, int max_atoms, int ngeta, int *counter, int precision) {
    TrainDev D{A.E_ref, A.fx_ref, A.fy_ref, A.fz_ref, A.G,    A.conf,  A.nconf, A.wE,  A.wF,
               A.theta, A.grad,   A.loss,   A.dgin,   A.eatin, A.xdot, A.arow};
    const size_t sm = train_total_smem(M, max_atoms, ngeta, precision);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    int per = 0;
    if (precision == 1) {
        e = cudaFuncSetAttribute(train_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, train_kernel<float>, 32 * TrainCfg<float>::warps, sm);
        const int grid = std::max(1, std::min(A.nconf, num_sms * std::max(per, 1)));
        train_kernel<float><<<grid, 32 * TrainCfg<float>::warps, sm, s>>>(B, M, X, D, max_atoms, ngeta, counter);
    } else {
        e = cudaFuncSetAttribute(train_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, train_kernel<double>, 32 * TrainCfg<double>::warps, sm);
        const int grid = std::max(1, std::min(A.nconf, num_sms * std::max(per, 1)));
        train_kernel<double><<<grid, 32 * TrainCfg<double>::warps, sm, s>>>(B, M, X, D, max_atoms, ngeta, counter);
    }
    return cudaGetLastError();
}

cudaError_t launch_adam(cudaStream_t s, float *theta, float *m, float *v, const double *grad, int n, double scale,
                        double lr, double b1, double b2, double eps, int step, const uint8_t *frozen) {
    const double bc1 = 1.0 - pow(b1, (double)step), bc2 = 1.0 - pow(b2, (double)step);
    adam_kernel<<<(n + 255) / 256, 256, 0, s>>>(theta, m, v, grad, n, scale, lr, b1, b2, eps, bc1, bc2, frozen);
    return cudaGetLastError();
}

cudaError_t launch_weights_to_model(cudaStream_t s, const float *theta, float *wf, double *wd, int n) {
    weights_to_model<<<(n + 255) / 256, 256, 0, s>>>(theta, wf, wd, n);
    return cudaGetLastError();
}

}  // namespace mdt
