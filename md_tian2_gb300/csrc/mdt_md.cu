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
#include "mdt_emt.cuh"
#include "mdt_internal.h"
#include "mdt_prop.cuh"

namespace mdt {


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
        for (int s = 0; s < nsteps; ++s) {
            if (B.status[t] != kStatusRunning) break;
            const int step = B.steps_done[t] + 1;
            propagate_1(B, P, T, S.cjk, step, S.red);
            calc_force<R>(B, E, P, S, T, true);
            propagate_2(B, P, T, step);
            {
                int near;
                double rv[3];
                const double dmin = closest_approach_step(B, T, S.cell, S.red, &near, rv);
                if (threadIdx.x == 0) observe_step(B, P, T, step, dmin, near, rv[0], rv[1], rv[2]);
            }
            end_of_step(B, P, T, step);
        }
    }
}

// trajectory observables at their initial values (trajectory_info.f90:55-70)
// (the reference keeps is_adsorbed from the previous trajectory, trajectory_info.f90:55-70
// does not reset it; here every trajectory starts not adsorbed)
__device__ void obs_reset_traj(const Batch &B, int t) {
    B.obs_turn[t] = 0;
    B.obs_up[t] = 0;
    B.obs_clstep[t] = 0;
    B.obs_cl[t] = kDefaultReal;
    B.obs_low[3 * t] = kDefaultReal;
    B.obs_low[3 * t + 1] = kDefaultReal;
    B.obs_low[3 * t + 2] = kDefaultReal;
    int *bn = B.obs_bnc + kObsInts * (size_t)t;
    for (int k = 0; k < kObsInts; ++k) bn[k] = 0;
    bn[kObsNear] = -1;
    bn[kObsPartner] = 1;
    for (int k = 0; k < kObsDots; ++k) B.obs_dot[kObsDots * (size_t)t + k] = kDefaultReal;
}

__global__ void obs_reset_kernel(Batch B) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < B.ntraj; t += gridDim.x * blockDim.x)
        obs_reset_traj(B, t);
}

cudaError_t launch_obs_reset(cudaStream_t s, const Batch &B) {
    obs_reset_kernel<<<(B.ntraj + 255) / 256, 256, 0, s>>>(B);
    return cudaGetLastError();
}

// Refill of stopped trajectories (the set-up of md_init.f90 for the next trajectory,
// prepare_next_traj :880-944, on the device): every bead-atom of a trajectory that ended
// normally (status 1-3; trajectories with an error status keep their state and status)
// gets the state of the last upload back; then the projectile (atom 0) is moved the way
// apply_pip (:546-549) and set_proj_incidence (:829-876) move it: its bead centroid goes to
// a uniform direct (u, v) in the first two cell vectors at height z0 (r_b - centroid +
// target, so the ring polymer keeps its spread), and its bead velocities lose their mean
// (remove_atomic_com) and gain the incidence velocity for an energy, polar and azimuth
// drawn uniformly (Philox keyed by seed, trajectory and generation).
struct RefillDev {
    double z0, emin, emax, pmin, pmax, azimuth;  // azimuth < 0: uniform in [0, 360)
    uint64_t seed;
};

__device__ __forceinline__ bool refillable(int status) {
    return status == kStatusExitUpper || status == kStatusExitLower || status == kStatusStepLimit;
}

__global__ void refill_kernel(Batch B, const double *tmpl, int64_t total_ba, RefillDev R, int *gen, int *skok,
                              int *count, double *draws) {
    for (int t = blockIdx.x; t < B.ntraj; t += gridDim.x) {
        if (!refillable(B.status[t])) continue;  // uniform over the block
        const TrajView T = traj_view(B, t);
        const int64_t n = (int64_t)T.nb * T.N;
        double *dst[6] = {B.rx, B.ry, B.rz, B.vx, B.vy, B.vz};
        for (int64_t k = threadIdx.x; k < n; k += blockDim.x)
            for (int a = 0; a < 6; ++a) dst[a][T.base + k] = tmpl[a * total_ba + T.base + k];
        __syncthreads();
        if (threadIdx.x == 0) {
            const int g = gen[t] + 1;
            gen[t] = g;
            const uint32_t tt = (uint32_t)t, gg = (uint32_t)g;
            const double u = uniform_deviate(R.seed, tt, gg, 0, kStreamRefill);
            const double w = uniform_deviate(R.seed, tt, gg, 1, kStreamRefill);
            const double e = R.emin + (R.emax - R.emin) * uniform_deviate(R.seed, tt, gg, 2, kStreamRefill);
            const double pol_deg = R.pmin + (R.pmax - R.pmin) * uniform_deviate(R.seed, tt, gg, 3, kStreamRefill);
            const double pol = pol_deg * (kPi / 180.0);
            const double azi_deg = R.azimuth < 0.0 ? 360.0 * uniform_deviate(R.seed, tt, gg, 4, kStreamRefill)
                                                   : R.azimuth;
            const double azi = azi_deg * (kPi / 180.0);
            double *dr = draws + 5 * (size_t)t;
            dr[0] = u;
            dr[1] = w;
            dr[2] = e;
            dr[3] = pol_deg;
            dr[4] = azi_deg;
            const double *h = B.box + 9 * (size_t)t;  // column major: h[3 k + d] = component d of vector k
            const double target[3] = {h[0] * u + h[3] * w, h[1] * u + h[4] * w, R.z0};
            const double vinc = sqrt(2.0 * e / B.mass[T.aoff]);
            const double vi[3] = {vinc * sin(pol) * cos(azi), vinc * sin(pol) * sin(azi), -vinc * cos(pol)};
            double *r[3] = {B.rx, B.ry, B.rz}, *v[3] = {B.vx, B.vy, B.vz};
            for (int d = 0; d < 3; ++d) {
                double cr = 0.0, cv = 0.0;
                for (int b = 0; b < T.nb; ++b) {
                    const int64_t k = T.base + (int64_t)b * T.N;
                    cr += r[d][k];
                    cv += v[d][k];
                }
                cr /= T.nb;
                cv /= T.nb;
                for (int b = 0; b < T.nb; ++b) {
                    const int64_t k = T.base + (int64_t)b * T.N;
                    r[d][k] = r[d][k] - cr + target[d];
                    v[d][k] = v[d][k] - cv + vi[d];
                }
            }
            if (skok)
                for (int b = 0; b < T.nb; ++b) skok[B.bead_off[t] + b] = 0;
            B.status[t] = kStatusRunning;
            B.steps_done[t] = 0;
            obs_reset_traj(B, t);
            atomicAdd(count, 1);
        }
        __syncthreads();
    }
}

cudaError_t launch_refill(cudaStream_t s, const Batch &B, const double *tmpl, int64_t total_ba, double z0,
                          double emin, double emax, double pmin, double pmax, double azimuth, uint64_t seed,
                          int *gen, int *skok, int *count, double *draws) {
    const RefillDev R{z0, emin, emax, pmin, pmax, azimuth, seed};
    const int grid = B.ntraj < 4096 ? (B.ntraj > 0 ? B.ntraj : 1) : 4096;
    refill_kernel<<<grid, 128, 0, s>>>(B, tmpl, total_ba, R, gen, skok, count, draws);
    return cudaGetLastError();
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

// A state upload in one pass: positions and velocities (each optional, null: kept) from
// their stage slices into the SoA arrays, and all six into the refill template.
__global__ void unpack_state_kernel(Batch B, const double *sr, const double *sv, double *tmpl, int64_t total_ba,
                                    const int *ba_traj) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total_ba;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[s];
        const int N = B.natoms[t];
        const int64_t loc = s - B.ba_off[t];
        const int b = (int)(loc / N), i = (int)(loc - (int64_t)b * N);
        const int64_t f = (B.ba_off[t] + (int64_t)i * B.nbeads[t] + b) * 3;
        double x, y, z;
        if (sr) {
            x = sr[f];
            y = sr[f + 1];
            z = sr[f + 2];
            B.rx[s] = x;
            B.ry[s] = y;
            B.rz[s] = z;
        } else {
            x = B.rx[s];
            y = B.ry[s];
            z = B.rz[s];
        }
        tmpl[s] = x;
        tmpl[total_ba + s] = y;
        tmpl[2 * total_ba + s] = z;
        if (sv) {
            x = sv[f];
            y = sv[f + 1];
            z = sv[f + 2];
            B.vx[s] = x;
            B.vy[s] = y;
            B.vz[s] = z;
        } else {
            x = B.vx[s];
            y = B.vy[s];
            z = B.vz[s];
        }
        tmpl[3 * total_ba + s] = x;
        tmpl[4 * total_ba + s] = y;
        tmpl[5 * total_ba + s] = z;
    }
}

// A state download's packs in one pass: positions, velocities, forces, accelerations (each
// optional, null: skipped) into their stage slices in the Fortran-order host layout.
__global__ void pack_state_kernel(Batch B, double *dr, double *dv, double *df, double *da, int64_t total_ba,
                                  const int *ba_traj) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < total_ba;
         s += (int64_t)gridDim.x * blockDim.x) {
        const int t = ba_traj[s];
        const int N = B.natoms[t];
        const int64_t loc = s - B.ba_off[t];
        const int b = (int)(loc / N), i = (int)(loc - (int64_t)b * N);
        const int64_t f = (B.ba_off[t] + (int64_t)i * B.nbeads[t] + b) * 3;
        if (dr) {
            dr[f] = B.rx[s];
            dr[f + 1] = B.ry[s];
            dr[f + 2] = B.rz[s];
        }
        if (dv) {
            dv[f] = B.vx[s];
            dv[f + 1] = B.vy[s];
            dv[f + 2] = B.vz[s];
        }
        if (df) {
            df[f] = B.fx[s];
            df[f + 1] = B.fy[s];
            df[f + 2] = B.fz[s];
        }
        if (da) {
            da[f] = B.ax[s];
            da[f + 1] = B.ay[s];
            da[f + 2] = B.az[s];
        }
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

cudaError_t launch_unpack_state(cudaStream_t s, const Batch &B, const double *sr, const double *sv, double *tmpl,
                                int64_t total_ba, const int *ba_traj) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    unpack_state_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(B, sr, sv, tmpl, total_ba, ba_traj);
    return cudaGetLastError();
}

cudaError_t launch_pack_state(cudaStream_t s, const Batch &B, double *dr, double *dv, double *df, double *da,
                              int64_t total_ba, const int *ba_traj) {
    const int grid = (int)std::min<int64_t>((total_ba + 255) / 256, 4096);
    pack_state_kernel<<<grid > 0 ? grid : 1, 256, 0, s>>>(B, dr, dv, df, da, total_ba, ba_traj);
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
