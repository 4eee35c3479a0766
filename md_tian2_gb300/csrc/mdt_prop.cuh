// mdt_prop.cuh -- propagators (src/md_algo.f90, src/rpmd.f90) as CTA-level device
// functions, shared by every fused step kernel.
#pragma once
#include "mdt_common.cuh"
#include "mdt_emt.cuh"

namespace mdt {


// ---------------------------------------------------------------------------
// Propagators (src/md_algo.f90).  Thread per atom, all beads of the atom.
// ---------------------------------------------------------------------------
struct TrajView {
    int t, N, nb, aoff;
    int64_t base;
};

static __device__ __forceinline__ TrajView traj_view(const Batch &B, int t) {
    return TrajView{t, B.natoms[t], B.nbeads[t], B.atom_off[t], B.ba_off[t]};
}

static __device__ __forceinline__ double temp_of(const Batch &B, const PropParams &P, int ty) {
    return B.is_proj[ty] ? P.Tproj : P.Tsurf;
}

// Deviate for (bead b, atom i, dimension d).  Host-provided arrays use the reference's
// Fortran order (3, nb, N) per trajectory, concatenated.
static __device__ __forceinline__ double rand_normal(const PropParams &P, const TrajView &T, int step, int b, int i,
                                              int d, uint32_t stream, const double *injected) {
    if (P.rng_mode == 1) return injected[(T.base + (int64_t)i * T.nb + b) * 3 + d];
    return normal_deviate(P.seed, (uint32_t)T.t, (uint32_t)step, (uint32_t)((b * T.N + i) * 3 + d), stream);
}

static __device__ __forceinline__ double &comp(double *x, double *y, double *z, int d, int64_t k) {
    return d == 0 ? x[k] : (d == 1 ? y[k] : z[k]);
}

// collect_trajectory_characteristics after a step (trajectory_info.f90:47-263), by one
// thread: the lowest projectile centroid position, the closest approach `dmin` of this step
// (computed by the caller, with the index `near` of the nearest atom and the vector
// (rx, ry, rz) from the projectile to it, minimum image, any length unit) with the step at
// which it was first reached, the adsorption flag with its hysteresis, the steps with a
// projectile force, the bounce counters and a turning point whenever the sign of the
// centroid's z velocity changes.  near < 0: no atom in reach (the segment goes on).
// The observables' state of trajectory t is read once, up front (independent loads, one
// memory round trip), updated in registers and written back: the projectile's thread runs
// this between two CTA barriers, so its latency is the whole CTA's.
static __device__ void observe_core(const Batch &B, const PropParams &P, int t, int step, double dmin, int near,
                                    double rx, double ry, double rz, double x, double y, double z, double vx,
                                    double vy, double vz, double fx, double fy, double fz, bool force) {
    int *bn = B.obs_bnc + kObsInts * (size_t)t;
    double *dt = B.obs_dot + kObsDots * (size_t)t;
    const int cur = step & 1, last = cur ^ 1;
    const double low_z = B.obs_low[3 * t + 2], cl = B.obs_cl[t];
    const int up = B.obs_up[t], turn = B.obs_turn[t];
    int s[kObsInts];
#pragma unroll
    for (int k = 0; k < kObsInts; ++k) s[k] = bn[k];
    const double rv0 = dt[last], rf0 = dt[2 + last], vf0 = dt[4 + last];
    if (z < low_z) {
        B.obs_low[3 * t] = x;
        B.obs_low[3 * t + 1] = y;
        B.obs_low[3 * t + 2] = z;
    }
    if (dmin < cl) {
        B.obs_cl[t] = dmin;
        B.obs_clstep[t] = step;
    }
    // adsorption hysteresis (check_for_closest_approach, :127-129)
    if (!s[kObsAds] && dmin < P.ads_start) s[kObsAds] = 1;
    if (s[kObsAds] && dmin > P.ads_end) s[kObsAds] = 0;
    if (force) s[kObsInter] += 1;  // check_for_proj_surf_interaction (:140-148)
    // check_for_bounce (:152-241): unit vectors, dot products in the slot of this step
    if (near >= 0) {
        const double ir = 1.0 / sqrt(rx * rx + ry * ry + rz * rz), iv = 1.0 / sqrt(vx * vx + vy * vy + vz * vz),
                     iff = 1.0 / sqrt(fx * fx + fy * fy + fz * fz);
        const double rv1 = (rx * vx + ry * vy + rz * vz) * (ir * iv);
        const double rf1 = (rx * fx + ry * fy + rz * fz) * (ir * iff);
        const double vf1 = (vx * fx + vy * fy + vz * fz) * (iv * iff);
        dt[cur] = rv1;
        dt[2 + cur] = rf1;
        dt[4 + cur] = vf1;
        const int prev = s[kObsNear] < 0 ? near : s[kObsNear];
        if (prev != near) {
            s[kObsBounces] += min(s[kObsPtm], min(s[kObsRF], s[kObsVF]));  // finalize_bounces
            s[kObsPartner] = -s[kObsPartner];
            s[kObsRF] = s[kObsVF] = s[kObsPtm] = 0;
        } else if (rf1 != 0.0) {
            if ((rv0 > rf0 && rv1 < rf1) || (rv0 < rf0 && rv1 > rf1)) s[kObsRF] += 1;
            if ((rv0 > vf0 && rv1 < vf1) || (rv0 < vf0 && rv1 > vf1)) s[kObsVF] += 1;
            if (rv0 > 0.0 && rv1 < 0.0) s[kObsPtm] += 1;
        }
        s[kObsNear] = near;
    }
#pragma unroll
    for (int k = 0; k < kObsInts; ++k) bn[k] = s[k];
    const int down = vz < 0.0 ? 1 : 0;
    if (down == up) {  // moving down now and up before, or the reverse
        B.obs_turn[t] = turn + 1;
        B.obs_up[t] = 1 - down;
    }
}

static __device__ void observe_step(const Batch &B, const PropParams &P, const TrajView &T, int step, double dmin,
                                    int near, double rx, double ry, double rz) {
    double x = 0.0, y = 0.0, z = 0.0, vx = 0.0, vy = 0.0, vz = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
    bool force = false;
    for (int b = 0; b < T.nb; ++b) {
        const int64_t k = T.base + (int64_t)b * T.N;
        x += B.rx[k];
        y += B.ry[k];
        z += B.rz[k];
        vx += B.vx[k];
        vy += B.vy[k];
        vz += B.vz[k];
        fx += B.fx[k];
        fy += B.fy[k];
        fz += B.fz[k];
        force |= B.fx[k] != 0.0 || B.fy[k] != 0.0 || B.fz[k] != 0.0;
    }
    observe_core(B, P, T.t, step, dmin, near, rx, ry, rz, x / T.nb, y / T.nb, z / T.nb, vx, vy, vz, fx, fy, fz,
                 force);
}

// Closest approach of the projectile (atom 0) after a step: the minimum image of the
// centroids of atom 0 and atom i over i >= 1 (trajectory_info.f90:92-105), CTA-wide; every
// thread gets the distance, *near the nearest atom (first index on ties) and r the vector
// from the projectile to it (`cell` and `red` are shared-memory scratch).
static __device__ double closest_approach_step(const Batch &B, const TrajView &T, Cell *cell, double *red, int *near,
                                               double *r) {
    __syncthreads();
    if (threadIdx.x == 0) load_cell(B, T.t, *cell);
    __syncthreads();
    double c0x = 0.0, c0y = 0.0, c0z = 0.0;
    for (int b = 0; b < T.nb; ++b) {
        const int64_t k = T.base + (int64_t)b * T.N;
        c0x += B.rx[k];
        c0y += B.ry[k];
        c0z += B.rz[k];
    }
    c0x /= T.nb;
    c0y /= T.nb;
    c0z /= T.nb;
    double dmin = kDefaultReal;
    int imin = T.N;
    for (int i = 1 + threadIdx.x; i < T.N; i += blockDim.x) {
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int b = 0; b < T.nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            cx += B.rx[k];
            cy += B.ry[k];
            cz += B.rz[k];
        }
        double dx, dy, dz;
        min_image(*cell, c0x - cx / T.nb, c0y - cy / T.nb, c0z - cz / T.nb, dx, dy, dz);
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        if (d < dmin) {
            dmin = d;
            imin = i;
        }
    }
    const double best = block_min(dmin, red);
    const int ib = (int)block_min(dmin == best ? (double)imin : (double)T.N, red);
    *near = ib < T.N ? ib : -1;
    r[0] = r[1] = r[2] = 0.0;
    if (ib < T.N) {
        double cx = 0.0, cy = 0.0, cz = 0.0;
        for (int b = 0; b < T.nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + ib;
            cx += B.rx[k];
            cy += B.ry[k];
            cz += B.rz[k];
        }
        min_image(*cell, cx / T.nb - c0x, cy / T.nb - c0y, cz / T.nb - c0z, r[0], r[1], r[2]);
    }
    return best;
}

// verlet_1 / verlet_2, md_algo.f90:110-142
static __device__ void verlet_half(const Batch &B, const PropParams &P, const TrajView &T, int i, bool move_r) {
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
static __device__ void langevin_coef(double xi, double step, double temp, bool all_big, bool second, LangCoef &c) {
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

static __device__ __forceinline__ double friction(const Batch &B, const PropParams &P, int algo, int64_t k) {
    return algo == kPropLangevinConst ? P.gamma_const : B.dens[k];
}

static __device__ bool all_xidt_big(const Batch &B, const PropParams &P, const TrajView &T, int i, int algo) {
    bool all_big = true;
    for (int b = 0; b < T.nb; ++b)
        if (!(friction(B, P, algo, T.base + (int64_t)b * T.N + i) * P.step > (double)1e-2f)) all_big = false;
    return all_big;
}

// langevin_1, md_algo.f90:146-232
static __device__ void langevin_1(const Batch &B, const PropParams &P, const TrajView &T, int i, int step, int algo) {
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
static __device__ bool ldfa(const Batch &B, const TrajView &T, int i) {
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
static __device__ void langevin_2(const Batch &B, const PropParams &P, const TrajView &T, int i, int step, int algo) {
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
static __device__ void andersen(const Batch &B, const PropParams &P, const TrajView &T, int i, int step) {
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

// Per-type, per-mode tables of the ring-polymer propagators, kept in the CTA's shared
// normal-mode area right after the trajectory's nb x nb cjk table (the area holds
// kRpTables x kMaxTypes x max_beads more doubles): the free ring-polymer coefficients
// wk, cos(wk dt), sin(wk dt) of rpmd.f90:360-378 and the PILE damping c1, c2 of
// md_algo.f90:461-466.  They depend on the type's temperature, nb, dt and pile_tau, not on
// the atom, so a CTA forms them once per call instead of once per atom and dimension (an
// FP64 sin, cos or exp is tens of instructions on the FP64 pipe, the GPU's slowest); the
// expressions are the per-atom ones.
enum { kRpWk, kRpCw, kRpSw, kRpC1, kRpC2, kRpTables };
static_assert(kRpTables * kMaxTypes * 1 + 1 == rp_cells(1), "rp_cells sizes the tables");
static __device__ __forceinline__ double *rp_table(double *cjk, int nb, int which) {
    return cjk + nb * nb + which * kMaxTypes * nb;
}

static __device__ void pile_tables(const Batch &B, const PropParams &P, const TrajView &T, double *cjk) {
    const int nb = T.nb;
    double *c1t = rp_table(cjk, nb, kRpC1), *c2t = rp_table(cjk, nb, kRpC2);
    for (int w = threadIdx.x; w < B.ntypes * nb; w += blockDim.x) {
        const int ty = w / nb, kk = w - ty * nb;
        const double betaN = 1.0 / (kBoltz * temp_of(B, P, ty) * nb);
        double gam;
        if (kk == 0) gam = 1 / P.pile_tau;
        else gam = 2 * (2 * (1 / betaN / kHbar) * sin(kk * kPi / nb));
        const double c1 = exp(-0.5 * P.step * gam);
        c1t[w] = c1;
        c2t[w] = sqrt(1 - c1 * c1);
    }
    __syncthreads();
}

// Normal-mode transforms with the table cjk(j, m) (column major: cjk[m nb + j - 1], beads
// j = 1..nb, modes m = 0..nb-1).  nm_forward: y_m = sum_j x_j cjk(j, m); nm_back:
// x_j = sum_m y_m cjk(j, m).  For an even nb >= 4 the table's symmetry halves the products:
// cjk(nb - j, m) = cjk(j, m) for m <= nb/2 (cosines, the constant and the alternating
// mode) and -cjk(j, m) for m > nb/2 (sines), j = 1..nb/2-1; beads nb/2 and nb pair with
// themselves and carry no sine modes (their sine entries are zero up to the rounding of
// the table).  The sums are the reference's matrix products in another order.
static __device__ __forceinline__ void nm_forward(const double *cjk, int nb, const double *x, double *y) {
    if ((nb & 1) || nb < 4) {
        for (int m = 0; m < nb; ++m) {
            double s = 0.0;
            for (int k = 0; k < nb; ++k) s = s + x[k] * cjk[m * nb + k];
            y[m] = s;
        }
        return;
    }
    const int h = nb / 2;
    double sp[16], sm[16];  // x_j + x_(nb-j), x_j - x_(nb-j) at j - 1 (nb <= 32)
    for (int j = 1; j < h; ++j) {
        sp[j - 1] = x[j - 1] + x[nb - j - 1];
        sm[j - 1] = x[j - 1] - x[nb - j - 1];
    }
    for (int m = 0; m <= h; ++m) {
        const double *c = cjk + m * nb;
        double s = c[h - 1] * x[h - 1] + c[nb - 1] * x[nb - 1];
        for (int j = 1; j < h; ++j) s = s + c[j - 1] * sp[j - 1];
        y[m] = s;
    }
    for (int m = h + 1; m < nb; ++m) {
        const double *c = cjk + m * nb;
        double s = 0.0;
        for (int j = 1; j < h; ++j) s = s + c[j - 1] * sm[j - 1];
        y[m] = s;
    }
}

static __device__ __forceinline__ void nm_back(const double *cjk, int nb, const double *y, double *x) {
    if ((nb & 1) || nb < 4) {
        for (int b = 0; b < nb; ++b) {
            double s = 0.0;
            for (int m = 0; m < nb; ++m) s = s + y[m] * cjk[m * nb + b];
            x[b] = s;
        }
        return;
    }
    const int h = nb / 2;
    for (int j = 1; j < h; ++j) {
        double a = 0.0, c = 0.0;
        for (int m = 0; m <= h; ++m) a = a + y[m] * cjk[m * nb + j - 1];
        for (int m = h + 1; m < nb; ++m) c = c + y[m] * cjk[m * nb + j - 1];
        x[j - 1] = a + c;
        x[nb - j - 1] = a - c;
    }
    double a = 0.0, c = 0.0;
    for (int m = 0; m <= h; ++m) {
        a = a + y[m] * cjk[m * nb + h - 1];
        c = c + y[m] * cjk[m * nb + nb - 1];
    }
    x[h - 1] = a;
    x[nb - 1] = c;
}

// pile_thermostat, md_algo.f90:440-502 (one thread per atom, all three dimensions; the
// per-type, per-mode damping from pile_tables)
static __device__ void pile(const Batch &B, const PropParams &P, const TrajView &T, double *cjk, int i, int step) {
    const int nb = T.nb;
    const int ty = B.type[T.aoff + i];
    const double m = B.mass[T.aoff + i];
    const double betaN = 1.0 / (kBoltz * temp_of(B, P, ty) * nb);
    const double sq = sqrt(m / betaN);
    const double *c1t = rp_table(cjk, nb, kRpC1) + ty * nb, *c2t = rp_table(cjk, nb, kRpC2) + ty * nb;
    for (int d = 0; d < 3; ++d) {
        double newP[32], atomP[32];
        for (int b = 0; b < nb; ++b) atomP[b] = m * comp(B.vx, B.vy, B.vz, d, T.base + (int64_t)b * T.N + i);
        nm_forward(cjk, nb, atomP, newP);
        for (int kk = 0; kk < nb; ++kk) {
            const double z = rand_normal(P, T, step, kk, i, d, kStreamPile, P.zeta);
            newP[kk] = c1t[kk] * newP[kk] + sq * c2t[kk] * z;
        }
        nm_back(cjk, nb, newP, atomP);
        for (int b = 0; b < nb; ++b) {
            const int64_t k = T.base + (int64_t)b * T.N + i;
            comp(B.vx, B.vy, B.vz, d, k) = (B.fixed[k] >> d & 1) ? 0.0 : atomP[b] / m;
        }
    }
}

// remove_com_velocity, universe_mod.f90:222-241.  Its 1000 subtraction sweeps have the
// closed form v -= v_cm0 * N * (1 - (1 - 1/N)^1000), applied to every bead-atom.
static __device__ void remove_com(const Batch &B, const TrajView &T, double *red) {
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

static __device__ bool traj_has_algo(const Batch &B, int id) {
    for (int ty = 0; ty < B.ntypes; ++ty)
        if (B.algo[ty] == id) return true;
    return false;
}

// propagate_1, md_algo.f90:37-76
static __device__ void propagate_1(const Batch &B, const PropParams &P, const TrajView &T, double *cjk, int step,
                            double *red) {
    if (traj_has_algo(B, kPropPile)) pile_tables(B, P, T, cjk);
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
static __device__ void propagate_2(const Batch &B, const PropParams &P, const TrajView &T, int step) {
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

// do_ring_polymer_step, rpmd.f90:309-452.  Thread per (atom, dimension); the free
// ring-polymer coefficients per type and mode in the table after cjk.
static __device__ void ring_polymer_step(const Batch &B, const PropParams &P, const TrajView &T, double *cjk) {
    const int nb = T.nb;
    const double prefactor = -1 * B.mass[T.aoff] * pow(kBoltz * P.Tproj * nb / kHbar, 2.0);
    const double piN = kPi / nb;
    double *wkt = rp_table(cjk, nb, kRpWk), *cwt = rp_table(cjk, nb, kRpCw), *swt = rp_table(cjk, nb, kRpSw);
    for (int w = threadIdx.x; w < B.ntypes * nb; w += blockDim.x) {
        const int ty = w / nb, b = w - ty * nb;
        double wk = 0.0, cw = 1.0, sw = 0.0;
        if (nb > 1 && b > 0) {
            const double betaN = 1.0 / (kBoltz * temp_of(B, P, ty) * nb);
            const double twown = 2.0 / betaN / kHbar;
            const int bb = (b <= nb / 2) ? b : nb - b;
            wk = twown * sin(bb * piN);
            const double wt = wk * P.step;
            cw = cos(wt);
            sw = sin(wt);
        }
        wkt[w] = wk;
        cwt[w] = cw;
        swt[w] = sw;
    }
    __syncthreads();
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
        nm_forward(cjk, nb, p, np);
        nm_forward(cjk, nb, q, nq);
        for (int b = 0; b < nb; ++b) {
            double c0 = 1.0, c1 = 0.0, c2 = P.step / m, c3 = 1.0;
            if (nb > 1 && b > 0) {
                const double wm = wkt[ty * nb + b] * m;
                const double cw = cwt[ty * nb + b], sw = swt[ty * nb + b];
                c0 = cw; c1 = -wm * sw; c2 = sw / wm; c3 = cw;
            }
            const double pn = np[b] * c0 + nq[b] * c1;
            nq[b] = np[b] * c2 + nq[b] * c3;
            np[b] = pn;
        }
        const int algo = B.algo[ty];
        const bool revert = (algo == kPropLangevin || algo == kPropLangevinConst);
        if (!revert) {
            // back to beads (p and q reused); v = sum_k p_k cjk(b,k) / m with the division
            // after the sum (one FP64 division per bead instead of per term)
            nm_back(cjk, nb, nq, q);
            nm_back(cjk, nb, np, p);
            for (int b = 0; b < nb; ++b) {
                const int64_t k = T.base + (int64_t)b * T.N + i;
                if (B.fixed[k] >> d & 1) continue;
                comp(B.rx, B.ry, B.rz, d, k) = q[b];
                comp(B.vx, B.vy, B.vz, d, k) = p[b] / m;
            }
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

// End of one fused MD step of the CTA that owns trajectory T (md_tian2.f90:78-92): the step
// count, the exit test on the projectile's beads, the step limit, and retirement of a
// trajectory whose state stopped being finite.  The reference has no such check (a NaN
// propagates until the run ends); here every bead-atom's position and velocity is
// tested after the step, and a broken trajectory stops with kStatusErrNonFinite while the
// others of the batch go on untouched.  An error status already set (ldfa's negative
// density) is kept.
static __device__ void end_of_step(const Batch &B, const PropParams &P, const TrajView &T, int step) {
    int bad = 0;
    const int tot = T.N * T.nb;
    for (int s = threadIdx.x; s < tot; s += blockDim.x) {
        const int64_t k = T.base + s;
        const double a = (B.rx[k] + B.ry[k]) + (B.rz[k] + B.vx[k]) + (B.vy[k] + B.vz[k]);
        bad |= isfinite(a) ? 0 : 1;
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        const int t = T.t;
        B.steps_done[t] = step;
        if (bad && B.status[t] == kStatusRunning) B.status[t] = kStatusErrNonFinite;
        if (P.use_exit && B.is_proj[B.type[T.aoff]] && B.status[t] == kStatusRunning) {
            bool up = true, lo = true;
            for (int b = 0; b < T.nb; ++b) {
                const double z = B.rz[T.base + (int64_t)b * T.N];
                up = up && (z > P.pul);
                lo = lo && (z < P.pll);
            }
            if (up) B.status[t] = kStatusExitUpper;
            else if (lo) B.status[t] = kStatusExitLower;
        }
        if (P.max_steps > 0 && step >= P.max_steps && B.status[t] == kStatusRunning) B.status[t] = kStatusStepLimit;
    }
    __syncthreads();
}

static __device__ void load_cjk(const Batch &B, int t, double *cjk_s) {
    const int nb = B.nbeads[t];
    const double *src = B.cjk + B.cjk_off[t];
    for (int k = threadIdx.x; k < nb * nb; k += blockDim.x) cjk_s[k] = src[k];
    __syncthreads();
}

}  // namespace mdt
