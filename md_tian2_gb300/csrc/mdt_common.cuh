// mdt_common.cuh -- shared device-side definitions of the md_tian2 GB300 engine.
//
// Data layout in HBM (structure of arrays, ragged):
//   trajectory t owns natoms[t] atoms and nbeads[t] beads.  A bead-atom (b, i) of t
//   lives at slot ba = ba_off[t] + b*natoms[t] + i (bead-major, so one bead's atoms are
//   contiguous and a CTA can stage a bead with coalesced loads).  Positions,
//   velocities, accelerations and forces are separate FP64 x/y/z arrays indexed by ba.
//   Per-atom data (mass, type) is indexed by atom_off[t] + i, per-bead data (epot) by
//   bead_off[t] + b, per-trajectory data (cell, status) by t.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mdt {

constexpr int kMaxTypes = 4;

// src/constants.f90:30-39,157-170
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kSqrt2 = 1.41421356237309504880168872420969808;
constexpr double kSqrt3 = 1.73205080756887729352744634150587237;
constexpr double kBoltz = 8.61733238496e-5;   // eV/K
constexpr double kHbar = 0.6582119514467406;  // eV fs
constexpr double kTwelfth = 1.0 / 12.0;
constexpr double kTolerance = 1.0e-9;
constexpr double kBohr2Ang = 0.529177211;
constexpr double kDefaultReal = 1.7976931348623157e308;  // huge(0_dp), constants.f90:101
constexpr double kAmu2Mass = 103.638239276;

// propagator ids, src/constants.f90:107-112; 1007 = constant-friction Langevin
// (this engine's addition, no reference counterpart)
constexpr int kPropVerlet = 1001;
constexpr int kPropLangevin = 1003;
constexpr int kPropAndersen = 1005;
constexpr int kPropPile = 1006;
constexpr int kPropLangevinConst = 1007;

// trajectory status codes
constexpr int kStatusRunning = 0;
constexpr int kStatusExitUpper = 1;   // projectile above pul (md_tian2.f90:88-89)
constexpr int kStatusExitLower = 2;   // projectile below pll (md_tian2.f90:91-92)
constexpr int kStatusStepLimit = 3;   // nsteps reached (the loop of md_tian2.f90:78 completed)
constexpr int kStatusErrDensity = -10;  // ldfa: negative EMT density (md_algo.f90:551-554)
constexpr int kStatusErrNonFinite = -11;

// Derived EMT constants, computed on the host exactly like
// compute_emt_2species (src/pes_emt_mod.f90:521-592).  Species slot 0 is the
// reference's "type1" (first type with pes(i,i)==emt), slot 1 its "type2".
struct EmtConst {
    int nspecies;                 // 1 or 2
    int slot_of_type[kMaxTypes];  // universe type (0-based) -> species slot, -1 = not EMT
    uint32_t pair_mask;           // bit ti*kMaxTypes+tj set when pes(ti,tj) == emt
    int hh_quirk;                 // 2 species: slot-0/slot-0 derivative uses eta2 of slot 1
    double cut2;                  // (1.5*rcut)^2
    double cut;                   // 1.5*rcut
    double rcut, acut;
    double eta2[2], betas0[2], kappadbeta[2], betaeta2[2];
    double igamma1[2], g2v0[2];   // 1/gamma1, v0/gamma2
    double n0[2], e0[2], lambda[2], kappa[2], v0[2], dens_exp[2];
    double chi[2][2];             // density at a from neighbour b scaled by chi[a][b]
};

// Everything a kernel needs to address the batch.  Passed by value.
struct Batch {
    int ntraj;
    int ntypes;
    const int *natoms, *nbeads;
    const int64_t *ba_off;     // bead-atom slot offset per trajectory
    const int *atom_off;       // atom offset per trajectory
    const int *bead_off;       // bead offset per trajectory (epot)
    const int64_t *pair_off;   // pair-scratch slot offset per trajectory
    double *rx, *ry, *rz, *vx, *vy, *vz, *ax, *ay, *az, *fx, *fy, *fz;
    double *dens;              // per bead-atom
    double *epot;              // per bead
    const double *mass;        // per atom
    const int8_t *type;        // per atom, 0-based universe type
    const uint8_t *fixed;      // per bead-atom, bit d set when dimension d is frozen
    const double *box, *ibox;  // per trajectory, 9 doubles column major
    int *status;               // per trajectory
    int *steps_done;           // per trajectory
    const int *cjk_off;        // per trajectory: offset of its nbeads x nbeads table
    const double *cjk;         // normal-mode tables, column major cjk(j,k)
    void *pair_scratch;        // per pair slot: dx, dy, dz, Q_ij, Q_ji, F_V (FP64 or FP32)
    // trajectory observables of trajectory_info.f90 (projectile = atom 0), updated by the
    // fused MD kernels after every step: turning points of the centroid's z velocity, 1
    // while it moves up, closest approach to any other atom (A, minimum image of the
    // centroids) with the step it was first reached, lowest centroid position (3 per traj)
    int *obs_turn, *obs_up, *obs_clstep;
    double *obs_cl, *obs_low;
    // bounce detection and adsorption of trajectory_info.f90:80-263, per trajectory: ints
    // [kObsNear] nearest atom of the last step (-1: none yet), [kObsRF] r.v x r.F crossings,
    // [kObsVF] r.v x v.F crossings, [kObsPtm] r.v + to - changes, [kObsBounces] closed
    // segments' bounces, [kObsPartner] partner-change sign, [kObsInter] steps with a
    // projectile force, [kObsAds] adsorbed; doubles: r.v, r.F, v.F of the two last steps
    int *obs_bnc;
    double *obs_dot;
    int max_atoms, max_beads;
    int algo[kMaxTypes];       // propagator per type
    int is_proj[kMaxTypes];
};

enum { kObsNear, kObsRF, kObsVF, kObsPtm, kObsBounces, kObsPartner, kObsInter, kObsAds, kObsInts };
constexpr int kObsDots = 6;

struct PropParams {
    double step, Tsurf, Tproj, pile_tau, andersen_time, gamma_const;
    double ads_start, ads_end;  // adsorption hysteresis (A): adsorbed below start, free above end
    double pul, pll;          // exit limits (use +/-inf to disable)
    uint64_t seed;
    int use_exit;             // stop trajectories at pul / pll
    int rng_mode;             // 0 = counter-based Philox, 1 = host-provided arrays
    int max_steps;            // > 0: a trajectory stops after this many steps (nsteps)
    const double *randy;      // rng_mode 1: (ba, d) normal deviates for Langevin
    const double *zeta;       // rng_mode 1: PILE deviates
    const double *andersen_v; // rng_mode 1: Andersen unit deviates
    const double *andersen_u; // rng_mode 1: Andersen uniforms (per ba)
};

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// uniform in (0, 1] with 53 random bits
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
    const uint64_t v = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);  // 27 + 26 bits
    return ((double)v + 1.0) * (1.0 / 9007199254740992.0);
}

// One N(0,1) deviate per (key, counter) by the Box-Muller form the reference uses
// (useful_things.f90:121-173: sqrt(-2 ln u1) cos(2 pi u2)), evaluated in FP32: on this
// GPU FP64 runs at 1/64 of FP32, and the thermostat noise needs no more than 24-bit
// uniforms (u1 in (0, 1]: tails end at sqrt(2 ln 2^24) = 5.77 sigma).
__device__ __forceinline__ double normal_deviate(uint64_t seed, uint32_t traj, uint32_t step,
                                                 uint32_t slot, uint32_t stream) {
    U4 r = philox4x32_10(U4{step, slot, stream, traj}, (uint32_t)seed, (uint32_t)(seed >> 32));
    const float u1 = (float)((r.x >> 8) + 1u) * (1.0f / 16777216.0f);
    const float u2 = (float)(r.z >> 8) * (1.0f / 16777216.0f);
    return (double)(sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2));
}

__device__ __forceinline__ double uniform_deviate(uint64_t seed, uint32_t traj, uint32_t step,
                                                  uint32_t slot, uint32_t stream) {
    U4 r = philox4x32_10(U4{step, slot, stream, traj}, (uint32_t)seed, (uint32_t)(seed >> 32));
    return u01_53(r.x, r.y) - (1.0 / 9007199254740992.0);  // [0, 1)
}

enum RngStream : uint32_t { kStreamLangevin = 1, kStreamPile = 2, kStreamAndersenV = 3,
                            kStreamAndersenU = 4, kStreamRefill = 5 };

}  // namespace mdt
