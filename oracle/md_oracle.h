/*
 * md_oracle.h -- CPU FP64 restatement of the md_tian2 force/propagation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA engine
 * (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg).  Nothing in
 * the product path (md_tian2_gb300/, libmdt_gpu.so) links or calls it.
 *
 * Parity status: unpinned by the reference itself.  The reference is Fortran and no
 * Fortran compiler exists in the build environment, so no reference run produced
 * golden vectors.  The restatement is checked instead against (a) the reference's own
 * parameter fixtures (pes/EMT-*.pes), (b) its binary geometry fixtures
 * (conf/latt/mxt_00000001.dat and siblings), (c) analytic properties (finite-difference
 * gradients, Newton's third law, NVE conservation, the force-sum rule of check_forces) and
 * (d) a second, independent restatement of the EMT and RuNNer energies in torch FP64
 * (tests/test_cpu_oracle_autodiff.py, with its own neighbour search), whose energies equal
 * this oracle's and whose autograd forces equal this oracle's hand-derived forces; the one
 * place they must differ, the reference's H-H density-derivative quirk, they do.
 * tests/golden/runner_cgraphene_ref.npz holds this oracle's own output on the reference's
 * example network: a regression fixture, not an independent golden vector.
 *
 * Layout: every per-trajectory array is in the reference's Fortran order,
 * r(3, nbeads, natoms) -> r[(i*nb + b)*3 + d], exactly like `type universe`
 * (src/universe_mod.f90:38-67).  Types are 1-based like universe%idx.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* propagator ids, src/constants.f90:107-112 (1007 is this project's constant-friction
   Langevin, which has no reference counterpart) */
enum { ORC_VERLET = 1001, ORC_LANGEVIN = 1003, ORC_ANDERSEN = 1005, ORC_PILE = 1006,
       ORC_LANGEVIN_CONST = 1007 };

typedef struct orc_params {
    double step;            /* fs */
    double Tsurf, Tproj;    /* K */
    double pile_tau;        /* fs */
    double andersen_time;   /* fs */
    double gamma_const;     /* 1/fs, only for ORC_LANGEVIN_CONST */
} orc_params;

typedef struct orc_universe {
    int natoms, nbeads, ntypes;
    double *r, *v, *f, *a;          /* (3,nb,N) */
    double *m;                      /* (N) eV fs^2/A^2 */
    uint8_t *is_fixed;              /* (3,nb,N) */
    int32_t *idx;                   /* (N) 1-based */
    int32_t *pes;                   /* (ntypes,ntypes) column major, 2003 = EMT */
    int32_t *algo;                  /* (ntypes) */
    uint8_t *is_proj;               /* (ntypes) */
    double *epot;                   /* (nb) */
    double simbox[9], isimbox[9];   /* column major (3,3) */
    double *dens;                   /* (nb,N): dens(b,i) -> dens[i*nb + b] */
    /* EMT parameters per type (eta2,n0,e0,lambda,v0,kappa,s0) -> emt[t*7 + k] */
    double *emt;
} orc_universe;

/* minimum-image vector r_j - r_i and distance for all beads,
   src/universe_mod.f90:411-428 */
void orc_minimg_beads(const orc_universe *u, int i, int j, double *r, double *vec);

/* calc_force, src/force.f90:40-86 (EMT only; includes the free ring-polymer step
   for nbeads > 1 exactly like the reference) */
int orc_calc_force(orc_universe *u, const orc_params *p);

/* compute_emt dispatcher + 1/2-species bodies, src/pes_emt_mod.f90:194-1027.
   Expects u->f / u->epot already initialised; accumulates like the reference. */
int orc_compute_emt(orc_universe *u, const double *distances, const double *vectors);

/* propagate_1 / propagate_2, src/md_algo.f90:37-106.
   randy: (3,nb,N) normal deviates for Langevin (drawn once per step, reused in
   propagate_2); zeta: (3,nb,N) normal deviates for PILE; andersen_v: (3,nb,N) unit
   normal deviates (scaled inside); andersen_u: (nb,N) uniform numbers. */
int orc_propagate_1(orc_universe *u, const orc_params *p, const double *randy,
                    const double *zeta, const double *andersen_v, const double *andersen_u);
int orc_propagate_2(orc_universe *u, const orc_params *p, const double *randy);

/* do_ring_polymer_step, src/rpmd.f90:309-452 */
int orc_ring_polymer_step(orc_universe *u, const orc_params *p);

/* remove_com_velocity, src/universe_mod.f90:222-241 (1000 iterations, literal) */
void orc_remove_com_velocity(orc_universe *u);

/* energies: atom_ekin (universe_mod.f90:433-458), bead_ekin (rpmd.f90:547-572),
   calc_bead_epot (rpmd.f90:244-267) */
void orc_atom_ekin(const orc_universe *u, double *ekin_p, double *ekin_l);
void orc_bead_ekin(const orc_universe *u, double *ekin_p, double *ekin_l);
double orc_bead_epot(const orc_universe *u, const orc_params *p);

/* One full MD step: propagate_1, calc_force, propagate_2 (md_tian2.f90:81-83). */
int orc_md_step(orc_universe *u, const orc_params *p, const double *randy,
                const double *zeta, const double *andersen_v, const double *andersen_u);

/* Velocity-Verlet trajectory for the CPU baseline: runs up to nsteps steps, stopping
   when every bead of atom 1 is above pul (md_tian2.f90:78-92).  Returns steps done. */
int orc_run_verlet(orc_universe *u, const orc_params *p, int nsteps, double pul);

/* Steady-state stepping for the timed CPU baseline: MD steps (orc_md_step) over the n
   universes round robin, every universe one step per sweep, until `seconds` of wall time
   have passed (checked after each sweep) or max_sweeps sweeps are done.  The Langevin and
   thermostat deviates come from a counter generator (splitmix64, Box-Muller) keyed by
   seed, so no Python runs inside the timed loop.  Returns the atom-steps done (natoms x
   nbeads per universe-step); *elapsed receives the seconds spent.  Negative on error. */
int64_t orc_run_steps(orc_universe **u, int n, const orc_params *p, double seconds, int64_t max_sweeps,
                      uint64_t seed, double *elapsed);

#ifdef __cplusplus
}
#endif
