"""GPU parity of the propagators (src/md_algo.f90, src/rpmd.f90) against the oracle.

Stochastic propagators take identical host-provided deviates on both sides (the
reference draws from the compiler's intrinsic generator, which cannot be reproduced),
so one step agrees to round-off: positions/velocities within 1e-10."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams

from .helpers import flat, injected, make_engine, max_abs, oracle_list

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _batch(algo_p, algo_l, nbeads=(1,), metal="Au", n=4, seed=0, z0=2.0):
    rng = np.random.default_rng(seed)
    us = []
    for t in range(n):
        nb = nbeads[t % len(nbeads)]
        k = 3 + t % 2
        u = W.h_on_metal(rng, metal, k, rng.uniform(0.5, 3), rng.uniform(0, 60), rng.uniform(0, 360), 300.0,
                         algo_p, algo_l, z0=z0, nbeads=nb)
        if nb > 1:
            u.r += rng.normal(scale=0.02, size=u.r.shape) * (~u.is_fixed)
        us.append(u)
    return us


def _step_both(us, emt, sp, steps=1, fused=False, seed=1):
    rng = np.random.default_rng(seed)
    eng = make_engine(us, emt)
    orcs = oracle_list(us, emt)
    sp_inj = SimParams(**{**sp.__dict__, "rng_mode": 1})
    # initial forces (md_tian2.f90:69)
    eng.calc_force(sp)
    for o in orcs:
        o.calc_force(sp)
    for _ in range(steps):
        randy, zeta, av, au = injected(us, rng)
        eng.set_random_arrays(flat(randy), flat(zeta), flat(av), flat(au))
        if fused:
            eng.md_steps(1, sp_inj)
        else:
            eng.propagate_1(sp_inj)
            eng.calc_force(sp_inj)
            eng.propagate_2(sp_inj)
        for t, o in enumerate(orcs):
            sh = o.r.shape
            o.propagate_1(sp, randy[t].reshape(sh), zeta[t].reshape(sh), av[t].reshape(sh),
                          au[t].reshape(sh[:2]))
            o.calc_force(sp)
            o.propagate_2(sp, randy[t].reshape(sh))
    out = eng.download()
    eng.close()
    ref = {k: np.concatenate([getattr(o, k).reshape(-1) for o in orcs]) for k in ("r", "v", "f", "a")}
    ref["dens"] = np.concatenate([o.dens.reshape(-1) for o in orcs])
    return out, ref


@pytest.mark.parametrize("fused", [False, True])
def test_verlet(built_lib, oracle_lib, fused):
    us = _batch(C.PROP_ID_VERLET, C.PROP_ID_VERLET)
    out, ref = _step_both(us, W.emt_params(), SimParams(step=0.1), steps=3, fused=fused)
    for k in ("r", "v", "a"):
        assert max_abs(out[k], ref[k]) < TOL, k


@pytest.mark.parametrize("fused", [False, True])
def test_langevin_ldfa(built_lib, oracle_lib, fused):
    # H with LDFA friction, Au with LDFA friction too (the reference applies ldfa to
    # every atom whose algorithm is 'lan')
    us = _batch(C.PROP_ID_LANGEVIN, C.PROP_ID_LANGEVIN, z0=1.5)
    out, ref = _step_both(us, W.emt_params(), SimParams(step=0.1, Tsurf=300, Tproj=300), steps=3, fused=fused)
    for k in ("r", "v", "a", "dens"):
        assert max_abs(out[k], ref[k]) < TOL, k


def test_langevin_const_and_verlet_mix(built_lib, oracle_lib):
    us = _batch(C.PROP_ID_VERLET, C.PROP_ID_LANGEVIN_CONST)
    out, ref = _step_both(us, W.emt_params(), SimParams(step=0.1, gamma_const=1e-3), steps=3, fused=True)
    for k in ("r", "v", "a"):
        assert max_abs(out[k], ref[k]) < TOL, k


def test_andersen(built_lib, oracle_lib):
    us = _batch(C.PROP_ID_ANDERSEN, C.PROP_ID_ANDERSEN)
    # andersen_time = step so that collisions happen with probability ~1/2 per bead... use 0.2
    out, ref = _step_both(us, W.emt_params(), SimParams(step=0.1, andersen_time=0.2), steps=2)
    for k in ("r", "v", "a"):
        assert max_abs(out[k], ref[k]) < 1e-9, k


@pytest.mark.parametrize("fused,nbeads", [(False, (4, 8)), (True, (4, 8)), (True, (16, 32)), (True, (3, 6)),
                                          (False, (5, 2)), (True, (1, 4))])
def test_pile_rpmd(built_lib, oracle_lib, fused, nbeads):
    """(16, 32): the largest bead counts of the RPMD benchmark mix, on 3x3 and 4x4 Pt(111).
    Odd bead counts and nb <= 2 take the direct normal-mode products, even nb >= 4 the
    folded ones (6: not a power of two); nb = 1 runs PILE on single beads."""
    us = _batch(C.PROP_ID_PILE, C.PROP_ID_PILE, nbeads=nbeads, metal="Pt", n=2, z0=1.5)
    out, ref = _step_both(us, W.emt_params("H", "Pt"), SimParams(step=0.1, Tsurf=300, Tproj=300), steps=2,
                          fused=fused)
    for k in ("r", "v", "a"):
        assert max_abs(out[k], ref[k]) < 1e-9, k


def test_rpmd_langevin_revert(built_lib, oracle_lib):
    us = _batch(C.PROP_ID_LANGEVIN, C.PROP_ID_VERLET, nbeads=(4,), n=2, z0=1.5)
    out, ref = _step_both(us, W.emt_params(), SimParams(step=0.1, Tsurf=300, Tproj=300), steps=2)
    for k in ("r", "v", "a"):
        assert max_abs(out[k], ref[k]) < 1e-9, k


def test_fused_matches_phases_with_philox(built_lib):
    """On-device deviates: the fused kernel and the three phase kernels draw the same
    counter-based numbers, so both paths give the same trajectory."""
    us = _batch(C.PROP_ID_VERLET, C.PROP_ID_LANGEVIN_CONST, n=3)
    emt = W.emt_params()
    sp = SimParams(step=0.1, gamma_const=2e-3, seed=99)
    e1 = make_engine(us, emt)
    e1.calc_force(sp)
    e1.md_steps(5, sp)
    a = e1.download()
    e2 = make_engine(us, emt)
    e2.calc_force(sp)
    for _ in range(5):
        e2.propagate_1(sp)
        e2.calc_force(sp)
        e2.propagate_2(sp)
    b = e2.download()
    for k in ("r", "v"):
        assert max_abs(a[k], b[k]) < 1e-12, k
    e1.close()
    e2.close()


def test_nve_conservation(built_lib):
    """Velocity Verlet on plain EMT conserves total energy.  Close H-Au encounters make
    the total energy fluctuate by a few meV at dt = 0.1 fs (the FP64 oracle shows the
    same), and the reference's pair loop drops a pair where it crosses cutoff*rcut while its
    Fermi factor is not yet zero there (pes_emt_mod.f90: `if (r > cutoff*rcut) cycle`), so
    E_tot also takes small steps whenever a pair of the free 300 K slab crosses that
    distance.  The secular drift is the mean slope of linear fits of E_tot(t) over 2 ps
    across 8 trajectories: below 1 meV/ps.  Each trajectory's own slope carries the noise of
    those steps (run-to-run, since FP64 shared-memory atomics make the chaotic trajectories
    diverge): below 5 meV/ps."""
    rng = np.random.default_rng(4)
    us = [W.h_on_metal(rng, "Au", 3, 1.0, 30.0, 0.0, 300.0, z0=2.5) for _ in range(8)]
    for u in us:
        u.is_fixed[:] = False
    emt = W.emt_params()
    sp = SimParams(step=0.1)
    eng = make_engine(us, emt)
    eng.calc_force(sp)
    chunk, nchunks = 200, 100
    ts, es = [], []
    for c in range(nchunks + 1):
        if c:
            eng.md_steps(chunk, sp)
        q = eng.query(sp)
        ts.append(c * chunk * sp.step * 1e-3)  # ps
        es.append(q["epot"] + q["ekin_p"] + q["ekin_l"])
    es = np.array(es)
    slope = np.array([np.polyfit(ts, es[:, t], 1)[0] for t in range(len(us))]) * 1e3  # meV/ps
    assert np.all(q["steps_done"] == chunk * nchunks)
    assert abs(float(np.mean(slope))) < 1.0, slope
    assert np.all(np.abs(slope) < 5.0), slope
    eng.close()


def test_exit_condition(built_lib):
    rng = np.random.default_rng(8)
    us = [W.h_on_metal(rng, "Au", 3, 2.0, 0.0, 0.0, 300.0, z0=6.0) for _ in range(3)]
    for u in us:
        u.v[0, :, 2] = +0.05  # moving away
    sp = SimParams(step=0.1, pul=6.05, use_exit=True)
    eng = make_engine(us, W.emt_params())
    eng.calc_force(sp)
    eng.md_steps(100, sp)
    q = eng.query(sp)
    assert np.all(q["status"] == 1)
    assert np.all(q["steps_done"] < 100)
    eng.close()
