"""Trajectory observables tracked by the fused MD kernels (turning points, closest
approach and its step, lowest projectile position, bounces, interaction time and the
adsorption flag; src/trajectory_info.f90) against a
host restatement of collect_trajectory_characteristics applied to the oracle's own
trajectory (FP64 EMT: identical turning points and steps, distances and positions within
1e-9 A), and for the FP32 radial surrogate kernel against the same restatement applied to
its downloaded states (its closest approach is an FP32 distance: 1e-4 A).  Then the
reference's mxt_fin record written from a GPU run and read back as its summary script
reads it."""
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.scatter import read_mxt_fin, run_to_exit, write_mxt_fin
from oracle.trajectory_info import TrajectoryInfo as Collect

pytestmark = pytest.mark.gpu
MODEL = Path(__file__).resolve().parents[1] / "md_tian2_gb300" / "data" / "surrogate_radial.npz"


def _batch(seed=3):
    rng = np.random.default_rng(seed)
    return [W.h_on_metal(rng, "Au", k, 2.0, 20.0, 30.0 * k, 300.0, z0=2.5) for k in (3, 4, 3)]


def test_emt_observables_match_oracle(built_lib, oracle_lib):
    from oracle.oracle import OracleUniverse
    us = _batch()
    emt = W.emt_params()
    sp = SimParams(step=0.5)
    nsteps = 120
    ads = (1.7, 2.2)  # adsorption limits (A)
    eng = Engine(0)
    eng.read_emt(emt)
    eng.define(us)
    eng.set_adsorption(*ads)
    eng.upload()
    eng.calc_force(sp)
    eng.md_steps(nsteps, sp)
    obs = eng.observables()
    bnc = eng.bounces(sp)
    eng.close()
    turns = bounces = 0
    for t, u in enumerate(us):
        o = OracleUniverse(u, emt)
        col = Collect(u.simbox, adsorption=ads, step=sp.step)
        o.calc_force(sp)
        for k in range(1, nsteps + 1):
            o.propagate_1(sp)
            o.calc_force(sp)
            o.propagate_2(sp)
            col(k, o.r, o.v, o.f)
        turns += col.turn
        bounces += col.final_bounces()
        assert obs["turn_pnts"][t] == col.turn, t
        assert obs["cl_appr_step"][t] == col.clstep, t
        assert abs(obs["cl_appr"][t] - col.cl) < 1e-9, t
        assert np.abs(obs["r_min_p"][t] - col.low).max() < 1e-9, t
        assert bnc["bounces"][t] == col.final_bounces(), (t, bnc["bounces"][t], col.final_bounces())
        assert bnc["interaction_time"][t] == pytest.approx(col.interaction_time()), t
        assert bnc["is_adsorbed"][t] == col.adsorbed, t
    assert turns >= 1 and bounces >= 1  # projectiles turned and collided in front of the surface


def test_radial_kernel_observables_match_its_states(built_lib):
    us = W.config2(6, seed=41)
    for u in us:  # start the projectiles 2.5 A above the surface
        u.r[0, :, 2] = 2.5
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=2)
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.read_nene(nene.load_npz(MODEL), ["H", "Au"], max_neighbors=80)
    eng.set_pes(PES_SURROGATE, 0.1)
    assert eng.nn_radial_kernel(True)
    eng.upload()
    eng.calc_force(sp, precision="fp32")
    eng.set_adsorption(1.7, 2.2)
    cols = [Collect(u.simbox, adsorption=(1.7, 2.2), step=sp.step) for u in us]
    for k in range(1, 41):
        eng.md_steps(1, sp, precision="fp32")
        out = eng.download()
        for t, c in enumerate(cols):
            c(k, eng.split(out["r"], t), eng.split(out["v"], t), eng.split(out["f"], t))
    obs = eng.observables()
    bnc = eng.bounces(sp)
    eng.close()
    assert sum(c.turn for c in cols) >= 1
    for t, c in enumerate(cols):
        assert obs["turn_pnts"][t] == c.turn, t
        assert np.abs(obs["r_min_p"][t] - c.low).max() < 1e-12, t
        assert abs(obs["cl_appr"][t] - c.cl) < 1e-4, t
        assert abs(c.dist[int(obs["cl_appr_step"][t])] - c.cl) < 1e-4, t
        # the kernel's nearest partner and unit vectors come from FP32 distances: a
        # crossing at the edge of FP32 rounding may be counted on one side only
        assert abs(int(bnc["bounces"][t]) - c.final_bounces()) <= 1, t
        assert bnc["interaction_time"][t] == pytest.approx(c.interaction_time()), t
        assert bnc["is_adsorbed"][t] == c.adsorbed, t


def test_mxt_fin_from_a_gpu_run(built_lib, tmp_path):
    us = _batch(5)
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.upload()
    sp = SimParams(step=0.5, pul=2.55, use_exit=True)
    res = run_to_exit(eng, sp, max_steps=200, chunk=50)
    eng.close()
    paths = write_mxt_fin(tmp_path / "traj", res)
    assert len(paths) == len(us)
    for t, p in enumerate(paths):
        d = read_mxt_fin(p)
        assert abs(d["ekin_p_i"] - res.ekin_i[t]) < 1e-6 and abs(d["ekin_p_f"] - res.ekin_f[t]) < 1e-6
        assert d["turn_pnts"] == res.record["turn_pnts"][t]
        assert abs(d["r_f"][2] - res.z_f[t]) < 1e-6
        if res.status[t] != 0:
            assert d["time"] == pytest.approx((res.steps[t] - 1) * 0.5)
