"""Device refill of stopped trajectories (mdt_refill) and the per-trajectory step limit:
the restored slab equals the uploaded state exactly, the new projectile starts at z0 with
an incidence energy and polar angle inside the requested ranges, status / steps /
observables restart, running trajectories are untouched; then a stream of trajectories
through a small batch (scatter.run_campaign)."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import Engine, SimParams
from md_tian2_gb300.scatter import run_campaign

pytestmark = pytest.mark.gpu


def _engine(us):
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.upload()
    return eng


def test_step_limit_and_refill(built_lib):
    us = W.config2(6, seed=51)
    eng = _engine(us)
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=4, pul=6.05, use_exit=True)
    up = eng.download()
    eng.set_step_limit(20)
    eng.calc_force(sp)
    eng.md_steps(10, sp)
    gen, n = eng.refill(z0=6.0, einc=(1.0, 2.0), polar=(0.0, 30.0), seed=9)
    assert n == 0 and not gen.any()  # nothing stopped yet
    eng.md_steps(15, sp)
    q = eng.query(sp)
    assert (q["status"] == 3).all() and (q["steps_done"] == 20).all()
    gen, n = eng.refill(z0=6.0, einc=(1.0, 2.0), polar=(0.0, 30.0), seed=9)
    assert n == 6 and (gen == 1).all()
    out = eng.download()
    q = eng.query(sp)
    assert (q["status"] == 0).all() and (q["steps_done"] == 0).all()
    obs = eng.observables()
    assert not obs["turn_pnts"].any() and (obs["cl_appr"] > 1e300).all()
    m_h = C.MASS_AMU["H"] * C.AMU2MASS
    for t, u in enumerate(us):
        r, v = eng.split(out["r"], t), eng.split(out["v"], t)
        r0, v0 = eng.split(up["r"], t), eng.split(up["v"], t)
        assert np.array_equal(r[1:], r0[1:]) and np.array_equal(v[1:], v0[1:])  # slab restored
        assert r[0, 0, 2] == 6.0
        f = np.linalg.solve(u.simbox, r[0, 0])
        assert 0.0 <= f[0] < 1.0 and 0.0 <= f[1] < 1.0
        e = 0.5 * m_h * np.sum(v[0, 0] ** 2)
        assert 1.0 - 1e-12 <= e <= 2.0 + 1e-12
        polar = np.degrees(np.arccos(-v[0, 0, 2] / np.linalg.norm(v[0, 0])))
        assert -1e-9 <= polar <= 30.0 + 1e-9
    # a second refill of the same slots draws new starts
    eng.md_steps(25, sp)
    gen2, n2 = eng.refill(z0=6.0, einc=(1.0, 2.0), polar=(0.0, 30.0), seed=9)
    out2 = eng.download()
    assert n2 == 6 and (gen2 == 2).all()
    assert not np.array_equal(eng.split(out2["r"], 0)[0], eng.split(out["r"], 0)[0])
    eng.close()


def test_refill_keeps_ring_polymer_spread(built_lib):
    """nb > 1: the projectile's beads move by (target - centroid) as in apply_pip, and their
    velocities lose their mean and gain the incidence velocity as in set_proj_incidence, so
    the bead spread and the internal bead velocities of the uploaded state are kept."""
    rng = np.random.default_rng(53)
    us = []
    for nb in (4, 8):
        u = W.h_on_metal(rng, "Pt", 3, 0.5, 0.0, 0.0, 300.0, C.PROP_ID_PILE, C.PROP_ID_PILE, z0=4.0, nbeads=nb)
        u.r[0] += rng.normal(scale=0.05, size=u.r[0].shape)  # zero-point spread of the projectile
        u.v[0] += rng.normal(scale=0.01, size=u.v[0].shape)  # internal bead velocities
        us.append(u)
    eng = Engine(0)
    eng.read_emt(W.emt_params("H", "Pt"))
    eng.define(us)
    eng.upload()
    up = eng.download()
    sp = SimParams(step=0.1, seed=4)
    eng.set_step_limit(3)
    eng.calc_force(sp)
    eng.md_steps(3, sp)
    gen, n = eng.refill(z0=6.0, einc=(0.2, 0.4), polar=(0.0, 0.0), azimuth=0.0, seed=2)
    assert n == 2
    out = eng.download()
    m_h = C.MASS_AMU["H"] * C.AMU2MASS
    for t, u in enumerate(us):
        r, v = eng.split(out["r"], t)[0], eng.split(out["v"], t)[0]   # (nb, 3) of the projectile
        r0, v0 = eng.split(up["r"], t)[0], eng.split(up["v"], t)[0]
        assert np.allclose(r - r.mean(0), r0 - r0.mean(0), rtol=0, atol=1e-12)
        assert np.allclose(v - v.mean(0), v0 - v0.mean(0), rtol=0, atol=1e-14)
        assert abs(r.mean(0)[2] - 6.0) < 1e-12
        vc = v.mean(0)
        assert abs(vc[0]) < 1e-14 and abs(vc[1]) < 1e-14 and vc[2] < 0.0  # normal incidence
        assert 0.2 - 1e-12 <= 0.5 * m_h * np.sum(vc ** 2) <= 0.4 + 1e-12
        assert np.array_equal(eng.split(out["r"], t)[1:], eng.split(up["r"], t)[1:])
    eng.close()


def test_error_status_is_not_refilled(built_lib):
    us = W.config2(4, seed=54)
    bad = [u.copy() for u in us]
    bad[2].r[3, 0, 1] = np.nan
    eng = _engine(bad)
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=4)
    eng.set_step_limit(5)
    eng.calc_force(sp)
    eng.md_steps(5, sp)
    q = eng.query(sp)
    assert q["status"][2] == -11 and (q["status"][[0, 1, 3]] == 3).all()
    gen, n = eng.refill(seed=1)
    q = eng.query(sp)
    assert n == 3 and gen[2] == 0 and q["status"][2] == -11 and (q["status"][[0, 1, 3]] == 0).all()
    eng.close()


def test_campaign_streams_trajectories(built_lib):
    us = W.config2(12, seed=52)
    eng = _engine(us)
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=6, pul=6.05, use_exit=True)
    res = run_campaign(eng, sp, total=40, refill={"z0": 6.0, "einc": (1.0, 3.0), "polar": (0.0, 45.0), "seed": 3},
                       precision="fp64", max_steps=200, chunk=50)
    eng.close()
    assert len(res.z_f) == 40
    assert set(np.unique(res.status)) <= {1, 3}
    assert (res.steps <= 200).all() and (res.steps > 0).all()
    assert (res.z_f[res.status == 1] > 6.05).all()
    assert np.isfinite(res.ekin_i).all() and (res.ekin_i > 0).all()


def test_refill_matches_host_md_init(built_lib):
    """The device refill against the host restatement of md_init (md_tian2_gb300.md_init):
    each restarted trajectory's draws (mdt_refill_draws: u, v, einc, polar, azimuth) fed to
    apply_pip with a numeric pip (the centroid moved to u a1 + v a2 + z0 e_z, md_init.f90:
    498-553) and to set_proj_incidence (:829-876) give the device's projectile beads to
    1e-12 (A, A/fs); trajectories not restarted report NaN draws."""
    from md_tian2_gb300.md_init import apply_pip, set_proj_incidence
    from md_tian2_gb300.universe import Universe
    rng = np.random.default_rng(55)
    us = []
    for nb in (4, 8, 4):
        u = W.h_on_metal(rng, "Pt", 3, 0.5, 10.0, 20.0, 300.0, C.PROP_ID_PILE, C.PROP_ID_PILE, z0=4.0, nbeads=nb)
        u.r[0] += rng.normal(scale=0.05, size=u.r[0].shape)
        u.v[0] += rng.normal(scale=0.01, size=u.v[0].shape)
        us.append(u)
    eng = Engine(0)
    eng.read_emt(W.emt_params("H", "Pt"))
    eng.define(us)
    eng.upload()
    up = eng.download()
    sp = SimParams(step=0.1, seed=4)
    eng.set_step_limit(3)
    eng.calc_force(sp)
    eng.md_steps(3, sp)
    eng.set_step_limit(0)
    gen, n = eng.refill(z0=6.5, einc=(0.2, 0.9), polar=(0.0, 40.0), azimuth=-1.0, seed=8)
    assert n == 3
    draws = eng.refill_draws()
    out = eng.download()
    for t, u in enumerate(us):
        du, dv, e, pol, azi = draws[t]
        box = u.simbox
        pip = [du * box[0, 0] + dv * box[0, 1], du * box[1, 0] + dv * box[1, 1], 6.5]
        r0, v0 = eng.split(up["r"], t)[0], eng.split(up["v"], t)[0]  # (nb, 3) uploaded projectile
        proj = Universe(r=r0[None].copy(), v=v0[None].copy(), m=u.m[:1].copy(), idx=np.array([1], np.int32),
                        is_fixed=np.zeros((1, u.nbeads, 3), bool), simbox=box.copy(), names=["H"],
                        is_proj=np.array([True]), algo=np.array([C.PROP_ID_PILE], np.int32))
        host = set_proj_incidence(apply_pip(proj, pip, rng), einc=e, polar_deg=pol, azimuth=str(azi))
        assert np.abs(eng.split(out["r"], t)[0] - host.r[0]).max() < 1e-12, t
        assert np.abs(eng.split(out["v"], t)[0] - host.v[0]).max() < 1e-12, t
        assert 0.2 <= e <= 0.9 and 0.0 <= pol <= 40.0 and 0.0 <= azi < 360.0
    gen2, n2 = eng.refill(seed=9)  # nothing stopped: nothing restarted, every row NaN
    assert n2 == 0 and np.isnan(eng.refill_draws()).all()
    eng.close()
