"""GPU parity of the thread-per-atom kernel of radial-only models (mdt_nnr.cu): shifted
G2 functions over H and Au neighbours, 24-32-32-1 softplus networks (the layout of the
shipped H/Au surrogate) and one-hidden-layer variants.

Bars: unscaled descriptors against the FP64 oracle, force RMSE below 1e-4 of the force
RMS and energies within 5e-5 relative (the exponentials use the hardware 2^x
approximation, as on the warp-per-atom fast kernel); against the warp-per-atom kernel on
the same batch the same bars; fused MD steps stay within 1e-6 A of the FP64 generic
kernels; the surrogate's EMT fallback is FP64-exact (1e-10 eV/A)."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_NENE, PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.surrogate import surrogate_model

pytestmark = pytest.mark.gpu
MAXNB = 120


def _engine(us, m, kind=PES_NENE, emt=None, margin=0.1, maxnb=MAXNB, radial=True, fast=True):
    eng = Engine(0)
    if emt is not None:
        eng.read_emt(emt)
    eng.define(us)
    eng.read_nene(m, ["H", "Au"], max_neighbors=maxnb)
    eng.set_pes(kind, margin)
    eng.nn_fast_path(fast)
    eng.nn_radial_kernel(radial)
    eng.upload()
    return eng


def _elems(u):
    return np.array([0] + [1] * (u.natoms - 1))


def _radial_model(seed, hidden=(32, 32), uniform=True):
    """uniform=False moves one r_s of the Au-neighbour grid by 0.05 bohr, which takes the
    model off the shifted-Gaussian recurrence onto one 2^x per function."""
    m = nene.random_model(["H", "Au"], hidden=hidden, act="p", seed=seed, neighbours=["H", "Au"],
                          descriptor="radial")
    if not uniform:
        for sfs in m.sfs:
            au = [f for f in sfs if f.e1 == 79]
            au[7].rshift += 0.05
    return m


def _scaled(us, m):
    eng = _engine(us, m, radial=False)
    G = eng.nn_descriptors()
    eng.close()
    nene.set_scaling(m, G, np.concatenate([_elems(u) for u in us]))
    return m


@pytest.mark.parametrize("hidden,uniform", [((32, 32), True), ((32,), True), ((20, 25), True),
                                            ((32, 32), False)])
def test_radial_kernel_matches_oracle(built_lib, oracle_lib, hidden, uniform):
    from oracle.oracle import NNOracle
    us = W.config2(7, seed=21)
    m = _radial_model(4, hidden, uniform)
    eng = _engine(us, m)
    assert eng.nn_radial_kernel(True)
    eng.calc_force(SimParams(), precision="fp32")
    out = eng.download()
    _, ov = eng.nn_stats()
    assert not ov.any()
    eng.close()
    o = NNOracle(m)
    for t, u in enumerate(us):
        E, F = o.energy_force(_elems(u), u.r[:, 0, :], u.simbox)
        f = eng.split(out["f"], t)[:, 0, :]
        assert np.sqrt(np.mean((f - F) ** 2)) < 1e-4 * np.sqrt(np.mean(F ** 2)), (hidden, t)
        assert abs(out["epot"][t] - E) < 5e-5 * max(1.0, abs(E)), (hidden, t)


def test_radial_kernel_matches_warp_kernel_scaled_and_energy_only(built_lib, oracle_lib):
    """A scaled model on a ragged batch larger than one pack: thread-per-atom against
    warp-per-atom, forces and energies, then the energy-only evaluation."""
    us = W.config2(40, seed=22)
    m = _scaled(us[:8], _radial_model(6))
    outs = {}
    for radial in (True, False):
        eng = _engine(us, m, radial=radial)
        eng.calc_force(SimParams(), precision="fp32")
        o = eng.download()
        eng.calc_force(SimParams(), flag=C.ENERGY_ONLY, precision="fp32")
        o["epot_only"] = eng.download()["epot"]
        outs[radial] = o
        eng.close()
    a, b = outs[True], outs[False]
    frms = np.sqrt(np.mean(b["f"] ** 2))
    assert np.sqrt(np.mean((a["f"] - b["f"]) ** 2)) < 1e-4 * frms
    assert np.abs(a["epot"] - b["epot"]).max() < 5e-5 * max(1.0, np.abs(b["epot"]).max())
    assert np.allclose(a["epot_only"], a["epot"], rtol=0, atol=1e-9)


def test_radial_md_steps_track_fp64(built_lib, oracle_lib):
    """Ten fused MD steps (constant-friction Langevin slab, Verlet projectile, same
    deviates on both sides) in FP32 forces stay within 1e-6 A of the FP64 kernels."""
    us = W.config2(6, seed=23)
    m = _radial_model(8)
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=5)
    res = {}
    for prec in ("fp32", "fp64"):
        eng = _engine(us, m)
        eng.calc_force(sp, precision=prec)
        eng.md_steps(10, sp, precision=prec)
        res[prec] = eng.download()
        eng.close()
    assert np.abs(res["fp32"]["r"] - res["fp64"]["r"]).max() < 1e-6
    assert np.abs(res["fp32"]["v"] - res["fp64"]["v"]).max() < 1e-6


def test_radial_langevin_coefficients_follow_the_parameters(built_lib, oracle_lib):
    """The thread-per-atom kernel forms its constant-friction Langevin coefficients once
    per parameter set: ten steps at one friction and time step, then ten at another,
    track the FP64 kernels (which form them every step) as closely as one parameter set
    does."""
    us = W.config2(6, seed=25)
    m = _radial_model(8)
    sps = [SimParams(step=0.1, gamma_const=1e-3, seed=5), SimParams(step=0.2, gamma_const=2e-2, seed=6)]
    res = {}
    for prec in ("fp32", "fp64"):
        eng = _engine(us, m)
        eng.calc_force(sps[0], precision=prec)
        for sp in sps:
            eng.md_steps(10, sp, precision=prec)
        res[prec] = eng.download()
        eng.close()
    assert np.abs(res["fp32"]["r"] - res["fp64"]["r"]).max() < 1e-5
    assert np.abs(res["fp32"]["v"] - res["fp64"]["v"]).max() < 1e-5


def test_radial_md_exit_and_skin(built_lib, oracle_lib):
    """Projectiles that leave through pul stop (status and step count as the warp
    kernel gives them); 40 steps with the 1 A skin equal 40 steps built every step.  Each
    step's neighbour forces are summed by shared-memory float atomics in no fixed order,
    and 40 steps of 0.5 fs amplify FP32 rounding differences: the skin comparison carries a
    1e-5 A bar; the two kernels also round differently (5e-5 A)."""
    us = W.config2(12, seed=24)
    m = _radial_model(9)
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=7, pul=6.05, use_exit=True)
    res = {}
    for radial, skin in ((True, 1.0), (True, 0.0), (False, 1.0)):
        eng = _engine(us, m, radial=radial)
        eng.nn_set_skin(skin)
        eng.calc_force(sp, precision="fp32")
        eng.md_steps(40, sp, precision="fp32")
        out = eng.download()
        q = eng.query(sp)
        res[(radial, skin)] = (out, q)
        eng.close()
    a, qa = res[(True, 1.0)]
    b, qb = res[(True, 0.0)]
    c, qc = res[(False, 1.0)]
    assert np.abs(a["r"] - b["r"]).max() < 1e-5
    assert np.abs(a["r"] - c["r"]).max() < 5e-5
    assert (qa["status"] == qc["status"]).all() and (qa["steps_done"] == qc["steps_done"]).all()


@pytest.mark.parametrize("prec", ["fp32", "bf16x3"])
def test_radial_md_launch_leaves_every_force_complete(built_lib, oracle_lib, prec):
    """The state a fused launch leaves carries every force of its last step: after one
    20-step launch, in which half the trajectories stop early through pul, the forces of
    all atoms (fixed ones included) equal a fresh force evaluation of the downloaded
    positions (1e-5 of the largest force: FP32 sums in no fixed order)."""
    us = W.config2(24, seed=27)
    for t, u in enumerate(us):  # half the projectiles start just below pul, moving up
        if t % 2 == 0:
            u.r[0, :, 2] = 6.0
            u.v[0, :, 2] = 0.05
    m = _radial_model(9)
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=7, pul=6.05, use_exit=True)
    eng = _engine(us, m)
    eng.calc_force(sp, precision=prec)
    eng.md_steps(20, sp, precision=prec)
    out = eng.download()
    q = eng.query(sp)
    eng.close()
    stopped = q["steps_done"] < 20
    assert stopped.any() and not stopped.all()
    fixed = np.concatenate([u.is_fixed.reshape(-1) for u in us]).astype(bool)
    assert fixed.sum() > len(fixed) // 3
    ref = _engine(us, m)
    ref.upload(out["r"], out["v"])
    ref.calc_force(sp, precision=prec)
    f = ref.download()["f"]
    ref.close()
    bar = 1e-5 * np.abs(f).max()
    assert np.abs(out["f"] - f)[fixed].max() < bar
    assert np.abs(out["f"] - f).max() < bar


def test_radial_surrogate_fallback_is_fp64_emt(built_lib, oracle_lib):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(4)
    train = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=5.0)]
    far = [W.h_on_metal(rng, "Au", 4, 1.0, 0.0, 0.0, 300.0, z0=0.8)]
    emt = W.emt_params()
    m = _scaled(train, _radial_model(10))
    sp = SimParams()
    eng = _engine(train + far, m, kind=PES_SURROGATE, emt=emt, margin=0.01)
    assert eng.nn_radial_kernel(True)
    eng.calc_force(sp, precision="fp32")
    out = eng.download()
    fb, ov = eng.nn_stats()
    assert fb[0] == 0 and fb[1] == 1 and not ov.any()
    o = OracleUniverse(far[0], emt)
    o.calc_force(sp)
    assert np.abs(eng.split(out["f"], 1) - o.f).max() < 1e-10
    assert abs(out["epot"][1] - o.epot[0]) < 1e-9
    eng.close()


def test_radial_neighbour_overflow_is_reported(built_lib):
    us = W.config2(3, seed=25)
    eng = _engine(us, _radial_model(2), maxnb=30)
    assert eng.nn_radial_kernel(True)
    eng.calc_force(SimParams(), precision="fp32")
    eng.download()
    _, ov = eng.nn_stats()
    assert ov.all()
    eng.close()


def test_radial_repack_over_running_trajectories(built_lib, oracle_lib):
    """Trajectories that leave through pul stop; re-packing the CTAs over those still running
    (mdt_nn_repack) changes which threads hold which atoms, not the trajectories: 40 more
    steps agree with the run that kept its packs (1e-5 A, FP32 sums in no fixed order)."""
    us = W.config2(48, seed=26)
    for t, u in enumerate(us):  # half the projectiles start just below pul, moving up
        if t % 2 == 0:
            u.r[0, :, 2] = 6.0
            u.v[0, :, 2] = 0.05
    m = _radial_model(9)
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=7, pul=6.05, use_exit=True)
    res = {}
    for repack in (False, True):
        eng = _engine(us, m)
        eng.calc_force(sp, precision="fp32")
        eng.md_steps(5, sp, precision="fp32")
        q = eng.query(sp)
        assert 0 < int(np.sum(q["status"] != 0)) < len(us)
        if repack:
            full = eng.nn_repack()
            assert full > 0
        eng.md_steps(40, sp, precision="fp32")
        res[repack] = (eng.download(), eng.query(sp))
        eng.close()
    (a, qa), (b, qb) = res[True], res[False]
    assert np.abs(a["r"] - b["r"]).max() < 1e-5
    assert (qa["status"] == qb["status"]).all() and (qa["steps_done"] == qb["steps_done"]).all()


def test_autotune_picks_a_shape_and_restores_the_state(built_lib, oracle_lib):
    """mdt_autotune times every candidate (CTA cap x skin) from the same saved state, keeps
    the fastest and puts the state back: positions, velocities, step counts and observables
    are bit-identical to before the call, and the batch runs on with the chosen shape."""
    from md_tian2_gb300.surrogate import shipped_surrogate
    us = W.config2(256, seed=27)
    emt = W.emt_params()
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=3, pul=6.05, use_exit=True)
    eng = _engine(us, shipped_surrogate(), kind=PES_SURROGATE, emt=emt)
    eng.calc_force(sp, precision="fp32")
    eng.md_steps(7, sp, precision="fp32")
    before, qb, ob = eng.download(), eng.query(sp), eng.observables()
    res = eng.autotune(sp, "fp32", nsteps=10)
    after, qa, oa = eng.download(), eng.query(sp), eng.observables()
    assert res["block"] in (256, 384, 512) and res["skin_A"] in (0.5, 0.75, 1.0) and res["ms_per_step"] > 0
    for k in ("r", "v", "f"):
        assert np.array_equal(before[k], after[k]), k
    assert (qa["steps_done"] == qb["steps_done"]).all() and (qa["status"] == qb["status"]).all()
    assert np.array_equal(ob["cl_appr"], oa["cl_appr"])
    eng.md_steps(5, sp, precision="fp32")
    assert (eng.query(sp)["steps_done"] >= qb["steps_done"]).all()
    eng.close()
