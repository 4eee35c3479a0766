"""GPU parity of the FP32 fast kernels (mdt_nnf.cu) for models they admit: the H/Au
surrogate's symmetry-function set (8 G2 + 16 G3 over Au neighbours, 6.5 A cosine cutoff,
zeta in {1, 4, 16}, lambda = +-1).

Bars: with unscaled descriptors, force RMSE below 2e-5 of the force RMS and energies
within 2e-6 relative of the FP64 oracle (FP32 arithmetic over ~800 triplets per atom);
with scaled descriptors the FP32 bar of the generic kernels (2e-3 eV/A, 5e-3 eV); the
EMT fallback of the surrogate stays FP64-exact (1e-10 eV/A)."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_NENE, PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.surrogate import surrogate_model

pytestmark = pytest.mark.gpu
MAXNB = 80


def _engine(us, m, kind=PES_NENE, emt=None, margin=0.1, maxnb=MAXNB, fast=True):
    eng = Engine(0)
    if emt is not None:
        eng.read_emt(emt)
    eng.define(us)
    eng.read_nene(m, ["H", "Au"], max_neighbors=maxnb)
    eng.set_pes(kind, margin)
    eng.nn_fast_path(fast)
    eng.upload()
    return eng


def _scaled_model(us, seed=11):
    m = surrogate_model(seed)
    eng = _engine(us, m)
    G = eng.nn_descriptors()
    eng.close()
    elem = np.concatenate([[0] + [1] * (u.natoms - 1) for u in us])
    nene.set_scaling(m, G, elem)
    return m


def _elems(u):
    return np.array([0] + [1] * (u.natoms - 1))


def test_fast_path_qualifies_and_matches_oracle(built_lib, oracle_lib):
    """Unscaled descriptors (no scaling.data amplification): FP32 rounding only."""
    from oracle.oracle import NNOracle
    us = W.config2(6, seed=3)
    m = surrogate_model(11)
    eng = _engine(us, m)
    assert eng.nn_fast_path(True)
    eng.calc_force(SimParams(), precision="fp32")
    out = eng.download()
    fb, ov = eng.nn_stats()
    assert not ov.any()
    eng.close()
    o = NNOracle(m)
    for t, u in enumerate(us):
        E, F = o.energy_force(_elems(u), u.r[:, 0, :], u.simbox)
        f = eng.split(out["f"], t)[:, 0, :]
        frms = np.sqrt(np.mean(F ** 2))
        assert np.sqrt(np.mean((f - F) ** 2)) < 2e-5 * frms, t
        assert abs(out["epot"][t] - E) < 2e-6 * max(1.0, abs(E)), t


def test_fast_path_radial_model_matches_oracle(built_lib, oracle_lib):
    """24 shifted G2 over Au and H neighbours, no angular functions (the triplet stages are
    skipped; the exponentials use the hardware 2^x approximation, so the bar is 1e-4 of
    the force RMS)."""
    from oracle.oracle import NNOracle
    us = W.config2(5, seed=8)
    m = surrogate_model(3, descriptor="radial")
    eng = _engine(us, m)
    assert eng.nn_fast_path(True)
    eng.calc_force(SimParams(), precision="fp32")
    out = eng.download()
    eng.close()
    o = NNOracle(m)
    for t, u in enumerate(us):
        E, F = o.energy_force(_elems(u), u.r[:, 0, :], u.simbox)
        f = eng.split(out["f"], t)[:, 0, :]
        assert np.sqrt(np.mean((f - F) ** 2)) < 1e-4 * np.sqrt(np.mean(F ** 2)), t
        assert abs(out["epot"][t] - E) < 5e-5 * max(1.0, abs(E)), t


def test_fast_path_scaled_model_matches_oracle_like_generic(built_lib, oracle_lib):
    """Scaled descriptors from six configurations: (g - min)/(max - min) amplifies FP32
    rounding of G by |g|/(max - min), for both FP32 paths alike.  The fast path stays
    within the documented FP32 bar (force RMSE 2e-3 eV/A, energy 5e-3 eV) and within
    2.5x the generic FP32 kernels' error."""
    from oracle.oracle import NNOracle
    us = W.config2(6, seed=3)
    m = _scaled_model(us)
    o = NNOracle(m)
    ref = [o.energy_force(_elems(u), u.r[:, 0, :], u.simbox) for u in us]
    err = {}
    for fast in (True, False):
        eng = _engine(us, m, fast=fast)
        eng.calc_force(SimParams(), precision="fp32")
        out = eng.download()
        eng.close()
        fe, ee = [], []
        for t, (E, F) in enumerate(ref):
            fe.append((eng.split(out["f"], t)[:, 0, :] - F).ravel())
            ee.append(out["epot"][t] - E)
        err[fast] = (np.sqrt(np.mean(np.concatenate(fe) ** 2)), np.abs(ee).max())
    assert err[True][0] < 2e-3 and err[True][1] < 5e-3
    assert err[True][0] < 2.5 * err[False][0] + 1e-5


def test_fast_and_generic_fp32_agree_energy_only_too(built_lib, oracle_lib):
    us = W.config2(8, seed=5)
    m = _scaled_model(us)
    outs = {}
    for fast in (True, False):
        eng = _engine(us, m, fast=fast)
        eng.calc_force(SimParams(), precision="fp32")
        o = eng.download()
        eng.calc_force(SimParams(), flag=C.ENERGY_ONLY, precision="fp32")
        o["epot_only"] = eng.download()["epot"]
        outs[fast] = o
        eng.close()
    a, b = outs[True], outs[False]
    assert np.sqrt(np.mean((a["f"] - b["f"]) ** 2)) < 2e-3
    assert np.abs(a["epot"] - b["epot"]).max() < 5e-3
    assert np.allclose(a["epot_only"], a["epot"], rtol=0, atol=1e-9)


def test_fast_md_steps_track_fp64(built_lib, oracle_lib):
    """Five fused MD steps (Langevin slab, Verlet projectile) in FP32 forces stay within
    1e-6 A of the FP64 generic kernels."""
    us = W.config2(4, seed=9)
    m = surrogate_model(11)  # unscaled: the scaled toy model leaves its range within steps
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=5)
    res = {}
    for prec in ("fp32", "fp64"):
        eng = _engine(us, m)
        eng.calc_force(sp, precision=prec)
        eng.md_steps(5, sp, precision=prec)
        res[prec] = eng.download()
        eng.close()
    assert np.abs(res["fp32"]["r"] - res["fp64"]["r"]).max() < 1e-6


def test_fast_surrogate_fallback_is_fp64_emt(built_lib, oracle_lib):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(4)
    train = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=5.0)]
    far = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=1.0)]
    emt = W.emt_params()
    m = _scaled_model(train)
    sp = SimParams()
    eng = _engine(train + far, m, kind=PES_SURROGATE, emt=emt, margin=0.01)
    assert eng.nn_fast_path(True)
    eng.calc_force(sp, precision="fp32")
    out = eng.download()
    fb, ov = eng.nn_stats()
    assert fb[0] == 0 and fb[1] == 1 and not ov.any()
    o = OracleUniverse(far[0], emt)
    o.calc_force(sp)
    assert np.abs(eng.split(out["f"], 1) - o.f).max() < 1e-10
    eng.close()


def test_fast_neighbour_overflow_is_reported(built_lib):
    us = W.config2(2, seed=1)
    m = surrogate_model()
    eng = _engine(us, m, maxnb=24)
    assert eng.nn_fast_path(True)
    eng.calc_force(SimParams(), precision="fp32")
    eng.download()
    _, ov = eng.nn_stats()
    assert ov.all()
    eng.close()


def test_skin_lists_do_not_change_results(built_lib, oracle_lib):
    """30 fused MD steps with the default 1 A skin (lists rebuilt when an atom moved more
    than 0.5 A) against lists built every step; then positions displaced by 0.4 A (no
    rebuild) and by 2 A (rebuild) through the state upload, both checked against the
    oracle.  Only FP32 summation order differs between the runs."""
    from oracle.oracle import NNOracle
    us = W.config2(6, seed=12)
    m = surrogate_model(5, descriptor="radial")
    sp = SimParams(step=0.5, gamma_const=1e-3, seed=3)
    res = {}
    for skin in (1.0, 0.0):
        eng = _engine(us, m)
        eng.nn_set_skin(skin)
        eng.calc_force(sp, precision="fp32")
        eng.md_steps(30, sp, precision="fp32")
        res[skin] = eng.download()
        eng.close()
    assert np.abs(res[1.0]["r"] - res[0.0]["r"]).max() < 1e-6
    o = NNOracle(m)
    eng = _engine(us, m)
    eng.calc_force(sp, precision="fp32")
    rng = np.random.default_rng(0)
    for amp in (0.4, 2.0):
        moved = []
        for u in us:
            d = rng.normal(size=u.r.shape)
            d *= amp / np.linalg.norm(d, axis=-1, keepdims=True) / np.sqrt(3.0)
            moved.append(u.r + d)
        eng.upload(r=np.concatenate([r.reshape(-1, 3) for r in moved]))
        eng.calc_force(sp, precision="fp32")
        out = eng.download()
        for t, u in enumerate(us):
            E, F = o.energy_force(_elems(u), moved[t][:, 0, :], u.simbox)
            f = eng.split(out["f"], t)[:, 0, :]
            assert np.sqrt(np.mean((f - F) ** 2)) < 1e-4 * np.sqrt(np.mean(F ** 2)), (amp, t)
    eng.close()
