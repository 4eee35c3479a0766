"""GPU parity of the tensor-core network (the thread-per-atom kernel with its four network
GEMMs per 128-atom tile on tcgen05, FP32 accumulation in TMEM; descriptors, activations,
scaling and forces in FP32) against the FP64 oracle, in its two operand formats:
MDT_PREC_BF16 (BF16 operands) and MDT_PREC_BF16X3 (every operand split in a BF16 high and
low part, three MMAs per K step).

Bars, stated per format: BF16 force RMSE below 1e-2 of the force RMS and energies within
5e-3 relative of the FP64 oracle (BF16 keeps 8 significant bits: one rounding of every
operand of a 24-32-32-1 network; the random test networks reach several eV per atom);
BF16X3 force RMSE below 2e-4 of the force RMS and energies within 1e-4 relative (about 16
significant bits, near the FP32 kernel's 1e-4 and 5e-5); the trained surrogate's forces
within 5 meV/A (BF16) and 0.5 meV/A (BF16X3) RMSE of its FP32 evaluation.  Results of the same model in FP32 agree with BF16 to the same bars, so a
wrong operand layout (which would scramble weights) cannot pass."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300._lib import EngineError
from md_tian2_gb300.engine import PES_EMT, PES_NENE, PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.surrogate import shipped_surrogate

pytestmark = pytest.mark.gpu
BARS = {"bf16": (1e-2, 5e-3), "bf16x3": (2e-4, 1e-4)}  # force RMSE / force RMS, energy relative


def _engine(us, m, kind=PES_NENE, emt=None, margin=0.1, names=("H", "Au")):
    eng = Engine(0)
    if emt is not None:
        eng.read_emt(emt)
    eng.define(us)
    eng.read_nene(m, list(names), max_neighbors=120)
    eng.set_pes(kind, margin)
    eng.upload()
    return eng


def _elems(u):
    return np.array([0] + [1] * (u.natoms - 1))


def _model(seed, hidden=(32, 32), act="p"):
    return nene.random_model(["H", "Au"], hidden=hidden, act=act, seed=seed, neighbours=["H", "Au"],
                             descriptor="radial")


def _scaled(us, m):
    eng = _engine(us, m)
    G = eng.nn_descriptors()
    eng.close()
    nene.set_scaling(m, G, np.concatenate([_elems(u) for u in us]))
    return m


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
@pytest.mark.parametrize("hidden,act", [((32, 32), "p"), ((32,), "t"), ((20, 25), "s")])
def test_bf16_network_matches_oracle(built_lib, oracle_lib, hidden, act, prec):
    from oracle.oracle import NNOracle
    F_REL, E_REL = BARS[prec]
    us = W.config2(9, seed=61)
    m = _scaled(us[:4], _model(3, hidden, act))
    eng = _engine(us, m)
    assert eng.nn_radial_kernel(True)
    eng.calc_force(SimParams(), precision=prec)
    out = eng.download()
    eng.close()
    o = NNOracle(m)
    fr, fd = [], []
    for t, u in enumerate(us):
        E, F = o.energy_force(_elems(u), u.r[:, 0, :], u.simbox)
        f = eng.split(out["f"], t)[:, 0, :]
        fr.append(F)
        fd.append(f - F)
        assert abs(out["epot"][t] - E) < E_REL * max(1.0, abs(E)), (hidden, t, out["epot"][t], E)
    fr, fd = np.concatenate(fr), np.concatenate(fd)
    rms = np.sqrt(np.mean(fr ** 2))
    err = np.sqrt(np.mean(fd ** 2))
    assert err < F_REL * rms, (hidden, err, rms)
    assert err > 0.0  # the tensor-core path really rounds its operands


@pytest.mark.parametrize("tprec", ["bf16", "bf16x3"])
def test_bf16_energy_only_and_packs(built_lib, oracle_lib, tprec):
    """A ragged batch of several packs: the tensor-core network against FP32 on the same
    kernel, forces and energies, and the energy-only evaluation equals the energies of the
    full one."""
    F_REL, E_REL = BARS[tprec]
    us = W.config2(60, seed=62)
    m = _scaled(us[:8], _model(5))
    res = {}
    for prec in ("fp32", tprec):
        eng = _engine(us, m)
        eng.calc_force(SimParams(), precision=prec)
        o = eng.download()
        eng.calc_force(SimParams(), flag=C.ENERGY_ONLY, precision=prec)
        o["epot_only"] = eng.download()["epot"]
        res[prec] = o
        eng.close()
    a, b = res[tprec], res["fp32"]
    rms = np.sqrt(np.mean(b["f"] ** 2))
    assert np.sqrt(np.mean((a["f"] - b["f"]) ** 2)) < F_REL * rms
    assert np.all(np.abs(a["epot"] - b["epot"]) < E_REL * np.maximum(1.0, np.abs(b["epot"])))
    assert np.allclose(a["epot_only"], a["epot"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("tprec,fbar,rbar", [("bf16", 5e-3, 1e-3), ("bf16x3", 5e-4, 1e-4)])
def test_bf16_shipped_surrogate_md_steps(built_lib, oracle_lib, tprec, fbar, rbar):
    """The trained surrogate: forces within 5 meV/A (BF16) / 0.5 meV/A (BF16X3) RMSE of its
    FP32 evaluation, and 20 fused MD steps track the FP32 steps (positions within 1e-3 /
    1e-4 A)."""
    us = W.config2(16, seed=63)
    emt = W.emt_params()
    m = shipped_surrogate()
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=5)
    res = {}
    for prec in ("fp32", tprec):
        eng = _engine(us, m, kind=PES_SURROGATE, emt=emt)
        eng.calc_force(sp, precision=prec)
        f0 = eng.download()["f"]
        eng.md_steps(20, sp, precision=prec)
        res[prec] = (f0, eng.download(), eng.query(sp))
        eng.close()
    fa, a, qa = res[tprec]
    fb, b, qb = res["fp32"]
    assert np.sqrt(np.mean((fa - fb) ** 2)) < fbar
    assert np.abs(a["r"] - b["r"]).max() < rbar
    assert (qa["status"] == qb["status"]).all() and (qa["steps_done"] == 20).all()


def test_bf16_fallback_is_fp64_emt(built_lib, oracle_lib):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(4)
    train = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=5.0)]
    far = [W.h_on_metal(rng, "Au", 4, 1.0, 0.0, 0.0, 300.0, z0=0.8)]
    emt = W.emt_params()
    m = _scaled(train, _model(10))
    eng = _engine(train + far, m, kind=PES_SURROGATE, emt=emt, margin=0.01)
    eng.calc_force(SimParams(), precision="bf16")
    out = eng.download()
    fb, _ = eng.nn_stats()
    eng.close()
    assert fb[0] == 0 and fb[1] == 1
    o = OracleUniverse(far[0], emt)
    o.calc_force(SimParams())
    assert np.abs(eng.split(out["f"], 1) - o.f).max() < 1e-10


def test_bf16_outside_its_scope_is_an_error(built_lib):
    us = W.config2(2, seed=64)
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.upload()
    eng.set_pes(PES_EMT)
    with pytest.raises(EngineError):
        eng.calc_force(SimParams(), precision="bf16")  # EMT has no GEMMs
    m = nene.random_model(["H", "Au"], hidden=(16, 16), act="t", seed=1, neighbours=["Au"])  # G3: not radial
    eng.read_nene(m, ["H", "Au"])
    eng.set_pes(PES_NENE)
    if eng.nn_fast_path(True):  # the descriptors' scaling table exists: the generic tensor-core pass runs
        eng.calc_force(SimParams(), precision="bf16")
    else:
        with pytest.raises(EngineError):
            eng.calc_force(SimParams(), precision="bf16")
    with pytest.raises(EngineError):
        eng.md_steps(2, SimParams(), precision="bf16")  # fused MD steps: thread-per-atom kernel only
    eng.close()


@pytest.mark.parametrize("prec", ["bf16", "bf16x3"])
def test_bf16_generic_network_at_graphene_benchmark_shape(built_lib, oracle_lib, prec):
    """The HDNNP benchmark shape (72 C + 1 H on graphene, 8 G2 + 16 G3, 24-25-25-1 tanh) with
    its network on the tensor cores as a pass of its own (descriptors and forces on the FP32
    generic kernel): forces and energies against the FP64 oracle within the bars of the
    radial kernel's tensor-core network, energy-only equal to the energies of the full
    evaluation."""
    F_REL, E_REL = BARS[prec]
    us = W.config4(12, seed=45)
    for u, z in zip(us, np.random.default_rng(8).uniform(1.0, 4.0, size=len(us))):
        u.r[0, 0, 2] = z
    m = nene.random_model(["H", "C"], hidden=(25, 25), act="t", seed=6, neighbours=["C"])
    eng = _engine(us, m, names=("H", "C"))
    G = eng.nn_descriptors()
    eng.close()
    nene.set_scaling(m, G, np.concatenate([_elems(u) for u in us]))
    eng = _engine(us, m, names=("H", "C"))
    eng.calc_force(SimParams(), precision=prec)
    out = eng.download()
    eng.calc_force(SimParams(), flag=C.ENERGY_ONLY, precision=prec)
    e_only = eng.download()["epot"]
    eng.close()
    from oracle.oracle import NNOracle
    o = NNOracle(m)
    fr, fd = [], []
    for t, u in enumerate(us):
        E, F = o.energy_force(_elems(u), u.r[:, 0, :], u.simbox)
        f = eng.split(out["f"], t)[:, 0, :]
        fr.append(F)
        fd.append(f - F)
        assert abs(out["epot"][t] - E) < E_REL * max(1.0, abs(E)), (t, out["epot"][t], E)
    rms = np.sqrt(np.mean(np.concatenate(fr) ** 2))
    err = np.sqrt(np.mean(np.concatenate(fd) ** 2))
    assert 0.0 < err < F_REL * rms, (err, rms)
    assert np.allclose(e_only, out["epot"], rtol=0, atol=1e-9)
