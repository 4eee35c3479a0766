"""GPU parity of the HDNNP path (compute_nene) and the surrogate fallback.

Bars: FP64 energies within 1e-9 eV and forces within 1e-10 eV/A of the FP64 oracle;
neighbour lists identical (same (j, image) words in the same order); FP32 force RMSE
below 2e-3 eV/A."""
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_EMT, PES_NENE, PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.universe import Universe

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _cgraphene_universe(perturb=0.0, seed=0):
    g = np.load(GOLD / "cgraphene_geometry.npz")
    r = g["r"] + np.random.default_rng(seed).normal(scale=perturb, size=g["r"].shape)
    n = len(r)
    return Universe(r=r[:, None, :].copy(), v=np.zeros((n, 1, 3)), m=np.full(n, 12.011 * C.AMU2MASS),
                    idx=np.ones(n, np.int32), is_fixed=np.zeros((n, 1, 3), bool), simbox=g["simbox"], names=["C"],
                    is_proj=np.array([False]), algo=np.array([C.PROP_ID_VERLET], np.int32))


def _engine_nn(us, model, names, kind=PES_NENE, emt=None, margin=0.1):
    eng = Engine(0)
    if emt is not None:
        eng.read_emt(emt)
    eng.define(us)
    eng.read_nene(model, names)
    eng.set_pes(kind, margin)
    eng.upload()
    return eng


def test_shipped_network_fp64_and_neighbours(built_lib, oracle_lib):
    m = nene.load_npz(GOLD / "runner_cgraphene.npz")
    ref = np.load(GOLD / "runner_cgraphene_ref.npz")
    eng = _engine_nn([_cgraphene_universe()], m, ["C"])
    eng.calc_force(SimParams())
    out = eng.download()
    assert abs(out["epot"][0] - float(ref["energy"])) < 1e-9
    assert np.abs(out["f"].reshape(-1, 3) - ref["forces"]).max() < 1e-10
    counts, words = eng.nn_neighbors()
    assert np.array_equal(counts, ref["nb_counts"])
    k = 0
    for i, c in enumerate(counts):
        w = words[i, :c]
        assert np.array_equal(w & 0xFFFF, ref["nb_j"][k:k + c])
        n = np.stack([((w >> s) & 15) - 8 for s in (16, 20, 24)], axis=1)
        assert np.array_equal(n, ref["nb_n"][k:k + c])
        k += c
    eng.close()


def test_shipped_network_perturbed_batch(built_lib, oracle_lib):
    from oracle.oracle import NNOracle
    m = nene.load_npz(GOLD / "runner_cgraphene.npz")
    us = [_cgraphene_universe(0.05, s) for s in range(5)]
    o = NNOracle(m)
    for prec, ftol in (("fp64", 1e-10), ("fp32", None)):
        eng = _engine_nn(us, m, ["C"])
        eng.calc_force(SimParams(), precision=prec)
        out = eng.download()
        eng.close()
        for t, u in enumerate(us):
            E, F = o.energy_force(np.zeros(u.natoms, int), u.r[:, 0, :], u.simbox)
            f = eng.split(out["f"], t)[:, 0, :]
            if ftol:
                assert abs(out["epot"][t] - E) < 1e-9
                assert np.abs(f - F).max() < ftol
            else:
                assert np.sqrt(np.mean((f - F) ** 2)) < 2e-3
                assert abs(out["epot"][t] - E) < 5e-3


def _hgraphene_model(us, seed=5, neighbours=("C",)):
    """Random two-element network whose scaling comes from the GPU's own descriptors.
    With both H and C as neighbours the G3 set is cut to 24 functions over two neighbour
    pairs, which exercises the general (non-grid) G3 kernels."""
    m = nene.random_model(["H", "C"], hidden=(25, 25), act="t", seed=seed, neighbours=list(neighbours))
    if len(neighbours) > 1:
        rng = np.random.default_rng(seed)
        for e in range(m.nelem):
            sfs = [sf for sf in m.sfs[e] if sf.type == 2 or ((sf.e1, sf.e2) in ((1, 6), (6, 6)) and sf.zeta != 16.0)]
            m.sfs[e] = sfs
            n = m.nodes[e]
            n[0] = len(sfs)
            w = []
            for l in range(1, len(n)):
                lim = np.sqrt(6.0 / (n[l - 1] + n[l]))
                w.extend(rng.uniform(-lim, lim, size=n[l - 1] * n[l]))
                w.extend(np.zeros(n[l]))
            m.weights[e] = np.array(w)
            m.smin[e], m.smax[e], m.savg[e] = np.zeros(len(sfs)), np.ones(len(sfs)), np.zeros(len(sfs))
    eng = _engine_nn(us, m, ["H", "C"])
    G = eng.nn_descriptors()
    eng.close()
    elem = np.concatenate([[0] + [1] * (u.natoms - 1) for u in us])
    nene.set_scaling(m, G, elem)
    return m


@pytest.mark.parametrize("neighbours", [("C",), ("H", "C")])
def test_two_element_network_fp64(built_lib, oracle_lib, neighbours):
    """("C",): every G3 shares one neighbour pair (grid-form kernels); ("H", "C"): G3 over
    three neighbour pairs (general kernels)."""
    from oracle.oracle import NNOracle
    rng = np.random.default_rng(9)
    us = [W.h_on_graphene(rng, 1.0, z0=z) for z in (1.2, 1.8, 3.0)]
    m = _hgraphene_model(us, neighbours=neighbours)
    o = NNOracle(m)
    eng = _engine_nn(us, m, ["H", "C"])
    eng.calc_force(SimParams())
    out = eng.download()
    for t, u in enumerate(us):
        elem = np.array([0] + [1] * (u.natoms - 1))
        E, F = o.energy_force(elem, u.r[:, 0, :], u.simbox)
        # the random network's forces reach 1e2 eV/A: hold them to 1e-12 relative
        assert abs(out["epot"][t] - E) < 1e-9 * max(1.0, abs(E))
        assert np.abs(eng.split(out["f"], t)[:, 0, :] - F).max() < 1e-12 * max(1.0, np.abs(F).max())
    eng.close()


def test_nn_md_steps_match_oracle(built_lib, oracle_lib):
    from oracle.oracle import NNOracle
    rng = np.random.default_rng(2)
    us = [W.h_on_graphene(rng, 1.0, z0=2.0) for _ in range(2)]
    m = _hgraphene_model(us)
    sp = SimParams(step=0.2)
    eng = _engine_nn(us, m, ["H", "C"])
    eng.calc_force(sp)
    eng.md_steps(5, sp)
    out = eng.download()
    o = NNOracle(m)
    for t, u in enumerate(us):
        elem = np.array([0] + [1] * (u.natoms - 1))
        r, v = u.r[:, 0, :].copy(), u.v[:, 0, :].copy()
        mass = u.m[:, None]
        _, F = o.energy_force(elem, r, u.simbox)
        for _ in range(5):  # velocity Verlet, md_algo.f90:110-142
            v = v + 0.5 * sp.step * F / mass
            r = r + sp.step * v
            _, F = o.energy_force(elem, r, u.simbox)
            v = v + 0.5 * sp.step * F / mass
        assert np.abs(eng.split(out["r"], t)[:, 0, :] - r).max() < 1e-10
        assert np.abs(eng.split(out["v"], t)[:, 0, :] - v).max() < 1e-10
    eng.close()


def test_surrogate_falls_back_to_emt(built_lib, oracle_lib):
    """A bead whose symmetry functions leave the training range is evaluated with FP64
    EMT, so its forces equal the EMT oracle's."""
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(4)
    train = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=5.0)]
    far = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=1.0)]
    emt = W.emt_params()
    m = nene.random_model(["H", "Au"], hidden=(32, 32), act="p", seed=1, neighbours=["Au"])
    eng = _engine_nn(train, m, ["H", "Au"])
    G = eng.nn_descriptors()
    eng.close()
    nene.set_scaling(m, G, np.array([0] + [1] * (train[0].natoms - 1)))
    sp = SimParams()
    eng = _engine_nn(train + far, m, ["H", "Au"], kind=PES_SURROGATE, emt=emt, margin=0.01)
    eng.calc_force(sp)
    out = eng.download()
    fb, ov = eng.nn_stats()
    assert fb[0] == 0 and fb[1] == 1 and not ov.any()
    o = OracleUniverse(far[0], emt)
    o.calc_force(sp)
    assert np.abs(eng.split(out["f"], 1) - o.f).max() < 1e-10
    eng.close()


def test_surrogate_requires_emt_and_rejects_ldfa(built_lib):
    from md_tian2_gb300._lib import EngineError
    rng = np.random.default_rng(0)
    us = [W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, C.PROP_ID_LANGEVIN, C.PROP_ID_LANGEVIN)]
    m = nene.random_model(["H", "Au"], hidden=(8,), act="t", seed=1, neighbours=["Au"])
    eng = _engine_nn(us, m, ["H", "Au"], kind=PES_SURROGATE)
    with pytest.raises(EngineError):
        eng.calc_force(SimParams())
    eng.read_emt(W.emt_params())
    with pytest.raises(EngineError):
        eng.md_steps(1, SimParams())
    eng.close()
