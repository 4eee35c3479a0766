"""CPU checks of the oracle and the input readers against the reference's own data
(golden fixtures in tests/golden/, regenerated by tests/golden/make_golden.py)."""
import json
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import io, nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams

from .refroot import reference_root

GOLD = Path(__file__).resolve().parent / "golden"
REF = reference_root()


def test_emt_table_matches_reference_pes_files():
    g = json.loads((GOLD / "emt_params.json").read_text())
    for name, (p, m) in (("EMT-HAu.pes", ("H", "Au")), ("EMT-HPt.pes", ("H", "Pt"))):
        t = W.emt_params(p, m)
        for k in io.EMT_KEYS:
            assert np.array_equal(t.values[k], np.array(g[name][k])), (name, k)


@pytest.mark.skipif(REF is None, reason="no reference checkout (set MDT_REFERENCE_ROOT)")
def test_readers_reproduce_golden_from_reference_files():
    p = io.read_pes(REF / "pes" / "EMT-HAu.pes", ["H", "Au"], [True, False])
    g = json.loads((GOLD / "emt_params.json").read_text())
    for k in io.EMT_KEYS:
        assert p.values[k].tolist() == g["EMT-HAu.pes"][k]
    u = io.read_mxt(REF / "conf" / "latt" / "mxt_00000001.dat")
    z = np.load(GOLD / "mxt_latt.npz")
    assert np.array_equal(u.r, z["r"]) and np.array_equal(u.simbox, z["simbox"])
    m = nene.read_runner(REF / "example" / "md" / "RuNNer_input")
    m2 = nene.load_npz(GOLD / "runner_cgraphene.npz")
    assert all(np.array_equal(a, b) for a, b in zip(m.weights, m2.weights))


def test_mxt_round_trip(tmp_path):
    z = np.load(GOLD / "mxt_latt.npz")
    from md_tian2_gb300.universe import Universe
    u = Universe(r=z["r"], v=z["v"], m=np.ones(len(z["idx"])), idx=z["idx"], is_fixed=z["is_fixed"],
                 simbox=z["simbox"], names=[str(n) for n in z["names"]], is_proj=z["is_proj"])
    io.write_mxt(tmp_path / "x.dat", u)
    v = io.read_mxt(tmp_path / "x.dat")
    assert np.array_equal(v.r, u.r) and np.array_equal(v.v, u.v) and np.array_equal(v.idx, u.idx)
    assert np.array_equal(v.simbox, u.simbox) and np.array_equal(v.is_fixed, u.is_fixed)


def test_pes_reader_errors(tmp_path):
    f = tmp_path / "bad.pes"
    f.write_text("pes emt\nH Au proj latt\n eta2 1.0 2.0\n")
    with pytest.raises(io.InputError):
        io.read_pes(f, ["H", "Au"], [True, False])


def test_symfunction_sort_and_duplicates():
    sfs = [nene.SymFunc(3, eta=0.1, lam=1, zeta=1, rc=12, e1=6, e2=6), nene.SymFunc(2, eta=0.5, rc=12, e1=6),
           nene.SymFunc(2, eta=0.1, rc=12, e1=6)]
    out = nene.sort_symfunctions(sfs)
    assert [s.type for s in out] == [2, 2, 3] and out[0].eta == 0.1
    with pytest.raises(nene.NNInputError):
        nene.sort_symfunctions(sfs + [nene.SymFunc(2, eta=0.1, rc=12, e1=6)])


def test_emt_oracle_newton_and_gradient(oracle_lib):
    from oracle.oracle import OracleUniverse
    rng = np.random.default_rng(1)
    u = W.h_on_metal(rng, "Au", 3, 1.0, 0.0, 0.0, 300.0, z0=1.5)
    u.r[1:] += rng.normal(scale=0.05, size=u.r[1:].shape)
    emt = W.emt_params()
    sp = SimParams()
    o = OracleUniverse(u, emt)
    o.calc_force(sp)
    assert np.abs(o.f.sum(axis=(0, 1))).max() < 1e-12
    h = 1e-5
    for (a, d) in [(0, 2), (4, 0), (20, 1)]:
        e = []
        for s in (h, -h):
            p = OracleUniverse(u, emt)
            p.r[a, 0, d] += s
            p.calc_force(sp)
            e.append(p.epot[0])
        assert abs(-(e[0] - e[1]) / (2 * h) - o.f[a, 0, d]) < 1e-7


def test_hdnnp_oracle_on_shipped_network(oracle_lib):
    """compute_nene on the shipped C-graphene network: the stored regression fixture (the
    oracle's own earlier output, which keeps it from drifting), the check_forces sum rule
    (pes_nene_mod.f90:7272-7287) and finite differences."""
    from oracle.oracle import NNOracle
    m = nene.load_npz(GOLD / "runner_cgraphene.npz")
    g = np.load(GOLD / "cgraphene_geometry.npz")
    ref = np.load(GOLD / "runner_cgraphene_ref.npz")
    o = NNOracle(m)
    E, F = o.energy_force(np.zeros(len(g["r"]), int), g["r"], g["simbox"])
    assert abs(E - float(ref["energy"])) < 1e-9
    assert np.abs(F - ref["forces"]).max() < 1e-10
    assert np.abs(F.sum(0)).max() < 1e-10
    h = 1e-5
    for (a, d) in [(0, 0), (7, 2), (19, 1)]:
        rp, rm = g["r"].copy(), g["r"].copy()
        rp[a, d] += h
        rm[a, d] -= h
        fd = -(o.energy_force(np.zeros(len(rp), int), rp, g["simbox"])[0] -
               o.energy_force(np.zeros(len(rm), int), rm, g["simbox"])[0]) / (2 * h)
        assert abs(fd - F[a, d]) < 1e-6


def test_hdnnp_oracle_two_elements_gradient(oracle_lib):
    from oracle.oracle import NNOracle
    rng = np.random.default_rng(3)
    m = nene.random_model(["H", "C"], hidden=(25, 25), act="t", seed=3, neighbours=["C"])
    u = W.h_on_graphene(rng, 1.0, z0=1.6)
    elem = np.array([0] + [1] * (u.natoms - 1))
    o = NNOracle(m)
    E, F, G, _ = o.energy_force(elem, u.r[:, 0, :], u.simbox, want_G=True)
    nene.set_scaling(m, G, elem)
    o = NNOracle(m)
    E, F = o.energy_force(elem, u.r[:, 0, :], u.simbox)
    assert np.abs(F.sum(0)).max() < 1e-9
    h = 1e-5
    for (a, d) in [(0, 2), (3, 0), (40, 1)]:
        rp, rm = u.r[:, 0, :].copy(), u.r[:, 0, :].copy()
        rp[a, d] += h
        rm[a, d] -= h
        fd = -(o.energy_force(elem, rp, u.simbox)[0] - o.energy_force(elem, rm, u.simbox)[0]) / (2 * h)
        assert abs(fd - F[a, d]) < 1e-6 * max(1.0, abs(F[a, d]))


@pytest.mark.skipif(REF is None, reason="no reference checkout (set MDT_REFERENCE_ROOT)")
def test_poscar_fixtures_match_reference_files():
    g = json.loads((GOLD / "poscar_ref.json").read_text())
    for name in ("example.POSCAR", "cart.POSCAR"):
        assert (REF / "conf" / name).read_text() == g[name]["text"]
        u = io.read_poscar(REF / "conf" / name, nprojectiles=1)
        assert np.allclose(u.r[:, 0, :], np.array(g[name]["coords"]) * g[name]["scale"], rtol=0, atol=0)
