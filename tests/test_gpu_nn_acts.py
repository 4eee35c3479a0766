"""GPU parity of every RuNNer activation, of addatoms and of the H/graphene HDNNP at its
benchmark shape, against the FP64 oracle.

* Activations t g l c s S e p h (calconenn.f90:124-146) with their derivatives
  (getdnodes_values.f90:76-108): FP64 generic kernels within 1e-9 relative (energies) and
  1e-11 relative (forces); FP32 kernels (warp-per-atom fast kernel and the generic one)
  with a force RMSE below 3e-3 of the force RMS and energies within 1e-3 relative (random
  Glorot networks on unscaled-range inputs give forces of 1e2-1e5 eV/A, so the bars are
  relative).  The thread-per-atom radial kernel takes
  p t s l; s and l are checked here (p and t in the radial tests).
* addatoms (RuNNer_src/addatoms.f90:23-56): with remove_atom_energies the energy gains the
  per-element reference energies of every atom, in Hartree converted to eV.
* 72 C + 1 H on 6x6 graphene, 8 G2 + 16 G3 per element, 24-25-25-1 tanh: a batch of 32
  trajectories; FP64 at 1e-10 eV/A, FP32 force RMSE stated and bounded."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_NENE, Engine, SimParams

pytestmark = pytest.mark.gpu
HA2EV = 27.21138602


def _engine(us, m, names=("H", "C"), fast=True, radial=True):
    eng = Engine(0)
    eng.define(us)
    eng.read_nene(m, list(names))
    eng.set_pes(PES_NENE, 0.1)
    eng.nn_fast_path(fast)
    eng.nn_radial_kernel(radial)
    eng.upload()
    return eng


def _elems(u):
    return np.array([0] + [1] * (u.natoms - 1))


def _scaled(us, m, names=("H", "C")):
    eng = _engine(us, m, names)
    G = eng.nn_descriptors()
    eng.close()
    nene.set_scaling(m, G, np.concatenate([_elems(u) for u in us]))
    return m


def _forces(us, m, prec, names=("H", "C"), fast=True, radial=True):
    eng = _engine(us, m, names, fast, radial)
    eng.calc_force(SimParams(), precision=prec)
    out = eng.download()
    f = [eng.split(out["f"], t)[:, 0, :] for t in range(len(us))]
    eng.close()
    return out["epot"], f


def _oracle(us, m):
    from oracle.oracle import NNOracle
    o = NNOracle(m)
    res = [o.energy_force(_elems(u), u.r[:, 0, :], u.simbox) for u in us]
    return np.array([r[0] for r in res]), [r[1] for r in res]


@pytest.mark.parametrize("act", list("tglcsSeph"))
def test_activation_matches_oracle(built_lib, oracle_lib, act):
    rng = np.random.default_rng(21)
    us = [W.h_on_graphene(rng, 1.0, z0=z) for z in (1.3, 2.2)]
    m = nene.random_model(["H", "C"], hidden=(16, 12), act=act, seed=3, neighbours=["C"])
    m.acts = [[a[0], a[1], "t" if act == "l" else "l"] for a in m.acts]  # one non-linear output layer too
    _scaled(us, m)
    E0, F0 = _oracle(us, m)
    e, f = _forces(us, m, "fp64")
    for t in range(len(us)):
        assert abs(e[t] - E0[t]) <= 1e-9 * max(1.0, abs(E0[t])), (act, t, e[t], E0[t])
        assert np.abs(f[t] - F0[t]).max() <= 1e-11 * max(1.0, np.abs(F0[t]).max()), act
    for fast in (True, False):
        e32, f32 = _forces(us, m, "fp32", fast=fast)
        for t in range(len(us)):
            rms = np.sqrt(np.mean(F0[t] ** 2))
            assert np.sqrt(np.mean((f32[t] - F0[t]) ** 2)) < 3e-3 * max(rms, 1e-3), (act, fast, t)
            ebar = 3e-3 if act == "e" else 1e-3  # exp(-x) layers reach thousands of eV: fast-exp error grows
            assert abs(e32[t] - E0[t]) <= ebar * max(1.0, abs(E0[t])), (act, fast, t)


@pytest.mark.parametrize("act", ["s", "l"])
def test_radial_kernel_other_activations(built_lib, oracle_lib, act):
    us = W.config2(6, seed=41)
    m = nene.random_model(["H", "Au"], hidden=(32, 32), act=act, seed=6, neighbours=["H", "Au"],
                          descriptor="radial")
    _scaled(us, m, ("H", "Au"))
    eng = _engine(us, m, ("H", "Au"))
    assert eng.nn_radial_kernel(True)
    eng.close()
    E0, F0 = _oracle(us, m)
    e32, f32 = _forces(us, m, "fp32", ("H", "Au"))
    for t in range(len(us)):
        rms = np.sqrt(np.mean(F0[t] ** 2))
        assert np.sqrt(np.mean((f32[t] - F0[t]) ** 2)) < 1e-4 * max(rms, 1e-3), (act, t)
        assert abs(e32[t] - E0[t]) <= 5e-5 * max(1.0, abs(E0[t])), (act, t)


def test_addatoms_adds_reference_energies(built_lib, oracle_lib):
    rng = np.random.default_rng(8)
    us = [W.h_on_graphene(rng, 1.0, z0=z) for z in (1.5, 2.5)]
    m = nene.random_model(["H", "C"], hidden=(25, 25), act="t", seed=9, neighbours=["C"])
    _scaled(us, m)
    e_plain, f_plain = _forces(us, m, "fp64")
    m.atom_energy = {"H": -0.4998, "C": -37.8450}
    E0, F0 = _oracle(us, m)
    for prec, tol in (("fp64", 1e-9), ("fp32", 1e-4)):
        e, f = _forces(us, m, prec)
        for t, u in enumerate(us):
            shift = HA2EV * (m.atom_energy["H"] + (u.natoms - 1) * m.atom_energy["C"])
            assert abs(e[t] - E0[t]) <= tol * abs(E0[t]), (prec, t)
            if prec == "fp64":
                assert abs((e[t] - e_plain[t]) - shift) <= 1e-9 * abs(shift), t
                # forces do not change (up to the unordered FP64 sums of two runs)
                assert np.abs(f[t] - f_plain[t]).max() <= 1e-10 * max(1.0, np.abs(f_plain[t]).max())
    # the oracle agrees on the shift itself
    m.atom_energy = {}
    E1, _ = _oracle(us, m)
    for t, u in enumerate(us):
        shift = HA2EV * (-0.4998 + (u.natoms - 1) * -37.8450)
        assert abs((E0[t] - E1[t]) - shift) <= 1e-9 * abs(shift)


def test_graphene_batch_at_benchmark_shape(built_lib, oracle_lib):
    """The HDNNP benchmark shape (72 C + 1 H, 8 G2 + 16 G3, 24-25-25-1 tanh) on a batch of
    32 trajectories: FP64 within 1e-10 eV/A (relative to the largest force), FP32 force RMSE
    below 1e-3 of the force RMS."""
    us = W.config4(32, seed=44)
    heights = np.random.default_rng(7).uniform(1.0, 4.0, size=len(us))
    for u, z in zip(us, heights):  # spread the projectile heights over the interaction region
        u.r[0, 0, 2] = z
    m = nene.random_model(["H", "C"], hidden=(25, 25), act="t", seed=5, neighbours=["C"])
    assert [len(s) for s in m.sfs] == [24, 24] and m.nodes[0] == [24, 25, 25, 1]
    assert us[0].natoms == 73
    _scaled(us, m)
    E0, F0 = _oracle(us, m)
    e, f = _forces(us, m, "fp64")
    for t in range(len(us)):
        assert abs(e[t] - E0[t]) < 1e-9 * max(1.0, abs(E0[t]))
        assert np.abs(f[t] - F0[t]).max() < 1e-10 * max(1.0, np.abs(F0[t]).max())
    e32, f32 = _forces(us, m, "fp32")
    d = np.concatenate([(a - b).reshape(-1) for a, b in zip(f32, F0)])
    rms = np.sqrt(np.mean(np.concatenate([b.reshape(-1) for b in F0]) ** 2))
    assert np.sqrt(np.mean(d ** 2)) < 1e-3 * rms, (np.sqrt(np.mean(d ** 2)), rms)
    assert np.all(np.abs(e32 - E0) <= 1e-3 * np.maximum(1.0, np.abs(E0)))
