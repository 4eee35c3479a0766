"""GPU parity of calc_force (EMT) against the FP64 oracle.

Bar: FP64 forces within 1e-10 eV/A of the oracle, bead energies within 1e-9 eV,
embedded densities within 1e-12 relative.  FP32 force arithmetic is held to a stated
RMSE against FP64 (2e-4 eV/A)."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams

from .helpers import make_engine, max_abs, oracle_list

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-10     # eV/A, FP64
EPOT_TOL = 1e-9       # eV, FP64
FP32_RMSE_TOL = 2e-4  # eV/A


def _ragged_batch(seed=11, n=12):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(n):
        k = 3 + t % 4
        out.append(W.h_on_metal(rng, "Au", k, rng.uniform(0.5, 5), rng.uniform(0, 60), rng.uniform(0, 360), 300.0))
    # pull some projectiles into the surface region so every EMT branch is exercised
    for t, u in enumerate(out):
        u.r[0, :, 2] = [6.0, 3.0, 1.5, 0.8][t % 4]
        u.r[1:, :, :] += rng.normal(scale=0.05, size=u.r[1:].shape)
    return out


def _compare(universes, emt, precision="fp64", flag=C.ENERGY_AND_FORCE):
    sp = SimParams()
    eng = make_engine(universes, emt)
    eng.calc_force(sp, flag=flag, precision=precision)
    out = eng.download()
    orcs = oracle_list(universes, emt)
    for o in orcs:
        o.calc_force(sp)
    f_ref = np.concatenate([o.f.reshape(-1) for o in orcs])
    e_ref = np.concatenate([o.epot for o in orcs])
    d_ref = np.concatenate([o.dens.reshape(-1) for o in orcs])
    a_ref = np.concatenate([o.a.reshape(-1) for o in orcs])
    eng.close()
    return out, f_ref, e_ref, d_ref, a_ref


def test_emt_fp64_config1_geometry(built_lib, oracle_lib):
    us = W.config1(4, seed=7)
    for u in us:
        u.r[0, 0, 2] = 1.2  # projectile inside the interaction range
    out, f_ref, e_ref, d_ref, a_ref = _compare(us, W.emt_params())
    assert max_abs(out["f"], f_ref) < FORCE_TOL
    assert max_abs(out["epot"], e_ref) < EPOT_TOL
    assert max_abs(out["a"], a_ref) < FORCE_TOL
    np.testing.assert_allclose(out["dens"], d_ref, rtol=1e-12, atol=1e-300)


def test_emt_fp64_ragged_sizes(built_lib, oracle_lib):
    us = _ragged_batch()
    out, f_ref, e_ref, d_ref, _ = _compare(us, W.emt_params())
    assert max_abs(out["f"], f_ref) < FORCE_TOL
    assert max_abs(out["epot"], e_ref) < EPOT_TOL
    np.testing.assert_allclose(out["dens"], d_ref, rtol=1e-12, atol=1e-300)


def test_emt_fp64_hpt_and_beads(built_lib, oracle_lib):
    rng = np.random.default_rng(3)
    us = [W.h_on_metal(rng, "Pt", 4, 0.5, 0.0, 0.0, 300.0, C.PROP_ID_PILE, C.PROP_ID_PILE, nbeads=nb, z0=1.0)
          for nb in (4, 8)]
    for u in us:
        u.r += rng.normal(scale=0.03, size=u.r.shape)
    emt = W.emt_params("H", "Pt")
    sp = SimParams()
    eng = make_engine(us, emt)
    # calc_force performs the free ring-polymer step first for nbeads > 1 (force.f90:54),
    # also when only energies are requested
    eng.calc_force(sp, flag=C.ENERGY_ONLY)
    e_only = eng.download()
    eng.upload()
    eng.calc_force(sp)
    out = eng.download()
    orcs = oracle_list(us, emt)
    for o in orcs:
        o.calc_force(sp)
    ref = {k: np.concatenate([getattr(o, k).reshape(-1) for o in orcs]) for k in ("r", "v", "f", "epot")}
    assert max_abs(e_only["epot"], ref["epot"]) < EPOT_TOL
    assert max_abs(out["epot"], ref["epot"]) < EPOT_TOL
    for k in ("r", "v", "f"):
        assert max_abs(out[k], ref[k]) < FORCE_TOL, k
    eng.close()


def test_emt_single_species_pt(built_lib, oracle_lib):
    rng = np.random.default_rng(5)
    pos, cell, fx = W.fcc111_slab(W.LATTICE_A["Pt"], 4)
    from md_tian2_gb300.universe import Universe
    us = []
    for _ in range(3):
        r = pos + rng.normal(scale=0.05, size=pos.shape)
        us.append(Universe(r[:, None, :].copy(), np.zeros((len(pos), 1, 3)),
                           np.full(len(pos), C.MASS_AMU["Pt"] * C.AMU2MASS), np.ones(len(pos), np.int32),
                           np.repeat(fx[:, None, None], 3, axis=2).copy(), cell, ["Pt"], np.array([False]),
                           np.array([C.PROP_ID_VERLET], np.int32)))
    emt = W.emt_params("H", "Pt", with_proj=False)
    out, f_ref, e_ref, d_ref, _ = _compare(us, emt)
    assert max_abs(out["f"], f_ref) < FORCE_TOL
    assert max_abs(out["epot"], e_ref) < EPOT_TOL


def test_emt_fp32_rmse(built_lib, oracle_lib):
    us = _ragged_batch(seed=19, n=8)
    out, f_ref, e_ref, _, _ = _compare(us, W.emt_params(), precision="fp32")
    rmse = float(np.sqrt(np.mean((out["f"] - f_ref) ** 2)))
    assert rmse < FP32_RMSE_TOL, rmse
    assert max_abs(out["epot"], e_ref) < 1e-3
