"""Host restatement of the reference's trajectory set-up (src/md_init.f90): projectile +
slab merge with centroid folding, projectile initial position (pip), incidence velocity
and bead replication, on the reference's lattice file (tests/golden/mxt_latt.npz)."""
import math
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import md_init
from md_tian2_gb300.universe import Universe, invert_matrix

GOLD = Path(__file__).resolve().parent / "golden"


def _slab():
    z = np.load(GOLD / "mxt_latt.npz")
    n = z["r"].shape[0]
    return Universe(r=z["r"].copy(), v=z["v"].copy(), m=np.full(n, C.MASS_AMU["Au"] * C.AMU2MASS),
                    idx=z["idx"].astype(np.int32), is_fixed=z["is_fixed"].copy(), simbox=z["simbox"].copy(),
                    names=[str(x) for x in z["names"]], is_proj=np.zeros(len(z["names"]), bool))


def _proj(pos, nb=1, v=(0.0, 0.0, 0.0)):
    r = np.tile(np.asarray(pos, float), (1, nb, 1))
    return Universe(r=r, v=np.tile(np.asarray(v, float), (1, nb, 1)), m=np.array([C.MASS_AMU["H"] * C.AMU2MASS]),
                    idx=np.array([1], np.int32), is_fixed=np.zeros((1, nb, 3), bool), simbox=np.eye(3) * 10.0,
                    names=["H"], is_proj=np.array([True]))


def test_merge_layout_and_folding():
    slab = _slab()
    box = slab.simbox
    # a projectile 2.3 cells along a1 (folds to 0.3) and -1.7 along a2 (int() truncates: -0.7)
    pos = box @ np.array([2.3, -1.7, 0.4])
    u = md_init.merge_universes(slab, _proj(pos), algo_p=C.PROP_ID_VERLET, algo_l=C.PROP_ID_LANGEVIN)
    assert u.natoms == slab.natoms + 1 and u.names == ["H"] + slab.names
    assert u.idx[0] == 1 and np.array_equal(u.idx[1:], slab.idx + 1)
    assert u.is_proj.tolist() == [True] + [False] * slab.ntypes
    assert u.algo.tolist() == [C.PROP_ID_VERLET, C.PROP_ID_LANGEVIN]
    f = invert_matrix(u.simbox) @ u.r[0, 0]
    assert np.allclose(f, [0.3, -0.7, 0.4])
    fs = np.einsum("ij,nj->ni", invert_matrix(box), slab.r[:, 0])
    fm = np.einsum("ij,nj->ni", invert_matrix(box), u.r[1:, 0])
    assert np.allclose(fm, fs - np.trunc(fs))
    with pytest.raises(ValueError, match="projectile atoms"):
        md_init.merge_universes(u, _proj(pos))


def test_pip_fixed_and_random():
    slab = _slab()
    box = slab.simbox
    p = md_init.apply_pip(_proj([1.0, 1.0, 1.0]), ["1.5", "2.5", "6.0"], np.random.default_rng(0))
    assert np.allclose(p.r[0, 0], [1.5, 2.5, 6.0])
    # random x, y: the reference's target arithmetic (whole vector scaled per drawn k)
    proj = _proj([1.0, 1.0, 1.0])
    proj.simbox = box
    rng = np.random.default_rng(7)
    u1, u2 = np.random.default_rng(7).random(2)
    t = np.zeros(3)
    t[0] = u1
    t = t * box[:, 0].sum()
    t[1] = u2
    t = t * box[:, 1].sum()
    q = md_init.apply_pip(proj, ["r", "r", "6.0"], rng)
    assert np.allclose(q.r[0, 0], box @ t + np.array([0.0, 0.0, 6.0]))


def test_incidence_velocity():
    u = md_init.merge_universes(_slab(), _proj([0.0, 0.0, 6.0], v=(0.3, -0.2, 0.1)))
    w = md_init.set_proj_incidence(u, 2.76, 45.0, azimuth="30.0")
    m = C.MASS_AMU["H"] * C.AMU2MASS
    vinc = math.sqrt(2 * 2.76 / m)
    pol, azi = math.radians(45.0), math.radians(30.0)
    assert np.allclose(w.v[0, 0], vinc * np.array([math.sin(pol) * math.cos(azi), math.sin(pol) * math.sin(azi),
                                                   -math.cos(pol)]))
    assert np.array_equal(w.v[1:], u.v[1:])  # lattice untouched
    assert 0.5 * m * np.sum(w.v[0, 0] ** 2) == pytest.approx(2.76)


def test_force_beads_and_incidence_removes_bead_drift():
    u = md_init.merge_universes(_slab(), _proj([0.0, 0.0, 6.0]))
    b = md_init.force_beads(u, 4)
    assert b.nbeads == 4 and np.array_equal(b.r[:, 3], u.r[:, 0])
    b.v[0] = np.array([[0.1, 0, 0], [0.3, 0, 0], [0.0, 0, 0], [0.0, 0, 0]])
    w = md_init.set_proj_incidence(b, 1.0, 0.0, azimuth="0")
    assert np.allclose(w.v[0].mean(axis=0), [0.0, 0.0, -math.sqrt(2 / (C.MASS_AMU["H"] * C.AMU2MASS))])
    assert np.allclose(w.v[0, 1] - w.v[0, 0], [0.2, 0, 0])  # bead spread kept, drift removed


def test_conf_merge_pipeline(tmp_path):
    """The reference's `conf merge` start of a trajectory: a projectile read from a POSCAR,
    the slab from an mxt file, merged with a fixed pip, incidence set, beads forced."""
    from md_tian2_gb300 import io
    p = tmp_path / "proj.POSCAR"
    p.write_text("H\n1.0\n 10 0 0\n 0 10 0\n 0 0 10\n H\n 1\ncartesian\n0.0 0.0 0.0\n")
    proj = io.read_poscar(p, nprojectiles=1)
    slab = _slab()
    u = md_init.merge_universes(slab, proj, pip=["2.0", "1.0", "6.0"], rng=np.random.default_rng(0),
                                algo_p=C.PROP_ID_VERLET, algo_l=C.PROP_ID_LANGEVIN)
    assert np.allclose(u.r[0, 0], [2.0, 1.0, 6.0] - slab.simbox @ np.trunc(np.linalg.solve(slab.simbox, [2.0, 1.0, 6.0])))
    u = md_init.set_proj_incidence(u, 2.76, 45.0, azimuth="0")
    u = md_init.force_beads(u, 2)
    assert u.nbeads == 2 and u.natoms == slab.natoms + 1
    assert u.names == ["H"] + slab.names and u.is_proj.tolist()[0]
    ek = 0.5 * u.m[0] * np.sum(u.v[0, 0] ** 2)
    assert ek == pytest.approx(2.76)
