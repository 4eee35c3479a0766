"""POSCAR reader and create_repetitions (src/md_init.f90:195-342,
src/universe_mod.f90:120-217) on the reference's own POSCAR files (tests/golden/
poscar_ref.json, made by make_golden.py) and on synthetic files for the bead count,
direct coordinates, mobility flags and the velocity section."""
import json
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import io

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "poscar_ref.json").read_text())


@pytest.mark.parametrize("name", ["example.POSCAR", "cart.POSCAR"])
def test_reference_poscars(tmp_path, name):
    g = GOLD[name]
    p = tmp_path / name
    p.write_text(g["text"])
    u = io.read_poscar(p, nprojectiles=1)
    coords = np.array(g["coords"])
    assert u.natoms == len(coords) and u.nbeads == 1
    assert u.names == g["elements"]
    assert np.allclose(u.r[:, 0, :], coords * g["scale"], atol=0, rtol=0)
    assert np.allclose(u.simbox, np.array(g["cell_rows"]).T * g["scale"])
    assert u.is_proj.tolist() == [True] + [False] * (len(u.names) - 1)
    assert u.idx[0] == 1 and np.all(u.idx[1:] == 2)
    assert not u.is_fixed.any() and not u.v.any()
    assert u.m[0] == pytest.approx(C.MASS_AMU["H"] * C.AMU2MASS)


def test_repetitions_of_reference_poscar(tmp_path):
    g = GOLD["cart.POSCAR"]
    p = tmp_path / "cart.POSCAR"
    p.write_text(g["text"])
    u = io.read_poscar(p, 1)
    w = io.read_poscar(p, 1, rep=(1, 2))
    n_latt = u.natoms - 1
    assert w.natoms == 1 + 3 * 5 * n_latt
    assert np.allclose(w.r[0], u.r[0], rtol=0, atol=1e-12)  # projectile first, unmoved (direct round trip)
    a1, a2 = u.simbox[:, 0], u.simbox[:, 1]
    k = 1
    for i in range(-1, 2):
        for j in range(-2, 3):  # second index fastest, as the reference loops
            assert np.allclose(w.r[k:k + n_latt, 0], u.r[1:, 0] + i * a1 + j * a2)
            k += n_latt
    assert np.allclose(w.simbox[:, 0], 3 * a1) and np.allclose(w.simbox[:, 1], 5 * a2)
    assert np.allclose(w.simbox[:, 2], u.simbox[:, 2])


def test_beads_direct_flags_and_velocities(tmp_path):
    text = "\n".join([
        "synthetic", "2.0", " 3.0 0.0 0.0", " 0.0 4.0 0.0", " 0.0 0.0 5.0", " H Au", " :2: 1 1", "Direct",
        "0.1 0.2 0.3 T T T", "0.1 0.2 0.31 T T T", "0.5 0.5 0.0 F F T", "0.5 0.5 0.0 F F T", "",
        "0.0 0.0 -0.1", "0.0 0.0 -0.1", "0.01 0.0 0.0", "0.0 0.02 0.0"])
    p = tmp_path / "s.POSCAR"
    p.write_text(text + "\n")
    u = io.read_poscar(p, 1)
    assert u.natoms == 2 and u.nbeads == 2
    box = np.diag([6.0, 8.0, 10.0])
    assert np.allclose(u.simbox, box)
    assert np.allclose(u.r[0, 1], [0.6, 1.6, 3.1])  # direct x scaled cell
    assert u.is_fixed[1, 0].tolist() == [True, True, False] and not u.is_fixed[0].any()
    assert np.allclose(u.v[1, 1], [0.0, 0.02, 0.0])


def test_poscar_errors(tmp_path):
    p = tmp_path / "bad.POSCAR"
    p.write_text("c\n1.0\n1 0 0\n0 1 0\n0 0 1\nH\n 1\nsideways\n0 0 0\n")
    with pytest.raises(io.InputError, match="coordinate system"):
        io.read_poscar(p)
    p.write_text("c\n1.0\n1 0 0\n0 1 0\n0 0 1\nH\n 1\ncart\n0 0 0\nnot blank\n")
    with pytest.raises(io.InputError, match="velocities"):
        io.read_poscar(p)
