"""GPU parity of the per-trajectory energies that mdt_query returns, against the oracle:
mean bead potential energy (calc_force's epot, force.f90:49-82), the centroid kinetic
energies of projectile and lattice (atom_ekin, universe_mod.f90:433-458) and the
ring-polymer spring energy (calc_bead_epot, rpmd.f90:244-267).

Both sides take the same host-provided deviates, so after a few steps the states agree
to round-off; the energies are FP64 reductions in a different order, held to 1e-10
relative (1e-10 eV absolute below 1 eV)."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import SimParams

from .helpers import flat, injected, make_engine, oracle_list

pytestmark = pytest.mark.gpu


def _close(a, b, rel=1e-10):
    return abs(a - b) <= rel * max(1.0, abs(b))


def _run(us, emt, sp, steps, seed=3):
    rng = np.random.default_rng(seed)
    eng = make_engine(us, emt)
    orcs = oracle_list(us, emt)
    sp_inj = SimParams(**{**sp.__dict__, "rng_mode": 1})
    eng.calc_force(sp)
    for o in orcs:
        o.calc_force(sp)
    for _ in range(steps):
        randy, zeta, av, au = injected(us, rng)
        eng.set_random_arrays(flat(randy), flat(zeta), flat(av), flat(au))
        eng.md_steps(1, sp_inj)
        for t, o in enumerate(orcs):
            sh = o.r.shape
            o.propagate_1(sp, randy[t].reshape(sh), zeta[t].reshape(sh), av[t].reshape(sh), au[t].reshape(sh[:2]))
            o.calc_force(sp)
            o.propagate_2(sp, randy[t].reshape(sh))
    q = eng.query(sp)
    eng.close()
    return q, orcs


@pytest.mark.parametrize("case", ["au_single_bead", "pt_rpmd"])
def test_query_energies_match_oracle(built_lib, oracle_lib, case):
    rng = np.random.default_rng(11)
    if case == "au_single_bead":
        us = [W.h_on_metal(rng, "Au", 3 + t % 2, 1.5, 30.0, 40.0 * t, 300.0, C.PROP_ID_VERLET,
                           C.PROP_ID_LANGEVIN_CONST, z0=2.0) for t in range(3)]
        emt = W.emt_params()
        sp = SimParams(step=0.1, gamma_const=1e-3)
    else:
        us = []
        for t, nb in enumerate((4, 8)):
            u = W.h_on_metal(rng, "Pt", 3, 0.5, 0.0, 0.0, 300.0, C.PROP_ID_PILE, C.PROP_ID_PILE, z0=1.8, nbeads=nb)
            u.r += rng.normal(scale=0.02, size=u.r.shape) * (~u.is_fixed)
            us.append(u)
        emt = W.emt_params("H", "Pt")
        sp = SimParams(step=0.1, Tsurf=300.0, Tproj=300.0)
    q, orcs = _run(us, emt, sp, steps=3)
    for t, o in enumerate(orcs):
        ep, el = o.atom_ekin()
        assert _close(q["epot"][t], float(np.mean(o.epot))), (t, q["epot"][t], o.epot)
        assert _close(q["ekin_p"][t], ep), (t, q["ekin_p"][t], ep)
        assert _close(q["ekin_l"][t], el), (t, q["ekin_l"][t], el)
        assert _close(q["ebead"][t], o.bead_epot(sp)), (t, q["ebead"][t], o.bead_epot(sp))
        assert q["steps_done"][t] == 3 and q["status"][t] == 0
    if case == "pt_rpmd":
        assert np.all(q["ebead"] > 0.0)
