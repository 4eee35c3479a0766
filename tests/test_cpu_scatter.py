"""Host logic of the scattering observables (no GPU): the analysis script's classes,
bin rule and the two-sample comparison on synthetic records."""
import numpy as np

from md_tian2_gb300.scatter import SHOT_THRU_LIMIT, ScatterResult, compare, numbins


def _result(rng, n, loss_mean, stick):
    z_i = np.full(n, 6.0)
    fate = rng.random(n)
    z_f = np.where(fate < stick, 1.0, 6.05)
    z_f[:3] = -8.0  # shot through the slab
    ekin_i = rng.uniform(0.5, 5.0, n)
    ekin_f = ekin_i - rng.normal(loss_mean, 0.05, n)
    return ScatterResult(ekin_i=ekin_i, ekin_f=ekin_f, z_i=z_i, z_f=z_f, steps=np.full(n, 100),
                         status=np.where(z_f > 6.0, 1, 0), shot_thru=SHOT_THRU_LIMIT["Au"])


def test_classes_and_histogram():
    rng = np.random.default_rng(0)
    r = _result(rng, 1000, 0.1, 0.2)
    assert (r.scattered ^ r.transmitted ^ r.adsorbed).all()
    assert r.transmitted.sum() == 3
    s = r.summary()
    assert s["scattered"] + s["transmitted"] + s["adsorbed"] == 1000
    dens, edges = r.eloss_histogram()
    assert len(dens) == numbins(int(r.scattered.sum())) == int(3 * r.scattered.sum() ** (1 / 3))
    assert abs(np.sum(dens * np.diff(edges)) - 1.0) < 1e-12
    assert abs(r.mean_eloss()[0] - 0.1) < 0.01


def test_compare_detects_shifts_only_when_present():
    rng = np.random.default_rng(1)
    a, b = _result(rng, 4000, 0.1, 0.2), _result(rng, 4000, 0.1, 0.2)
    c = compare(a, b)
    assert abs(c["mean_eloss_z"]) < 4 and abs(c["sticking_z"]) < 4 and c["ks_p"] > 1e-3
    d = compare(a, _result(rng, 4000, 0.15, 0.3))
    assert abs(d["mean_eloss_z"]) > 10 and abs(d["sticking_z"]) > 6 and d["ks_p"] < 1e-6
