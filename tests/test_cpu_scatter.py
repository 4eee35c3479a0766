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


def test_mxt_fin_layout_and_times(tmp_path):
    """The record has the 23 lines the summary script requires, every value reads back,
    and time / cl_appr_time follow output_scatter and check_for_closest_approach."""
    from md_tian2_gb300.scatter import read_mxt_fin, record_times, write_mxt_fin
    rng = np.random.default_rng(2)
    r = _result(rng, 3, 0.1, 0.0)
    r.status = np.array([1, 0, 1])
    r.steps = np.array([120, 400, 7])
    r.record = {"ekin_l_i": np.array([0.9, 1.0, 1.1]), "epot_i": np.array([-392.2094094123, -10.0, -0.5]),
                "etotal_i": np.array([-369.3, -9.0, 0.5]), "r_i": rng.normal(size=(3, 3)),
                "v_i": np.array([[0.01, 0.0, -0.2], [0.0, 0.01, -0.1], [0.1, 0.1, -0.1]]),
                "ekin_l_f": np.array([0.95, 1.0, 1.2]), "epot_f": np.array([-391.9, -10.1, -0.4]),
                "etotal_f": np.array([-369.3, -9.0, 0.5]), "r_f": rng.normal(size=(3, 3)),
                "v_f": np.array([[0.0, 0.01, 0.15], [0.0, 0.0, -0.1], [0.1, 0.0, 0.1]]), "step": 0.1,
                "max_steps": 400, "turn_pnts": np.array([1, 4, 0], np.int32), "cl_appr": np.array([1.5, 0.9, 2.0]),
                "cl_appr_step": np.array([60, 399, 7], np.int32), "r_min_p": rng.normal(size=(3, 3))}
    time, clt = record_times(r)
    assert np.allclose(time, [11.9, 40.0, 0.6])
    # exited at 120 with the minimum at 60: 60 dt^(120 - 60 + 1); ran to 400 (401 collects)
    assert np.allclose(clt, [60 * 0.1 ** 61, 399 * 0.1 ** 3, 7 * 0.1])
    paths = write_mxt_fin(tmp_path, r, first_id=5)
    assert [p.name for p in paths] == ["mxt_fin00000005.dat", "mxt_fin00000006.dat", "mxt_fin00000007.dat"]
    for t, p in enumerate(paths):
        lines = p.read_text().splitlines()
        assert len(lines) == 23 and lines[8] == "" and lines[17] == ""
        d = read_mxt_fin(p)
        assert abs(d["epot_i"] - r.record["epot_i"][t]) < 1e-9 * max(1.0, abs(r.record["epot_i"][t]))
        assert np.allclose(d["v_f"], r.record["v_f"][t], atol=1e-7)
        assert d["turn_pnts"] == r.record["turn_pnts"][t]
        assert abs(d["time"] - time[t]) < 1e-6
        v = r.record["v_i"][t]
        assert abs(d["polar_i"] - (180 - np.degrees(np.arccos(v[2] / np.linalg.norm(v))))) < 1e-6
    assert "-0.3922094094E+03" in paths[0].read_text()


def test_trajectory_info_restatement():
    """The checker of the device observables on a hand-made projectile path: moving down
    at the start, a turning point at each sign change of v_z, the first closest step, the
    lowest centroid, and the minimum image across the cell boundary."""
    from oracle.trajectory_info import TrajectoryInfo
    ti = TrajectoryInfo(np.eye(3) * 10.0)
    path = [(5.0, -1.0), (3.0, -1.0), (2.0, 1.0), (4.0, 1.0), (3.5, -1.0), (2.0, -1.0)]
    for k, (z, vz) in enumerate(path, start=1):
        r = np.array([[[9.5, 1.0, z]], [[0.5, 1.0, 0.0]]])  # 1 A apart in x through the boundary
        v = np.array([[[0.0, 0.0, vz]], [[0.0, 0.0, 0.0]]])
        ti(k, r, v)
    assert ti.turn == 2
    assert ti.clstep == 3 and abs(ti.cl - np.hypot(1.0, 2.0)) < 1e-12
    assert np.allclose(ti.low, [9.5, 1.0, 2.0])
