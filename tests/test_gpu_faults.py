"""Failures injected on the host retire one trajectory and leave the rest of the batch
untouched.

* A NaN position in a Verlet trajectory: the fused MD steps stop it with status
  MDT_TRAJ_ERR_NONFINITE (-11) after the step in which it appears (the reference would
  carry the NaN to the end of its run).
* A negative EMT density under LDFA Langevin stops the trajectory with
  MDT_TRAJ_ERR_DENSITY (-10), where the reference stops the program ("EMT density array
  contains negative values", md_algo.f90:551-554); a NaN position in an LDFA trajectory stops
  that trajectory with an error status.
* A projectile placed 0.05 A from a lattice atom: huge but finite forces; whatever that
  trajectory does, the others are unaffected.
Every other trajectory must equal a clean run of the same batch: bit for bit where the
kernel is deterministic (checked by running the clean batch twice), else within the
run-to-run spread of the kernel's unordered FP32 shared-memory sums.

* The tensor-core network's bounded wait, on a barrier that nothing completes: it gives up
  within its poll limit, reports the time-out, and the GPU goes on computing correctly."""
import numpy as np
import pytest

from md_tian2_gb300 import constants as C
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.surrogate import shipped_surrogate

pytestmark = pytest.mark.gpu
ERR_NONFINITE, ERR_DENSITY = -11, -10


def _slots(us, t):
    off = np.concatenate([[0], np.cumsum([u.natoms * u.nbeads for u in us])])
    return slice(3 * off[t], 3 * off[t + 1])


def _emt_run(us, algo_h, steps=40):
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.upload()
    sp = SimParams(step=0.1, gamma_const=1e-3, Tsurf=300.0, Tproj=300.0)
    eng.calc_force(sp)
    eng.md_steps(steps, sp)
    out, q = eng.download(), eng.query(sp)
    eng.close()
    return out, q


def _batch(algo_h, n=6, seed=5):
    rng = np.random.default_rng(seed)
    return [W.h_on_metal(rng, "Au", 3 + t % 3, 2.0, 20.0, 60.0 * t, 300.0, algo_h, C.PROP_ID_LANGEVIN_CONST,
                         z0=2.5) for t in range(n)]


def _faulted(us, nan_traj, close_traj):
    bad = [u.copy() for u in us]
    bad[nan_traj].r[5, 0, 0] = np.nan
    if close_traj is not None:
        u = bad[close_traj]
        u.r[0, 0, :] = u.r[1, 0, :] + np.array([0.05, 0.0, 0.0])  # H onto the first Au atom
    return bad


def _assert_others_equal(us, out, clean, clean2, skip, rtol):
    deterministic = all(np.array_equal(clean[k], clean2[k]) for k in ("r", "v"))
    for t in range(len(us)):
        if t in skip:
            continue
        sl = _slots(us, t)
        for k in ("r", "v", "f"):
            a, b = out[k][sl], clean[k][sl]
            if deterministic:
                assert np.array_equal(a, b), (t, k)
            else:
                assert np.max(np.abs(a - b)) <= rtol * max(1.0, np.max(np.abs(b))), (t, k)
    return deterministic


def test_nan_and_close_pair_in_emt_batch(built_lib):
    us = _batch(C.PROP_ID_VERLET)
    clean, qc = _emt_run(us, C.PROP_ID_VERLET)
    clean2, _ = _emt_run(us, C.PROP_ID_VERLET)
    out, q = _emt_run(_faulted(us, 1, 3), C.PROP_ID_VERLET)
    assert q["status"][1] == ERR_NONFINITE and q["steps_done"][1] == 1, q[1]
    assert np.all(qc["status"] == 0)
    others = [t for t in range(len(us)) if t not in (1, 3)]
    assert np.all(q["status"][others] == 0) and np.all(q["steps_done"][others] == 40)
    # FP64 shared-memory density atomics in no fixed order: runs may differ in the last bit
    _assert_others_equal(us, out, clean, clean2, skip=(1, 3), rtol=1e-10)


def test_negative_density_stops_ldfa_trajectories(built_lib):
    """A negative EMT density (here from a negative n0 of H, so every trajectory has one) is
    the reference's `stop` in ldfa (md_algo.f90:551-554): every trajectory ends after its
    first step with MDT_TRAJ_ERR_DENSITY."""
    us = _batch(C.PROP_ID_LANGEVIN, n=4)
    emt = W.emt_params()
    emt.values["n0"][0] = -abs(emt.values["n0"][0])
    eng = Engine(0)
    eng.read_emt(emt)
    eng.define(us)
    eng.upload()
    sp = SimParams(step=0.1, gamma_const=1e-3, Tsurf=300.0, Tproj=300.0)
    eng.calc_force(sp)
    eng.md_steps(10, sp)
    q = eng.query(sp)
    eng.close()
    assert np.all(q["status"] == ERR_DENSITY) and np.all(q["steps_done"] == 1), q


def test_nan_in_ldfa_batch_stops_only_its_trajectory(built_lib):
    us = _batch(C.PROP_ID_LANGEVIN, n=4)
    bad = [u.copy() for u in us]
    bad[2].r[0, 0, 2] = np.nan  # the projectile, whose density feeds ldfa
    out, q = _emt_run(bad, C.PROP_ID_LANGEVIN, steps=10)
    assert q["status"][2] < 0 and q["steps_done"][2] == 1, q[2]
    assert np.all(q["status"][[0, 1, 3]] == 0) and np.all(q["steps_done"][[0, 1, 3]] == 10)


def test_nan_in_surrogate_batch(built_lib):
    """The thread-per-atom surrogate kernel (FP32 forces, packs of several trajectories
    per CTA): the NaN trajectory stops within two steps, its pack neighbours run on."""
    us = W.config2(12, seed=31)
    emt = W.emt_params()
    m = shipped_surrogate()

    def run(batch, steps=30):
        eng = Engine(0)
        eng.read_emt(emt)
        eng.define(batch)
        eng.read_nene(m, ["H", "Au"])
        eng.set_pes(PES_SURROGATE, 0.1)
        assert eng.nn_radial_kernel(True)
        eng.upload()
        sp = SimParams(step=0.1, gamma_const=1e-3)
        eng.calc_force(sp, precision="fp32")
        eng.md_steps(steps, sp, precision="fp32")
        o, qq = eng.download(), eng.query(sp)
        eng.close()
        return o, qq

    clean, qc = run(us)
    clean2, _ = run(us)
    out, q = run(_faulted(us, 4, None))
    assert q["status"][4] == ERR_NONFINITE and q["steps_done"][4] <= 2, q[4]
    others = [t for t in range(len(us)) if t != 4]
    assert np.all(q["status"][others] == qc["status"][others])
    assert np.all(q["steps_done"][others] == qc["steps_done"][others])
    # unordered red.shared sums: runs of the same batch differ by FP32 rounding
    _assert_others_equal(us, out, clean, clean2, skip=(4,), rtol=1e-6)


def test_tensor_core_wait_gives_up_and_the_gpu_stays_usable(built_lib):
    import ctypes as ct
    from md_tian2_gb300._lib import load
    lib = load()
    to, ms = ct.c_int32(-1), ct.c_double(-1.0)
    assert lib.mdt_wait_check(0, 1, ct.byref(to), ct.byref(ms)) == 0
    assert to.value == 0  # a completed phase is seen
    assert lib.mdt_wait_check(0, 0, ct.byref(to), ct.byref(ms)) == 0
    assert to.value == 1  # the lost completion ends in the error word
    assert 0.0 < ms.value < 5000.0, ms.value  # within the limit, not a hang
    # the context-free check left the device usable: a split-BF16 evaluation right after
    # agrees with FP32 on the same batch, and its own error word stays clear
    us = W.config2(8, seed=65)
    res = {}
    for prec in ("fp32", "bf16x3"):
        eng = Engine(0)
        eng.read_emt(W.emt_params())
        eng.define(us)
        eng.read_nene(shipped_surrogate(), ["H", "Au"], max_neighbors=80)
        eng.set_pes(PES_SURROGATE, 0.1)
        eng.upload()
        eng.calc_force(SimParams(), precision=prec)
        eng.synchronize()
        res[prec] = eng.download()["f"]
        eng.close()
    rms = np.sqrt(np.mean(res["fp32"] ** 2))
    assert np.sqrt(np.mean((res["bf16x3"] - res["fp32"]) ** 2)) < 2e-4 * rms
