"""What the trained surrogate gains over the method without it (plain EMT), on the GPU:

- accuracy: force RMSE of the shipped network against FP64 EMT on held-out
  configurations (other seeds than training) stays within 20 meV/A;
- speed: its fused MD step is at least 2.5x faster than the FP64 EMT step on the same
  ragged batch (the bench measures ~4x; the bar leaves room for a shared GPU);
- physics: from identical initial states, the scattering observables of the reference's
  analysis (mean energy loss of scattered projectiles, sticking probability, energy-loss
  distribution) agree with FP64 EMT within statistical error (|z| < 3.5, two-sample KS
  p > 0.01)."""
import time
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300 import nene
from md_tian2_gb300 import workloads as W
from md_tian2_gb300.engine import PES_EMT, PES_SURROGATE, Engine, SimParams
from md_tian2_gb300.scatter import compare, run_to_exit
from md_tian2_gb300.surrogate import force_rmse, generate_dataset

pytestmark = pytest.mark.gpu
MODEL = Path(__file__).resolve().parents[1] / "md_tian2_gb300" / "data" / "surrogate_radial.npz"


def _engine(us, kind):
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.read_nene(nene.load_npz(MODEL), ["H", "Au"], max_neighbors=80)
    eng.set_pes(kind, 0.1)
    eng.upload()
    return eng


def test_trained_surrogate_accuracy_on_held_out_emt(built_lib):
    held = generate_dataset(128, 4, 50, seed=4343)
    frmse, ermse = force_rmse(nene.load_npz(MODEL), held, precision="fp32", max_neighbors=80)
    assert frmse < 0.020, frmse
    assert ermse < 0.005, ermse


def test_surrogate_step_faster_than_fp64_emt(built_lib):
    us = W.config2(2048, seed=31)
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=3)
    ms = {}
    for kind, prec in ((PES_SURROGATE, "fp32"), (PES_EMT, "fp64")):
        eng = _engine(us, kind)
        eng.calc_force(sp, precision=prec)
        eng.md_steps(5, sp, precision=prec)
        eng.synchronize()
        t0 = time.perf_counter()
        eng.md_steps(40, sp, precision=prec)
        eng.synchronize()
        ms[kind] = (time.perf_counter() - t0) / 40 * 1e3
        eng.close()
    assert ms[PES_EMT] > 2.5 * ms[PES_SURROGATE], ms


def test_scattering_observables_match_fp64_emt(built_lib):
    us = W.config2(768, seed=32)
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=5, pul=6.05, use_exit=True)
    res = {}
    for kind, prec in ((PES_EMT, "fp64"), (PES_SURROGATE, "fp32")):
        eng = _engine(us, kind)
        res[kind] = run_to_exit(eng, sp, precision=prec, max_steps=4000, chunk=500)
        if kind == PES_SURROGATE:
            fb, _ = eng.nn_stats()
        eng.close()
    a, b = res[PES_EMT], res[PES_SURROGATE]
    assert a.scattered.sum() > 100 and b.scattered.sum() > 100
    c = compare(b, a)
    assert abs(c["mean_eloss_z"]) < 3.5, c
    assert abs(c["sticking_z"]) < 3.5, c
    assert c["ks_p"] > 0.01, c
