"""The reference's own analysis pipeline on GPU-written scatter records.

tests/golden/gpu_scatter_records.npz holds every field of the scatter record of 400
config-1 trajectories (fixed incidence) run to the exit on a GB300 by the fused FP64 EMT
kernel (tests/golden/make_gpu_records.py); scatter.write_mxt_fin writes them as
traj/mxt_fin%08d.dat files.  Copies of the reference's
scripts/analysis/1_CreateMXTSummary2.02.py and 2_AnalyzePESTrajectory2.12.py (stdlib and
numpy only) run unchanged on them in a scratch directory (numpy's histogram2d gets back the
`normed` keyword the script uses); their classification counts and energy-loss histogram
must equal what md_tian2_gb300.scatter computes from the same files
(ScatterResult.from_records) with the shot-through limit the summary script writes into
plot_settings.dat.  Needs the reference checkout (tests/refroot.py); skipped where there is
none."""
import re
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from md_tian2_gb300.scatter import ScatterResult, numbins, write_mxt_fin

from .refroot import reference_root

GOLD = Path(__file__).resolve().parent / "golden" / "gpu_scatter_records.npz"
REF = reference_root()
pytestmark = pytest.mark.skipif(REF is None or not GOLD.exists(), reason="no reference checkout or no GPU records")


def _gpu_result():
    z = np.load(GOLD)
    rec = {k[4:]: (z[k].item() if z[k].ndim == 0 else z[k]) for k in z.files if k.startswith("rec_")}
    return ScatterResult(ekin_i=z["ekin_i"], ekin_f=z["ekin_f"], z_i=z["z_i"], z_f=z["z_f"], steps=z["steps"],
                         status=z["status"], shot_thru=float(z["shot_thru"]), record=rec)


# The analysis script was written for numpy < 1.24, whose histogram2d still took the
# `normed` keyword (same meaning as `density`).  The script runs unchanged; this launcher
# gives numpy back that keyword before running it.
LAUNCH = """
import runpy, sys, numpy
_h2 = numpy.histogram2d
def histogram2d(*a, normed=None, **k):
    if normed is not None:
        k.setdefault("density", normed)
    return _h2(*a, **k)
numpy.histogram2d = histogram2d
script = sys.argv[1]
sys.argv = [script]
runpy.run_path(script, run_name="__main__")
"""


def _run(script, cwd):
    r = subprocess.run([sys.executable, "-c", LAUNCH, script.name], cwd=cwd, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r.stdout


def test_reference_scripts_on_gpu_records(tmp_path):
    ana = REF / "scripts" / "analysis"
    s1 = shutil.copy(ana / "1_CreateMXTSummary2.02.py", tmp_path / "1_CreateMXTSummary2.02.py")
    s2 = shutil.copy(ana / "2_AnalyzePESTrajectory2.12.py", tmp_path / "2_AnalyzePESTrajectory2.12.py")
    files = write_mxt_fin(tmp_path / "traj", _gpu_result())
    assert len(files) == 400
    # the analysis script reads Tsurf from md_tian.inp for its plot parameters
    (tmp_path / "md_tian.inp").write_text("Tsurf 300\n")
    _run(Path(s1), tmp_path)
    summary = (tmp_path / "MXT2Summary.txt").read_text().splitlines()
    assert len(summary) == 1 + len(files)
    settings = dict(l.split() for l in (tmp_path / "plot_settings.dat").read_text().splitlines())
    shot_thru = float(settings["SHOT_THRU_LIMIT"])
    _run(Path(s2), tmp_path)
    log = (tmp_path / "AnalyzePESTrajectory.log").read_text()
    got = {k: int(re.search(rf"trajs {k}: (\d+) out of total", log).group(1))
           for k in ("with scattering", "with adsorption", "transmitted")}

    ours = ScatterResult.from_records(files, shot_thru)
    s = ours.summary()
    assert got["with scattering"] == s["scattered"]
    assert got["with adsorption"] == s["adsorbed"]
    assert got["transmitted"] == s["transmitted"]
    assert s["scattered"] > 0 and s["adsorbed"] > 0  # both outcomes are present in the sample
    # the engine's own classification of the same run (full-precision state, not the records)
    direct = _gpu_result()
    direct.shot_thru = shot_thru
    assert direct.summary()["scattered"] == s["scattered"] and direct.summary()["adsorbed"] == s["adsorbed"]

    # energy-loss histogram of the scattered trajectories (analysis/eloss.txt, column "all")
    rows = np.array([[float(x) for x in l.split()] for l in (tmp_path / "analysis" / "eloss.txt").read_text()
                     .splitlines() if l and not l.startswith("#")])
    dens, edges = ours.eloss_histogram()
    assert len(rows) == len(dens) == numbins(s["scattered"])
    np.testing.assert_allclose(rows[:, 0], 0.5 * (edges[1:] + edges[:-1]), rtol=0, atol=1e-6)
    np.testing.assert_allclose(rows[:, 1], dens, rtol=0, atol=1e-6)
    # and the summary line of each trajectory carries the record's energies
    first = summary[1].split()
    rec = ours
    assert abs(float(first[1]) - rec.ekin_i[0]) < 1e-12 and abs(float(first[13]) - rec.ekin_f[0]) < 1e-12
