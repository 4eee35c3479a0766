"""Scatter records of a GPU run for the CPU tests that feed the reference's own analysis
scripts: 400 config-1 H/Au(111) trajectories (3x3 slab, Einc 2.76 eV, polar 45 deg,
azimuth 0, Verlet, dt 0.1 fs, FP64 EMT) run by the fused MD kernel to the exit (z > 6.05 A)
or 6000 steps, observables tracked on the device.  Saves every field that output_scatter
writes (src/output_mod.f90:634-697) to tests/golden/gpu_scatter_records.npz; the tests
write the traj/mxt_fin%08d.dat files from it with scatter.write_mxt_fin.  Fixed incidence,
as in the experiments the analysis scripts were written for (their in-plane, specular and
ion-imaging selections need it).  Needs a GPU:  python tests/golden/make_gpu_records.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))


def main():
    from md_tian2_gb300 import workloads as W
    from md_tian2_gb300.engine import Engine, SimParams
    from md_tian2_gb300.scatter import run_to_exit
    us = W.config1(400, seed=77)
    eng = Engine(0)
    eng.read_emt(W.emt_params())
    eng.define(us)
    eng.upload()
    sp = SimParams(step=0.1, pul=6.05, use_exit=True, seed=7)
    res = run_to_exit(eng, sp, precision="fp64", max_steps=6000, chunk=1000)
    eng.close()
    flat = {f"rec_{k}": np.asarray(v) for k, v in res.record.items()}
    np.savez_compressed(HERE / "gpu_scatter_records.npz", ekin_i=res.ekin_i, ekin_f=res.ekin_f, z_i=res.z_i,
                        z_f=res.z_f, steps=res.steps, status=res.status, shot_thru=res.shot_thru, **flat)
    print(f"{len(res.z_f)} records written; {res.summary()}")


if __name__ == "__main__":
    main()
