"""Train the H/Au EMT surrogate on the GPU and write it as an .npz model.

    python -m md_tian2_gb300.train_surrogate --out md_tian2_gb300/data/surrogate_HAu.npz

Steps: FP64 EMT trajectories (config-2 generator) sampled every 50 steps -> scaling
from the training descriptors -> fused GPU training (energy + force loss, Adam) ->
force RMSE against FP64 EMT on held-out configurations from other seeds.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

from . import nene
from .surrogate import Dataset, Trainer, force_rmse, generate_dataset, surrogate_model


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent / "data" / "surrogate_HAu.npz"))
    ap.add_argument("--ntraj", type=int, default=4096)
    ap.add_argument("--nsamples", type=int, default=49)
    ap.add_argument("--every", type=int, default=50)
    ap.add_argument("--epochs", type=float, default=20)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-final", type=float, default=1e-4)
    ap.add_argument("--w-energy", type=float, default=10.0)
    ap.add_argument("--w-force", type=float, default=1.0)
    ap.add_argument("--time-budget", type=float, default=None)
    ap.add_argument("--scale-margin", type=float, default=0.02)
    ap.add_argument("--descriptor", choices=("acsf", "radial"), default="acsf")
    ap.add_argument("--max-neighbors", type=int, default=80)
    ap.add_argument("--seed", type=int, default=11)
    ap.add_argument("--long-samples", type=int, default=0,
                    help="extra samples per trajectory taken every --long-every steps (late-time coverage)")
    ap.add_argument("--long-every", type=int, default=400)
    ap.add_argument("--init", default=None, help="warm start from this .npz model (same descriptor)")
    ap.add_argument("--precision", choices=("fp32", "bf16", "bf16x3"), default="fp32",
                    help="arithmetic of the network products: the training kernel's FP32 lanes, BF16 GEMMs, "
                         "or split-BF16 GEMMs")
    a = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    data = generate_dataset(a.ntraj, a.nsamples, a.every, seed=7)
    if a.long_samples > 0:
        late = generate_dataset(a.ntraj, a.long_samples, a.long_every, seed=8)
        data = Dataset(data.universes + late.universes, np.concatenate([data.energy, late.energy]),
                       data.forces + late.forces)
    t_data = time.perf_counter() - t0
    log(f"dataset: {len(data.universes)} configurations, {sum(u.natoms for u in data.universes)} atoms, {t_data:.1f} s")
    model = nene.load_npz(a.init) if a.init else surrogate_model(a.seed, descriptor=a.descriptor)
    t1 = time.perf_counter()
    tr = Trainer(data, model, scale_margin=a.scale_margin, max_neighbors=a.max_neighbors, keep_function=bool(a.init))
    t_setup = time.perf_counter() - t1
    hist = tr.train(epochs=a.epochs, batch=a.batch, lr=a.lr, lr_final=a.lr_final, w_energy=a.w_energy,
                    w_force=a.w_force, time_budget=a.time_budget, log=log, precision=a.precision)
    report = {"descriptor": a.descriptor, "precision": a.precision, "init": Path(a.init).name if a.init else None,
              "samples": {"every": a.every, "nsamples": a.nsamples, "long_every": a.long_every,
                          "long_samples": a.long_samples}, "max_neighbors": a.max_neighbors, "configs": len(data.universes), "atoms": int(sum(u.natoms for u in data.universes)),
              "dataset_s": t_data, "setup_s": t_setup, "train_s": tr.seconds, "steps": tr.steps,
              "atoms_per_s": tr.atoms_trained / tr.seconds, "train_force_rmse_last": hist[-1][2],
              "train_energy_rmse_last": hist[-1][1]}
    tr.close()
    del data
    held = generate_dataset(512, 8, a.every, seed=1234)
    f32, e32 = force_rmse(model, held, precision="fp32", max_neighbors=a.max_neighbors)
    f64, e64 = force_rmse(model, held, precision="fp64", max_neighbors=a.max_neighbors)
    report.update({"heldout_configs": len(held.universes), "heldout_force_rmse_fp32": f32,
                   "heldout_force_rmse_fp64": f64, "heldout_energy_rmse_per_atom_fp64": e64})
    Path(a.out).parent.mkdir(parents=True, exist_ok=True)
    nene.save_npz(model, a.out)
    Path(a.out).with_suffix(".json").write_text(json.dumps(report, indent=1))
    print(json.dumps(report))


if __name__ == "__main__":
    main()
