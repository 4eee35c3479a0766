"""Learned EMT surrogate: a per-element ACSF -> MLP network trained on the GPU on
energies and forces that the batched FP64 EMT kernels generate.

* dataset: ragged H/Au(111) trajectories (the ``config2`` generator) propagated with
  plain FP64 EMT; every ``every`` steps each trajectory contributes its positions, EMT
  total energy and forces;
* model: 8 G2 + 16 G3 per element (neighbour element Au, 6.5 A cosine cutoff, see
  ``nene.acsf_set``) -> 24-32-32-1 softplus network per element (H, Au);
* training: libmdt_gpu's fused training kernels (network forward/backward, descriptor
  VJP for forces, descriptor JVP + forward-over-reverse sweep for the force-loss
  gradient) and Adam on FP32 master weights;
* use: ``PES_SURROGATE`` in the engine, with FP64 EMT as the fallback for beads whose
  symmetry functions leave the training range.
"""
from __future__ import annotations

import ctypes as ct
import time
from dataclasses import dataclass

from pathlib import Path

import numpy as np

from . import constants as C
from . import nene
from . import workloads as W
from ._lib import TrainOpts
from .engine import PES_EMT, PES_NENE, PES_SURROGATE, Engine, SimParams


@dataclass
class Dataset:
    universes: list         # one single-bead Universe per configuration
    energy: np.ndarray      # eV per configuration
    forces: list            # (N, 3) eV/A per configuration


def generate_dataset(ntraj: int = 4096, nsamples: int = 8, every: int = 50, seed: int = 7, device: int = 0,
                     precision: str = "fp64") -> Dataset:
    """Propagate ``ntraj`` config-2 trajectories with EMT and sample every ``every`` steps."""
    us = W.config2(ntraj, seed=seed)
    emt = W.emt_params()
    sp = SimParams(step=0.1, gamma_const=1e-3, seed=seed)
    eng = Engine(device)
    eng.read_emt(emt)
    eng.define(us)
    eng.upload()
    eng.calc_force(sp, precision=precision)
    out_u, out_e, out_f = [], [], []
    for s in range(nsamples):
        eng.md_steps(every, sp, precision=precision)
        o = eng.download()  # forces and energies of the current positions (precision given)
        for t, u in enumerate(us):
            r = eng.split(o["r"], t)
            f = eng.split(o["f"], t)[:, 0, :]
            v = W.Universe(r=r.copy(), v=np.zeros_like(r), m=u.m, idx=u.idx, is_fixed=u.is_fixed, simbox=u.simbox,
                           names=u.names, is_proj=u.is_proj, algo=u.algo)
            out_u.append(v)
            out_e.append(o["epot"][eng.bead_off[t]])
            out_f.append(f.copy())
    eng.close()
    return Dataset(out_u, np.array(out_e), out_f)


SHIPPED = Path(__file__).resolve().parent / "data" / "surrogate_radial.npz"


def shipped_surrogate() -> nene.NNModel:
    """The trained H/Au surrogate shipped with the package (24 radial G2 -> 32 -> 32 -> 1
    softplus; provenance in data/surrogate_radial.json)."""
    return nene.load_npz(SHIPPED)


def surrogate_model(seed: int = 11, descriptor: str = "acsf") -> nene.NNModel:
    """Untrained surrogate network: ``descriptor`` "acsf" = 8 G2 + 16 G3 per element over
    Au neighbours (``nene.acsf_set``), "radial" = 24 G2 over Au and H neighbours
    (``nene.radial_set``); 24-32-32-1 softplus."""
    nbr = ["Au"] if descriptor == "acsf" else ["H", "Au"]
    return nene.random_model(["H", "Au"], hidden=(32, 32), act="p", seed=seed, neighbours=nbr,
                             descriptor=descriptor)


def _opts(lr, w_energy, w_force, precision):
    """precision: fp64 (gradient checks), fp32 (the training kernel's own network on CUDA
    cores), bf16 (the network's products as BF16 GEMMs on the tensor cores, FP32 master
    weights and accumulation) or bf16x3 (the same with split BF16 operands)."""
    return TrainOpts(w_energy, w_force, lr, 0.9, 0.999, 1e-8, {"fp64": 0, "fp32": 1, "bf16": 2, "bf16x3": 3}[precision])


class Trainer:
    """Holds a training set on the GPU (one configuration per batch trajectory)."""

    def __init__(self, data: Dataset, model: nene.NNModel, device: int = 0, scale_margin: float = 0.0,
                 max_neighbors: int = 0, keep_function: bool = False):
        """keep_function: the model is already trained (warm start); its first layer is
        changed with the new scaling so that it starts from the same function."""
        self.data = data
        self.model = model
        self.eng = Engine(device)
        self.eng.define(data.universes)
        self.eng.upload()
        # scaling.data from the training set's own descriptors (RuNNer's scaling mode)
        self.eng.read_nene(model, data.universes[0].names, max_neighbors=max_neighbors)
        self.eng.set_pes(PES_NENE, 0.0)
        G = self.eng.nn_descriptors()
        elem = np.concatenate([[model.elements.index(u.names[i - 1]) for i in u.idx] for u in data.universes])
        old = ([np.array(x) for x in model.smin], [np.array(x) for x in model.smax]) if keep_function else None
        nene.set_scaling(model, G, elem, margin=scale_margin)
        if old is not None:
            nene.rescale_first_layer(model, *old)
        self.eng.read_nene(model, data.universes[0].names, max_neighbors=max_neighbors)
        self.eng.set_pes(PES_NENE, 0.0)
        forces = np.concatenate([f.reshape(-1) for f in data.forces])
        self.eng._check(self.eng.lib.mdt_train_set_labels(self.eng.h, np.ascontiguousarray(data.energy).ctypes.data,
                                                          np.ascontiguousarray(forces).ctypes.data),
                        "mdt_train_set_labels")
        self.n = len(data.universes)

    def gradient(self, conf_ids, w_energy=1.0, w_force=1.0, precision="fp64"):
        ids = np.ascontiguousarray(conf_ids, np.int32)
        nw = self.model.nelem * max(self.model.n_weights(e) for e in range(self.model.nelem))
        g = np.zeros(nw)
        o = _opts(0.0, w_energy, w_force, precision)
        self.eng._check(self.eng.lib.mdt_train_gradient(self.eng.h, ct.byref(o), ids.ctypes.data, len(ids),
                                                        g.ctypes.data), "mdt_train_gradient")
        return g

    def train(self, epochs: float = 10, batch: int = 256, lr: float = 2e-3, lr_final: float = 2e-4,
              w_energy: float = 10.0, w_force: float = 1.0, seed: int = 0, time_budget: float | None = None,
              log=None, precision: str = "fp32"):
        rng = np.random.default_rng(seed)
        nsteps = max(1, int(epochs * self.n / batch))
        stats = np.zeros(3)
        t0 = time.perf_counter()
        order = rng.permutation(self.n)
        pos = 0
        hist = []
        for k in range(nsteps):
            if pos + batch > self.n:
                order = rng.permutation(self.n)
                pos = 0
            ids = np.ascontiguousarray(order[pos:pos + batch], np.int32)
            pos += batch
            frac = k / max(1, nsteps - 1)
            o = _opts(lr * (lr_final / lr) ** frac, w_energy, w_force, precision)
            self.eng._check(self.eng.lib.mdt_train_step(self.eng.h, ct.byref(o), ids.ctypes.data, len(ids),
                                                        stats.ctypes.data), "mdt_train_step")
            hist.append((k, float(np.sqrt(stats[0])), float(np.sqrt(stats[1]))))
            if log and (k % 50 == 0 or k == nsteps - 1):
                log(f"step {k}/{nsteps} energy rmse/atom {np.sqrt(stats[0]) * 1e3:.2f} meV "
                    f"force rmse {np.sqrt(stats[1]) * 1e3:.2f} meV/A")
            if time_budget and time.perf_counter() - t0 > time_budget:
                break
        self.seconds = time.perf_counter() - t0
        self.steps = len(hist)
        self.atoms_trained = self.steps * batch * float(np.mean([u.natoms for u in self.data.universes]))
        w = np.zeros(self.model.nelem * max(self.model.n_weights(e) for e in range(self.model.nelem)))
        self.eng._check(self.eng.lib.mdt_train_commit(self.eng.h, w.ctypes.data), "mdt_train_commit")
        mw = max(self.model.n_weights(e) for e in range(self.model.nelem))
        for e in range(self.model.nelem):
            self.model.weights[e] = w[e * mw: e * mw + self.model.n_weights(e)].copy()
        return hist

    def close(self):
        self.eng.close()


def force_rmse(model: nene.NNModel, data: Dataset, device: int = 0, precision: str = "fp32",
               max_neighbors: int = 0) -> tuple:
    """Force RMSE (eV/A) and per-atom energy RMSE (eV) of the network on a dataset."""
    eng = Engine(device)
    eng.define(data.universes)
    eng.upload()
    eng.read_nene(model, data.universes[0].names, max_neighbors=max_neighbors)
    eng.set_pes(PES_NENE, 0.0)
    eng.calc_force(SimParams(), precision=precision)
    out = eng.download()
    eng.close()
    f = np.concatenate([fr.reshape(-1) for fr in data.forces])
    nat = np.array([u.natoms for u in data.universes])
    return (float(np.sqrt(np.mean((out["f"] - f) ** 2))),
            float(np.sqrt(np.mean(((out["epot"] - data.energy) / nat) ** 2))))


def nve_drift(model: nene.NNModel, precision: str = "fp32", ntraj: int = 8, chunk: int = 200, nchunks: int = 100,
              seed: int = 4, device: int = 0) -> dict:
    """NVE energy drift of the surrogate path: velocity Verlet with no friction, all atoms
    free, ``ntraj`` H/Au(111) 3x3 trajectories (H at 2.5 A, 1 eV, polar 30 deg) for
    chunk x nchunks steps of 0.1 fs, forces from the network (``precision``).  The total
    energy is read every chunk from the per-trajectory FP64 sums of an FP32 evaluation of the
    same network: for BF16 dynamics that measures what the dynamics conserve rather than the
    BF16 energy readout, whose operand rounding adds O(10) meV of noise per configuration.
    Returns the slope of a linear fit of E_tot(t) per trajectory (meV/ps), their mean, the
    spread of the BF16 readout against FP32 (``readout_rms_meV``) and the EMT fallbacks (a
    fallback switches the potential, so it must be zero for the slopes to measure drift)."""
    rng = np.random.default_rng(seed)
    us = [W.h_on_metal(rng, "Au", 3, 1.0, 30.0, 0.0, 300.0, z0=2.5) for _ in range(ntraj)]
    for u in us:
        u.is_fixed[:] = False

    def engine():
        e = Engine(device)
        e.read_emt(W.emt_params())
        e.define(us)
        e.read_nene(model, ["H", "Au"])
        e.set_pes(PES_SURROGATE, 0.1)
        e.upload()
        return e

    eng = engine()
    radial = eng.nn_radial_kernel(True)
    probe = engine() if precision != "fp32" else None  # FP32 energies of the same states
    sp = SimParams(step=0.1)
    eng.calc_force(sp, precision=precision)
    ts, es, dev = [], [], []
    for c in range(nchunks + 1):
        if c:
            eng.md_steps(chunk, sp, precision=precision)
        q = eng.query(sp)
        epot = q["epot"]
        if probe is not None:
            o = eng.download()
            probe.upload(o["r"], o["v"])
            probe.calc_force(sp, flag=C.ENERGY_ONLY, precision="fp32")
            e32 = probe.query(sp)["epot"]
            dev.append(epot - e32)
            epot = e32
        ts.append(c * chunk * sp.step * 1e-3)  # ps
        es.append(epot + q["ekin_p"] + q["ekin_l"])
    fb, _ = eng.nn_stats()
    steps_ok = bool(np.all(q["steps_done"] == chunk * nchunks))
    eng.close()
    if probe is not None:
        probe.close()
    es = np.array(es)
    slope = np.array([np.polyfit(ts, es[:, t], 1)[0] for t in range(ntraj)]) * 1e3
    return {"slopes_meV_per_ps": slope, "mean_meV_per_ps": float(np.mean(slope)),
            "max_abs_meV_per_ps": float(np.max(np.abs(slope))), "fallbacks": int(fb.sum()),
            "steps_ok": steps_ok, "radial_kernel": bool(radial), "ps": chunk * nchunks * sp.step * 1e-3,
            "readout_rms_meV": float(1e3 * np.sqrt(np.mean(np.square(dev)))) if dev else 0.0}
