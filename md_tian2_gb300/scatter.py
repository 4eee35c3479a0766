"""Scattering observables of a batch of projectile trajectories: the quantities the
reference's analysis script derives from its per-trajectory summary records
(scripts/analysis/2_AnalyzePESTrajectory2.12.py:171-183, 357-411), computed from the
engine's final state instead of from mxt_fin files.

Per trajectory (projectile = atom 0, bead 0):
- eloss = Ekin_p(initial) - Ekin_p(final)             (:174)
- scattered   : final projectile z above its initial z   (:177)
- transmitted : final projectile z below the slab's shot-through limit (:178)
- adsorbed    : neither of the two (:179); the adsorbed fraction is the sticking
  probability.
The energy-loss histogram is taken over scattered trajectories with int(3 n^(1/3)) bins
over [min, max] and density normalisation, as the analysis script does (:357-411).

``run_to_exit`` propagates a batch with ``mdt_md_steps`` in chunks until every
trajectory has left through ``pul``/``pll`` or the step limit is reached (the reference's
nsteps loop with its exit test, src/md_tian2.f90:78-92).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# shot-through limits of the analysis script (A, z of the projectile below the slab)
SHOT_THRU_LIMIT = {"Au": -7.27636607765, "Pd": -6.8256, "C": 0.0}


def numbins(n: int) -> int:
    """Histogram bin count of the analysis script (numbins, :357-366)."""
    return max(1, int(3 * (n ** (1.0 / 3.0))))


@dataclass
class ScatterResult:
    ekin_i: np.ndarray   # projectile kinetic energy at the start (eV)
    ekin_f: np.ndarray   # ... at the end
    z_i: np.ndarray      # projectile z at the start (A)
    z_f: np.ndarray      # ... at the end
    steps: np.ndarray    # MD steps run per trajectory
    status: np.ndarray   # engine status (0 running = stopped by the step limit)
    shot_thru: float

    @property
    def eloss(self) -> np.ndarray:
        return self.ekin_i - self.ekin_f

    @property
    def scattered(self) -> np.ndarray:
        return self.z_f > self.z_i

    @property
    def transmitted(self) -> np.ndarray:
        return self.z_f < self.shot_thru

    @property
    def adsorbed(self) -> np.ndarray:
        return ~(self.scattered | self.transmitted)

    def sticking(self) -> tuple[float, float]:
        """Adsorbed fraction and its binomial standard error."""
        n = len(self.z_f)
        p = float(np.mean(self.adsorbed))
        return p, math.sqrt(max(p * (1.0 - p), 0.25 / n) / n)

    def mean_eloss(self) -> tuple[float, float]:
        """Mean energy loss of the scattered trajectories and its standard error."""
        e = self.eloss[self.scattered]
        if len(e) < 2:
            return float("nan"), float("nan")
        return float(np.mean(e)), float(np.std(e, ddof=1) / math.sqrt(len(e)))

    def eloss_histogram(self, bins: int | None = None, span: tuple[float, float] | None = None):
        """Density histogram of the scattered trajectories' energy loss: (density, edges)."""
        e = self.eloss[self.scattered]
        if len(e) == 0:
            return np.zeros(0), np.zeros(1)
        bins = bins or numbins(len(e))
        span = span or (float(e.min()), float(e.max()))
        return np.histogram(e, bins=bins, range=span, density=True)

    def summary(self) -> dict:
        m, se = self.mean_eloss()
        p, pse = self.sticking()
        return {"trajectories": int(len(self.z_f)), "scattered": int(self.scattered.sum()),
                "transmitted": int(self.transmitted.sum()), "adsorbed": int(self.adsorbed.sum()),
                "sticking": p, "sticking_se": pse, "mean_eloss_eV": m, "mean_eloss_se_eV": se,
                "still_running": int(np.sum(self.status == 0))}


def run_to_exit(eng, sp, precision: str = "fp64", max_steps: int = 10000, chunk: int = 500,
                metal: str = "Au") -> ScatterResult:
    """Propagate the engine's batch (state uploaded, exit test on in ``sp``) until every
    trajectory has stopped or ``max_steps`` have run; returns the scattering record."""
    if not sp.use_exit:
        raise ValueError("run_to_exit needs SimParams.use_exit (the pul/pll exit test)")
    T = eng.T
    q0 = eng.query(sp)
    r0 = eng.download()["r"]
    z_i = np.array([eng.split(r0, t)[0, 0, 2] for t in range(T)])
    eng.calc_force(sp, precision=precision)
    done = 0
    while done < max_steps:
        n = min(chunk, max_steps - done)
        eng.md_steps(n, sp, precision=precision)
        done += n
        if not np.any(eng.query(sp)["status"] == 0):
            break
    q = eng.query(sp)
    r = eng.download()["r"]
    z_f = np.array([eng.split(r, t)[0, 0, 2] for t in range(T)])
    return ScatterResult(ekin_i=q0["ekin_p"].copy(), ekin_f=q["ekin_p"].copy(), z_i=z_i, z_f=z_f,
                         steps=q["steps_done"].copy(), status=q["status"].copy(),
                         shot_thru=SHOT_THRU_LIMIT.get(metal, -np.inf))


def compare(a: ScatterResult, b: ScatterResult) -> dict:
    """Two-sample comparison of two batches' observables: differences of the mean energy
    loss and of the sticking probability in units of their combined standard errors, and
    the two-sample Kolmogorov-Smirnov statistic of the scattered energy losses."""
    ma, sa = a.mean_eloss()
    mb, sb = b.mean_eloss()
    pa, psa = a.sticking()
    pb, psb = b.sticking()
    out = {"mean_eloss_eV": [ma, mb], "mean_eloss_z": (ma - mb) / math.sqrt(sa * sa + sb * sb),
           "sticking": [pa, pb], "sticking_z": (pa - pb) / math.sqrt(psa * psa + psb * psb)}
    ea, eb = np.sort(a.eloss[a.scattered]), np.sort(b.eloss[b.scattered])
    if len(ea) and len(eb):
        grid = np.concatenate([ea, eb])
        cdf_a = np.searchsorted(ea, grid, side="right") / len(ea)
        cdf_b = np.searchsorted(eb, grid, side="right") / len(eb)
        d = float(np.max(np.abs(cdf_a - cdf_b)))
        ne = len(ea) * len(eb) / (len(ea) + len(eb))
        # asymptotic two-sample KS p-value (Kolmogorov distribution, first terms)
        lam = (math.sqrt(ne) + 0.12 + 0.11 / math.sqrt(ne)) * d
        p = 2.0 * sum((-1) ** (k - 1) * math.exp(-2.0 * k * k * lam * lam) for k in range(1, 101))
        out["ks_d"] = d
        out["ks_p"] = float(min(1.0, max(0.0, p)))
    return out
