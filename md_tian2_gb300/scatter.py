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
nsteps loop with its exit test, src/md_tian2.f90:78-98), and collects the fields of the
reference's per-trajectory scatter record; ``write_mxt_fin`` writes them as the
reference's ``traj/mxt_fin%08d.dat`` files (output_scatter, src/output_mod.f90:634-697),
which its summary scripts (scripts/analysis/1_CreateMXTSummary2.02.py) read unchanged.
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
    # the rest of the reference's scatter record (None when not collected)
    record: dict | None = None

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

    @classmethod
    def from_records(cls, paths, shot_thru: float) -> "ScatterResult":
        """The observables of a set of mxt_fin files (read_mxt_fin), as the analysis script
        classifies them: initial and final projectile energy and height from the records."""
        recs = [read_mxt_fin(p) for p in paths]
        col = lambda k: np.array([r[k] for r in recs])  # noqa: E731
        return cls(ekin_i=col("ekin_p_i"), ekin_f=col("ekin_p_f"), z_i=np.array([r["r_i"][2] for r in recs]),
                   z_f=np.array([r["r_f"][2] for r in recs]), steps=np.rint(col("time")).astype(np.int64),
                   status=np.ones(len(recs), np.int32), shot_thru=shot_thru)

    def summary(self) -> dict:
        m, se = self.mean_eloss()
        p, pse = self.sticking()
        return {"trajectories": int(len(self.z_f)), "scattered": int(self.scattered.sum()),
                "transmitted": int(self.transmitted.sum()), "adsorbed": int(self.adsorbed.sum()),
                "sticking": p, "sticking_se": pse, "mean_eloss_eV": m, "mean_eloss_se_eV": se,
                "still_running": int(np.sum(self.status == 0))}


def run_to_exit(eng, sp, precision: str = "fp64", max_steps: int = 10000, chunk: int = 500,
                metal: str = "Au", repack: bool = True) -> ScatterResult:
    """Propagate the engine's batch (state uploaded, exit test on in ``sp``) until every
    trajectory has stopped or ``max_steps`` have run; returns the scattering record.  With
    ``repack`` the thread-per-atom kernel's CTAs are re-packed over the running trajectories
    after every chunk in which some stopped (no effect on the other kernels)."""
    if not sp.use_exit:
        raise ValueError("run_to_exit needs SimParams.use_exit (the pul/pll exit test)")
    T = eng.T
    eng.calc_force(sp, precision=precision)  # epot_i: output follows calc_force (md_tian2.f90:69-73)
    q0 = eng.query(sp)
    o0 = eng.download()
    z_i = np.array([eng.split(o0["r"], t)[0, 0, 2] for t in range(T)])
    done = 0
    running = T
    while done < max_steps:
        n = min(chunk, max_steps - done)
        eng.md_steps(n, sp, precision=precision)
        done += n
        now = int(np.sum(eng.query(sp)["status"] == 0))
        if now == 0:
            break
        if repack and now < running:  # stopped trajectories give their CTA threads back
            eng.nn_repack()
        running = now
    q = eng.query(sp)
    o = eng.download()
    z_f = np.array([eng.split(o["r"], t)[0, 0, 2] for t in range(T)])

    def centroid(flat, t):  # projectile centroid over beads
        return eng.split(flat, t)[0].mean(axis=0)

    obs = eng.observables()
    record = {"ekin_l_i": q0["ekin_l"].copy(), "epot_i": q0["epot"].copy(),
              "etotal_i": q0["ekin_p"] + q0["ekin_l"] + q0["epot"] + q0["ebead"],
              "r_i": np.array([centroid(o0["r"], t) for t in range(T)]),
              "v_i": np.array([centroid(o0["v"], t) for t in range(T)]),
              "ekin_l_f": q["ekin_l"].copy(), "epot_f": q["epot"].copy(),
              "etotal_f": q["ekin_p"] + q["ekin_l"] + q["epot"] + q["ebead"],
              "r_f": np.array([centroid(o["r"], t) for t in range(T)]),
              "v_f": np.array([centroid(o["v"], t) for t in range(T)]),
              "step": float(sp.step), "max_steps": int(max_steps), **obs}
    return ScatterResult(ekin_i=q0["ekin_p"].copy(), ekin_f=q["ekin_p"].copy(), z_i=z_i, z_f=z_f,
                         steps=q["steps_done"].copy(), status=q["status"].copy(),
                         shot_thru=SHOT_THRU_LIMIT.get(metal, -np.inf), record=record)


# ---- the reference's mxt_fin record -------------------------------------------------------
RAD2DEG = 180.0 / math.pi


def fortran_f(x: float, w: int = 14, d: int = 7) -> str:
    """Fortran Fw.d."""
    return f"{x:{w}.{d}f}"


def fortran_e(x: float, w: int = 21, d: int = 10) -> str:
    """Fortran Ew.d (0.ddddE+xx, d significant digits)."""
    if x == 0.0 or not math.isfinite(x):
        body = ("0." + "0" * d + "E+00") if x == 0.0 else str(x)
        return body.rjust(w)
    mant, exp = f"{abs(x):.{d - 1}e}".split("e")
    body = "0." + mant.replace(".", "") + f"E{int(exp) + 1:+03d}"
    return (("-" if x < 0 else "") + body).rjust(w)


def _polar_azi(v):
    n = math.sqrt(float(np.dot(v, v)))
    polar = math.acos(v[2] / n) * RAD2DEG if n > 0 else float("nan")
    return polar, math.atan2(v[1], v[0]) * RAD2DEG


def record_times(res: ScatterResult) -> tuple[np.ndarray, np.ndarray]:
    """time and cl_appr_time as output_scatter writes them.  The loop of md_tian2.f90:78-98
    leaves at the exit step S (time = (S-1) dt) or runs to completion (istep = nsteps + 1,
    time = nsteps dt, one more collect of the last configuration).  check_for_closest_approach
    (trajectory_info.f90:103-118) sets the time to k (the step of the minimum) and multiplies
    it by dt on every call from then on: k dt^(calls - k + 1)."""
    rec = res.record
    dt = rec["step"]
    exited = res.status != 0
    S = res.steps.astype(np.int64)
    time = np.where(exited, (S - 1) * dt, S * dt)
    calls = np.where(exited, S, S + 1)
    k = rec["cl_appr_step"].astype(np.int64)
    with np.errstate(under="ignore", over="ignore"):
        clt = np.where(k > 0, k * np.power(dt, (calls - k + 1).astype(float)), 0.0)
    return time, clt


def write_mxt_fin(directory, res: ScatterResult, first_id: int = 1) -> list:
    """One traj/mxt_fin%08d.dat file per trajectory, in output_scatter's layout
    (src/output_mod.f90:660-697): the 8-line initial block, a blank line, the 8-line final
    block, a blank line and time, turn_pnts, cl_appr, cl_appr_time, r_min_p."""
    from pathlib import Path
    rec = res.record
    if rec is None:
        raise ValueError("the result holds no scatter record (run_to_exit collects it)")
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    time, clt = record_times(res)
    paths = []
    for t in range(len(res.z_f)):
        pol_i, azi_i = _polar_azi(rec["v_i"][t])
        pol_f, azi_f = _polar_azi(rec["v_f"][t])
        f3 = lambda v: "".join(fortran_f(x) for x in v)  # noqa: E731
        lines = [
            "ekin_p_i = " + fortran_f(res.ekin_i[t]),
            "ekin_l_i = " + fortran_f(rec["ekin_l_i"][t]),
            "epot_i   = " + fortran_e(rec["epot_i"][t]),
            "etotal_i = " + fortran_e(rec["etotal_i"][t]),
            "r_i      = " + f3(rec["r_i"][t]),
            "v_i      = " + f3(rec["v_i"][t]),
            "polar_i  = " + fortran_f(180.0 - pol_i),
            "azi_i    = " + fortran_f(azi_i),
            "",
            "ekin_p_f     = " + fortran_f(res.ekin_f[t]),
            "ekin_l_f     = " + fortran_f(rec["ekin_l_f"][t]),
            "epot_f       = " + fortran_e(rec["epot_f"][t]),
            "etotal_f     = " + fortran_e(rec["etotal_f"][t]),
            "r_f          = " + f3(rec["r_f"][t]),
            "v_f          = " + f3(rec["v_f"][t]),
            "polar_f      = " + fortran_f(pol_f),
            "azi_f        = " + fortran_f(azi_f),
            "",
            "time         = " + fortran_f(time[t]),
            "turn_pnts    = " + f"{int(rec['turn_pnts'][t]):12d}",
            "cl_appr      = " + fortran_f(rec["cl_appr"][t]),
            "cl_appr_time = " + fortran_f(clt[t]),
            "r_min_p      = " + f3(rec["r_min_p"][t]),
        ]
        p = d / f"mxt_fin{first_id + t:08d}.dat"
        p.write_text("\n".join(lines) + "\n")
        paths.append(p)
    return paths


def read_mxt_fin(path) -> dict:
    """The values of one mxt_fin file, taken as the reference's summary script takes them
    (last whitespace-separated token(s) of each line, in line order)."""
    lines = [l for l in open(path).read().splitlines()]
    if len(lines) != 23:
        raise ValueError(f"{path}: {len(lines)} lines, a finished trajectory has 23")
    tok = [l.split() for l in lines]
    vec = lambda i: np.array([float(x) for x in tok[i][-3:]])  # noqa: E731
    num = lambda i: float(tok[i][-1])  # noqa: E731
    return {"ekin_p_i": num(0), "ekin_l_i": num(1), "epot_i": num(2), "etotal_i": num(3), "r_i": vec(4),
            "v_i": vec(5), "polar_i": num(6), "azi_i": num(7), "ekin_p_f": num(9), "ekin_l_f": num(10),
            "epot_f": num(11), "etotal_f": num(12), "r_f": vec(13), "v_f": vec(14), "polar_f": num(15),
            "azi_f": num(16), "time": num(18), "turn_pnts": int(tok[19][-1]), "cl_appr": num(20),
            "cl_appr_time": num(21), "r_min_p": vec(22)}


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


def run_campaign(eng, sp, total: int, refill: dict, precision: str = "fp64", max_steps: int = 10000,
                 chunk: int = 1000, metal: str = "Au") -> ScatterResult:
    """A stream of trajectories through a fixed batch: run ``chunk`` steps, take the
    records of every trajectory that has stopped (exit test or the ``max_steps`` limit),
    restart those slots on the device with new projectile starts (``Engine.refill(**refill)``)
    and go on until ``total`` trajectories have finished.  Returns their scattering records
    (the observables part: energies, projectile heights, steps, status).  A trajectory that
    stops with an error status (negative) is recorded once with that status; refill leaves
    its slot stopped, so the batch goes on with one slot fewer."""
    if not sp.use_exit:
        raise ValueError("run_campaign needs SimParams.use_exit (the pul/pll exit test)")
    if max_steps <= 0:
        raise ValueError("run_campaign needs a step limit (max_steps > 0)")
    eng.set_step_limit(max_steps)
    T = eng.T

    def proj_z(o, t):
        return eng.split(o["r"], t)[0, :, 2].mean()

    eng.calc_force(sp, precision=precision)
    q = eng.query(sp)
    o = eng.download()
    e_start = q["ekin_p"].copy()
    z_start = np.array([proj_z(o, t) for t in range(T)])
    cols = {k: [] for k in ("ekin_i", "ekin_f", "z_i", "z_f", "steps", "status")}
    done = 0
    dead = np.zeros(T, bool)  # slots stopped by an error status, already recorded
    try:
        while done < total:
            if dead.all():
                raise RuntimeError("run_campaign: every trajectory slot stopped with an error status")
            eng.md_steps(chunk, sp, precision=precision)
            q = eng.query(sp)
            fin = np.nonzero((q["status"] != 0) & ~dead)[0]
            if len(fin) == 0:
                continue
            o = eng.download()
            for t in fin[:total - done]:
                cols["ekin_i"].append(e_start[t])
                cols["ekin_f"].append(q["ekin_p"][t])
                cols["z_i"].append(z_start[t])
                cols["z_f"].append(proj_z(o, t))
                cols["steps"].append(q["steps_done"][t])
                cols["status"].append(q["status"][t])
            done += min(len(fin), total - done)
            dead[fin[q["status"][fin] < 0]] = True
            if done >= total:
                break
            eng.refill(**refill)
            eng.calc_force(sp, precision=precision)
            q1 = eng.query(sp)
            o1 = eng.download()
            for t in fin:
                e_start[t] = q1["ekin_p"][t]
                z_start[t] = proj_z(o1, t)
    finally:
        eng.set_step_limit(0)
    a = {k: np.array(v) for k, v in cols.items()}
    return ScatterResult(ekin_i=a["ekin_i"], ekin_f=a["ekin_f"], z_i=a["z_i"], z_f=a["z_f"], steps=a["steps"],
                         status=a["status"], shot_thru=SHOT_THRU_LIMIT.get(metal, -np.inf))
