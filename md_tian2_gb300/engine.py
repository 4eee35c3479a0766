"""Host-side mirror of the reference's force/propagation interface for a batch.

The reference drives one ``universe`` through ``calc_force`` (src/force.f90:40),
``propagate_1``/``propagate_2`` (src/md_algo.f90:37,80) and the step loop of
src/md_tian2.f90:78-92.  :class:`Engine` drives T universes at once through
libmdt_gpu.so with the same names, argument meaning and error behaviour: a bad input
raises (the reference would ``stop``), nothing is silently skipped.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass

import numpy as np

from . import constants as C
from ._lib import EngineError, NNModelC, PropParams, TrajSummary, load
from .io import EmtParams
from .universe import Universe

PREC = {"fp64": 0, "fp32": 1, "bf16": 2, "bf16x3": 3}
PES_EMT, PES_NENE, PES_SURROGATE = C.PES_ID_EMT, C.PES_ID_NENE, 2100


@dataclass
class SimParams:
    """The ``simparams`` fields the hot path reads (src/run_config.f90:34-85)."""

    step: float = 0.1
    Tsurf: float = 300.0
    Tproj: float = 300.0
    pile_tau: float = 200.0        # run_config.f90:120
    andersen_time: float = 30.0    # run_config.f90:119
    gamma_const: float = 0.001     # 1/fs (1/ps), constant-friction Langevin only
    pul: float = float("inf")
    pll: float = float("-inf")
    seed: int = 12345
    use_exit: bool = False
    rng_mode: int = 0

    def c(self) -> PropParams:
        return PropParams(self.step, self.Tsurf, self.Tproj, self.pile_tau, self.andersen_time, self.gamma_const,
                          self.pul, self.pll, self.seed & 0xFFFFFFFFFFFFFFFF, int(self.use_exit), int(self.rng_mode))


def _p(a, ctype):
    return a.ctypes.data_as(ct.POINTER(ctype))


class Engine:
    """A batch of trajectories on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ct.c_void_p()
        rc = self.lib.mdt_create(device, ct.byref(h))
        if rc != 0:
            raise EngineError(f"mdt_create failed ({rc}): no usable CUDA device {device}")
        self.h = h
        self.T = 0
        self.universes: list[Universe] = []

    # -- errors ----------------------------------------------------------------
    def _check(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = self.lib.mdt_last_error(self.h)
            raise EngineError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.mdt_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order varies
        try:
            self.close()
        except Exception:
            pass

    # -- set-up ----------------------------------------------------------------
    def read_emt(self, params: EmtParams) -> None:
        """read_emt (src/pes_emt_mod.f90:49-190) equivalent: install EMT parameters."""
        arrs = params.arrays()
        pes = np.ascontiguousarray(params.pes.T, dtype=np.int32)  # column major (ntypes, ntypes)
        self._check(self.lib.mdt_emt_set_params(self.h, params.ntypes, *[_p(a, ct.c_double) for a in arrs],
                                                _p(pes, ct.c_int32)), "mdt_emt_set_params")
        self._keep_params = (arrs, pes)

    def read_nene(self, model, type_names: list, max_neighbors: int = 0) -> None:
        """read_nene (src/pes_nene_mod.f90:123) equivalent: install an HDNNP
        (``nene.NNModel``).  ``type_names``: element symbol of each universe type."""
        from .nene import Z_OF
        f = model.flat()
        keep = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in f.items()}
        c = NNModelC()
        c.nelem, c.maxsf = model.nelem, model.maxsf
        for name in ("z", "nsf", "sftype", "eta", "rshift", "zeta", "rc", "e1", "e2", "smin", "smax", "savg",
                     "nodes", "act", "weights", "atom_energy"):
            setattr(c, name, keep[name].ctypes.data)
        c.lambda_ = keep["lambda"].ctypes.data
        c.scalesym, c.centersym = int(model.scalesym), int(model.centersym)
        c.scmin, c.scmax = model.scmin, model.scmax
        c.cutoff_type, c.cutoff_alpha = model.cutoff_type, model.cutoff_alpha
        c.nlayers, c.maxnodes, c.maxweights = keep["nlayers"], keep["maxnodes"], keep["maxweights"]
        c.normnodes = int(model.normnodes)
        c.remove_atom_energies = int(bool(model.atom_energy))
        zt = np.array([Z_OF.get(n, 0) if n in model.elements else 0 for n in type_names], np.int32)
        self._check(self.lib.mdt_nn_set_model(self.h, ct.byref(c), len(type_names), _p(zt, ct.c_int32),
                                              max_neighbors), "mdt_nn_set_model")
        self.nn_model = model
        self.max_neighbors = max_neighbors or 192

    def set_pes(self, kind: int, range_margin: float = 0.1) -> None:
        self._check(self.lib.mdt_set_pes(self.h, kind, range_margin), "mdt_set_pes")

    def nn_fast_path(self, enable: bool = True) -> bool:
        """Allow (default) or forbid the FP32 fast kernels; True if the model qualifies."""
        r = self.lib.mdt_nn_fast_path(self.h, 1 if enable else 0)
        if r < 0:
            self._check(r, "mdt_nn_fast_path")
        return bool(r)

    def nn_radial_kernel(self, enable: bool = True) -> bool:
        """Allow (default) or forbid the thread-per-atom kernel of radial-only models;
        True if the installed model qualifies."""
        r = self.lib.mdt_nn_radial_kernel(self.h, 1 if enable else 0)
        if r < 0:
            self._check(r, "mdt_nn_radial_kernel")
        return bool(r)

    def nn_radial_block(self, max_block: int = 512) -> None:
        """Largest CTA (atoms per pack) the thread-per-atom kernel's plan may use."""
        self._check(self.lib.mdt_nn_radial_block(self.h, max_block), "mdt_nn_radial_block")

    def nn_set_skin(self, skin_ang: float) -> None:
        """Verlet skin (A) of the fast kernels' neighbour lists; 0 rebuilds every step."""
        self._check(self.lib.mdt_nn_set_skin(self.h, skin_ang), "mdt_nn_set_skin")

    def autotune(self, sp: SimParams, precision: str = "fp32", nsteps: int = 20) -> dict:
        """Pick the thread-per-atom kernel's CTA size and skin by timing candidate launches
        (mdt_autotune); the batch's state is restored afterwards."""
        b = ct.c_int32(0)
        sk = ct.c_double(0.0)
        ms = ct.c_double(0.0)
        p = sp.c()
        self._check(self.lib.mdt_autotune(self.h, PREC[precision], nsteps, ct.byref(p), ct.byref(b), ct.byref(sk),
                                          ct.byref(ms)), "mdt_autotune")
        return {"block": int(b.value), "skin_A": float(sk.value), "ms_per_step": float(ms.value)}

    def nn_repack(self) -> int:
        """Re-pack the thread-per-atom kernel's CTAs over the trajectories still running;
        returns the number of packs (0: the batch does not run on that kernel)."""
        n = ct.c_int32(0)
        self._check(self.lib.mdt_nn_repack(self.h, ct.byref(n)), "mdt_nn_repack")
        return int(n.value)

    def nn_stats(self):
        fb = np.zeros(self.T, np.int32)
        ov = np.zeros(self.T, np.int32)
        self._check(self.lib.mdt_nn_stats(self.h, fb.ctypes.data, ov.ctypes.data), "mdt_nn_stats")
        return fb, ov

    def nn_descriptors(self, precision: str = "fp64") -> np.ndarray:
        """Raw symmetry functions, shape (nslots, maxsf), Fortran slot order."""
        G = np.zeros((self.nslots, self.nn_model.maxsf))
        self._check(self.lib.mdt_nn_descriptors(self.h, PREC[precision], G.ctypes.data), "mdt_nn_descriptors")
        return G

    def nn_neighbors(self):
        tot = int(np.sum(self.natoms))
        counts = np.zeros(tot, np.int32)
        words = np.zeros(tot * self.max_neighbors, np.int32)
        self._check(self.lib.mdt_nn_neighbors(self.h, counts.ctypes.data, words.ctypes.data), "mdt_nn_neighbors")
        return counts, words.reshape(tot, self.max_neighbors)

    def define(self, universes: list[Universe]) -> None:
        """Lay out T universes (ragged sizes and bead counts) on the device."""
        if not universes:
            raise ValueError("empty batch")
        u0 = universes[0]
        for u in universes:
            if u.ntypes != u0.ntypes or list(u.names) != list(u0.names):
                raise ValueError("all trajectories of a batch share one type table")
        self.universes = list(universes)
        self.T = len(universes)
        natoms = np.array([u.natoms for u in universes], np.int32)
        nbeads = np.array([u.nbeads for u in universes], np.int32)
        idx = np.concatenate([np.asarray(u.idx, np.int32) for u in universes])
        mass = np.concatenate([np.asarray(u.m, np.float64) for u in universes])
        fixed = np.concatenate([np.asarray(u.is_fixed, np.uint8).reshape(-1) for u in universes])
        box = np.concatenate([np.asarray(u.simbox, np.float64).T.reshape(-1) for u in universes])  # column major
        algo = np.ascontiguousarray(u0.algo, np.int32)
        is_proj = np.ascontiguousarray(u0.is_proj, np.uint8)
        self._check(self.lib.mdt_batch_define(self.h, self.T, _p(natoms, ct.c_int32), _p(nbeads, ct.c_int32),
                                              _p(idx, ct.c_int32), _p(mass, ct.c_double), _p(fixed, ct.c_uint8),
                                              _p(box, ct.c_double), u0.ntypes, _p(algo, ct.c_int32),
                                              _p(is_proj, ct.c_uint8)), "mdt_batch_define")
        self.natoms, self.nbeads = natoms, nbeads
        self.nslots = int(np.sum(natoms.astype(np.int64) * nbeads))
        self.ba_off = np.concatenate([[0], np.cumsum(natoms.astype(np.int64) * nbeads)])
        self.bead_off = np.concatenate([[0], np.cumsum(nbeads)])

    def upload(self, r: np.ndarray | None = None, v: np.ndarray | None = None) -> None:
        """Positions/velocities of all trajectories, Fortran order, concatenated.
        Defaults to the universes given to :meth:`define`."""
        if r is None:
            r = np.concatenate([u.r.reshape(-1) for u in self.universes])
        if v is None:
            v = np.concatenate([u.v.reshape(-1) for u in self.universes])
        r = np.ascontiguousarray(r, np.float64).reshape(-1)
        v = np.ascontiguousarray(v, np.float64).reshape(-1)
        if r.size != 3 * self.nslots or v.size != 3 * self.nslots:
            raise ValueError("state arrays do not match the batch layout")
        self._check(self.lib.mdt_state_upload(self.h, r.ctypes.data, v.ctypes.data), "mdt_state_upload")

    def upload_ptr(self, r_ptr: int, v_ptr: int) -> None:
        """Upload from raw host pointers (e.g. pinned buffers)."""
        self._check(self.lib.mdt_state_upload(self.h, r_ptr, v_ptr), "mdt_state_upload")

    def set_random_arrays(self, randy=None, zeta=None, andersen_v=None, andersen_u=None) -> None:
        keep = [None if a is None else np.ascontiguousarray(a, np.float64).reshape(-1)
                for a in (randy, zeta, andersen_v, andersen_u)]
        ptrs = [None if a is None else a.ctypes.data for a in keep]
        self._check(self.lib.mdt_set_random_arrays(self.h, *ptrs), "mdt_set_random_arrays")

    # -- hot path ----------------------------------------------------------------
    def calc_force(self, sp: SimParams, flag: int = C.ENERGY_AND_FORCE, precision: str = "fp64") -> None:
        p = sp.c()
        self._check(self.lib.mdt_calc_force(self.h, flag, PREC[precision], ct.byref(p)), "mdt_calc_force")

    def propagate_1(self, sp: SimParams) -> None:
        p = sp.c()
        self._check(self.lib.mdt_propagate_1(self.h, ct.byref(p)), "mdt_propagate_1")

    def propagate_2(self, sp: SimParams) -> None:
        p = sp.c()
        self._check(self.lib.mdt_propagate_2(self.h, ct.byref(p)), "mdt_propagate_2")

    def md_steps(self, nsteps: int, sp: SimParams, precision: str = "fp64") -> None:
        p = sp.c()
        self._check(self.lib.mdt_md_steps(self.h, nsteps, PREC[precision], ct.byref(p)), "mdt_md_steps")

    def synchronize(self) -> None:
        self._check(self.lib.mdt_synchronize(self.h), "mdt_synchronize")

    # -- results -----------------------------------------------------------------
    def download(self):
        """Returns dict of r, v, f, a (3*nslots, Fortran order), epot (total beads), dens."""
        out = {k: np.empty(3 * self.nslots) for k in ("r", "v", "f", "a")}
        out["epot"] = np.empty(int(self.bead_off[-1]))
        out["dens"] = np.empty(self.nslots)
        self._check(self.lib.mdt_state_download(self.h, *[out[k].ctypes.data for k in
                                                         ("r", "v", "f", "a", "epot", "dens")]),
                    "mdt_state_download")
        return out

    def split(self, flat: np.ndarray, t: int, per: int = 3) -> np.ndarray:
        """Slice trajectory t out of a flat Fortran-order array -> (N, nb, per)."""
        a, b = self.ba_off[t], self.ba_off[t + 1]
        x = flat[per * a: per * b]
        return x.reshape(self.natoms[t], self.nbeads[t], per) if per > 1 else x.reshape(self.natoms[t], self.nbeads[t])

    def query(self, sp: SimParams) -> np.ndarray:
        arr = (TrajSummary * self.T)()
        p = sp.c()
        self._check(self.lib.mdt_query(self.h, ct.byref(p), arr), "mdt_query")
        return np.array([(s.status, s.steps_done, s.epot, s.ekin_p, s.ekin_l, s.ebead) for s in arr],
                        dtype=[("status", "i4"), ("steps_done", "i4"), ("epot", "f8"), ("ekin_p", "f8"),
                               ("ekin_l", "f8"), ("ebead", "f8")])

    def observables(self) -> dict:
        """Per-trajectory observables of the fused MD steps (trajectory_info.f90): turning
        points, closest approach (A) and its step, lowest projectile position (T, 3)."""
        turn = np.zeros(self.T, np.int32)
        cl = np.zeros(self.T)
        clstep = np.zeros(self.T, np.int32)
        low = np.zeros((self.T, 3))
        self._check(self.lib.mdt_traj_observables(self.h, turn.ctypes.data, cl.ctypes.data, clstep.ctypes.data,
                                                  low.ctypes.data), "mdt_traj_observables")
        return {"turn_pnts": turn, "cl_appr": cl, "cl_appr_step": clstep, "r_min_p": low}

    def bounces(self, sp: SimParams) -> dict:
        """Bounce count, interaction time (fs) and adsorption flag per trajectory
        (trajectory_info.f90's check_for_bounce, check_for_proj_surf_interaction and
        adsorption hysteresis, tracked by the fused MD steps)."""
        b = np.zeros(self.T, np.int32)
        ti = np.zeros(self.T)
        ads = np.zeros(self.T, np.int32)
        p = sp.c()
        self._check(self.lib.mdt_traj_bounces(self.h, b.ctypes.data, ti.ctypes.data, ads.ctypes.data, ct.byref(p)),
                    "mdt_traj_bounces")
        return {"bounces": b, "interaction_time": ti, "is_adsorbed": ads.astype(bool)}

    def set_adsorption(self, start: float, end: float) -> None:
        """Adsorption limits (A): adsorbed below start, free again above end."""
        self._check(self.lib.mdt_set_adsorption(self.h, float(start), float(end)), "mdt_set_adsorption")

    def set_step_limit(self, max_steps: int) -> None:
        """Stop each trajectory after max_steps steps (status 3); 0 = no limit."""
        self._check(self.lib.mdt_set_step_limit(self.h, int(max_steps)), "mdt_set_step_limit")

    def refill(self, z0: float = 6.0, einc=(0.5, 5.0), polar=(0.0, 60.0), azimuth: float = -1.0,
               seed: int = 1):
        """Restart every stopped trajectory from the uploaded state with a new projectile
        start (mdt_refill); returns (generation per trajectory, number refilled)."""
        from ._lib import RefillParams
        p = RefillParams(z0, einc[0], einc[1], polar[0], polar[1], azimuth, seed & 0xFFFFFFFFFFFFFFFF)
        gen = np.zeros(self.T, np.int32)
        n = ct.c_int32(0)
        self._check(self.lib.mdt_refill(self.h, ct.byref(p), gen.ctypes.data, ct.byref(n)), "mdt_refill")
        return gen, int(n.value)

    def refill_draws(self) -> np.ndarray:
        """(T, 5): u, v, einc (eV), polar, azimuth (deg) the last refill drew; NaN rows for
        trajectories it did not restart."""
        d = np.zeros((self.T, 5))
        self._check(self.lib.mdt_refill_draws(self.h, d.ctypes.data), "mdt_refill_draws")
        return d

    def launch_count(self) -> int:
        return int(self.lib.mdt_launch_count(self.h))
