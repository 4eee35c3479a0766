"""ctypes wrapper of the CPU FP64 oracle (md_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, always as the checker.  The product (md_tian2_gb300) never
imports it.  Parity of the oracle itself is unpinned by a reference run (no Fortran
compiler exists here); see md_oracle.h for what pins it.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "build"
LIB = BUILD / "libmd_oracle.so"
SOURCES = ["md_oracle.cpp", "nene_oracle.cpp"]

ORC_VERLET, ORC_LANGEVIN, ORC_ANDERSEN, ORC_PILE, ORC_LANGEVIN_CONST = 1001, 1003, 1005, 1006, 1007


def build(force: bool = False) -> Path:
    srcs = [HERE / s for s in SOURCES] + [HERE / "md_oracle.h"]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(s.stat().st_mtime for s in srcs):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".tmp.so")
    # -O3 without -ffast-math keeps IEEE semantics in source order (the checker's values do
    # not depend on it); no -march=native: the same flags build the same results on the x86
    # build machine and the Arm GPU hosts
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", str(tmp)] + [str(HERE / s) for s in SOURCES]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


class Params(ct.Structure):
    _fields_ = [("step", ct.c_double), ("Tsurf", ct.c_double), ("Tproj", ct.c_double), ("pile_tau", ct.c_double),
                ("andersen_time", ct.c_double), ("gamma_const", ct.c_double)]


class CUniverse(ct.Structure):
    _fields_ = [("natoms", ct.c_int), ("nbeads", ct.c_int), ("ntypes", ct.c_int),
                ("r", ct.POINTER(ct.c_double)), ("v", ct.POINTER(ct.c_double)), ("f", ct.POINTER(ct.c_double)),
                ("a", ct.POINTER(ct.c_double)), ("m", ct.POINTER(ct.c_double)),
                ("is_fixed", ct.POINTER(ct.c_uint8)), ("idx", ct.POINTER(ct.c_int32)),
                ("pes", ct.POINTER(ct.c_int32)), ("algo", ct.POINTER(ct.c_int32)),
                ("is_proj", ct.POINTER(ct.c_uint8)), ("epot", ct.POINTER(ct.c_double)),
                ("simbox", ct.c_double * 9), ("isimbox", ct.c_double * 9),
                ("dens", ct.POINTER(ct.c_double)), ("emt", ct.POINTER(ct.c_double))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ct.CDLL(str(build()))
        P = ct.POINTER
        _lib.orc_calc_force.argtypes = [P(CUniverse), P(Params)]
        _lib.orc_propagate_1.argtypes = [P(CUniverse), P(Params)] + [ct.c_void_p] * 4
        _lib.orc_propagate_2.argtypes = [P(CUniverse), P(Params), ct.c_void_p]
        _lib.orc_md_step.argtypes = [P(CUniverse), P(Params)] + [ct.c_void_p] * 4
        _lib.orc_run_verlet.argtypes = [P(CUniverse), P(Params), ct.c_int, ct.c_double]
        _lib.orc_ring_polymer_step.argtypes = [P(CUniverse), P(Params)]
        _lib.orc_bead_epot.argtypes = [P(CUniverse), P(Params)]
        _lib.orc_bead_epot.restype = ct.c_double
        _lib.orc_atom_ekin.argtypes = [P(CUniverse), P(ct.c_double), P(ct.c_double)]
        _lib.orc_bead_ekin.argtypes = [P(CUniverse), P(ct.c_double), P(ct.c_double)]
        _lib.orc_remove_com_velocity.argtypes = [P(CUniverse)]
        _lib.orc_run_steps.argtypes = [ct.c_void_p, ct.c_int, P(Params), ct.c_double, ct.c_int64, ct.c_uint64,
                                       P(ct.c_double)]
        _lib.orc_run_steps.restype = ct.c_int64
    return _lib


def run_steps(orcs, sp, seconds: float, max_sweeps: int = 1 << 40, seed: int = 1):
    """Steady-state MD stepping of OracleUniverse objects inside C (orc_run_steps) for
    ``seconds`` of wall time; returns (atom-steps, elapsed seconds)."""
    arr = (ct.POINTER(CUniverse) * len(orcs))(*[ct.pointer(o.c) for o in orcs])
    p = OracleUniverse.params(sp)
    el = ct.c_double()
    n = lib().orc_run_steps(ct.cast(arr, ct.c_void_p), len(orcs), ct.byref(p), seconds, max_sweeps,
                            seed & 0xFFFFFFFFFFFFFFFF, ct.byref(el))
    if n < 0:
        raise RuntimeError("orc_run_steps failed")
    return int(n), el.value


class OracleUniverse:
    """Owns numpy buffers in the reference's Fortran order and a C view of them."""

    def __init__(self, u, emt):
        """``u``: md_tian2_gb300.universe.Universe; ``emt``: io.EmtParams."""
        self.N, self.nb, self.nt = u.natoms, u.nbeads, u.ntypes
        self.r = np.ascontiguousarray(u.r, np.float64).copy()
        self.v = np.ascontiguousarray(u.v, np.float64).copy()
        self.f = np.zeros_like(self.r)
        self.a = np.zeros_like(self.r)
        self.m = np.ascontiguousarray(u.m, np.float64).copy()
        self.fixed = np.ascontiguousarray(u.is_fixed, np.uint8).copy()
        self.idx = np.ascontiguousarray(u.idx, np.int32).copy()
        self.pes = np.ascontiguousarray(emt.pes.T, np.int32).copy()  # column major
        self.algo = np.ascontiguousarray(u.algo, np.int32).copy()
        self.is_proj = np.ascontiguousarray(u.is_proj, np.uint8).copy()
        self.epot = np.zeros(self.nb)
        self.dens = np.zeros((self.N, self.nb))
        self.emt = np.ascontiguousarray(np.stack(emt.arrays(), axis=1), np.float64).copy()  # (ntypes, 7)
        from md_tian2_gb300.universe import invert_matrix  # pure numpy helper
        self.simbox = np.asarray(u.simbox, np.float64)
        self.isimbox = invert_matrix(self.simbox)
        self.c = CUniverse()
        P = lambda a, t: a.ctypes.data_as(ct.POINTER(t))  # noqa: E731
        self.c.natoms, self.c.nbeads, self.c.ntypes = self.N, self.nb, self.nt
        self.c.r, self.c.v, self.c.f, self.c.a = (P(x, ct.c_double) for x in (self.r, self.v, self.f, self.a))
        self.c.m = P(self.m, ct.c_double)
        self.c.is_fixed = P(self.fixed, ct.c_uint8)
        self.c.idx = P(self.idx, ct.c_int32)
        self.c.pes = P(self.pes, ct.c_int32)
        self.c.algo = P(self.algo, ct.c_int32)
        self.c.is_proj = P(self.is_proj, ct.c_uint8)
        self.c.epot = P(self.epot, ct.c_double)
        self.c.dens = P(self.dens, ct.c_double)
        self.c.emt = P(self.emt, ct.c_double)
        for k in range(9):
            self.c.simbox[k] = self.simbox.T.reshape(-1)[k]
            self.c.isimbox[k] = self.isimbox.T.reshape(-1)[k]

    @staticmethod
    def params(sp) -> Params:
        return Params(sp.step, sp.Tsurf, sp.Tproj, sp.pile_tau, sp.andersen_time, sp.gamma_const)

    def calc_force(self, sp):
        p = self.params(sp)
        rc = lib().orc_calc_force(ct.byref(self.c), ct.byref(p))
        if rc:
            raise RuntimeError(f"orc_calc_force {rc}")

    def propagate_1(self, sp, randy=None, zeta=None, andersen_v=None, andersen_u=None):
        p = self.params(sp)
        keep = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (randy, zeta, andersen_v, andersen_u)]
        rc = lib().orc_propagate_1(ct.byref(self.c), ct.byref(p), *[None if a is None else a.ctypes.data for a in keep])
        if rc:
            raise RuntimeError(f"orc_propagate_1 {rc}")

    def propagate_2(self, sp, randy=None):
        p = self.params(sp)
        keep = None if randy is None else np.ascontiguousarray(randy, np.float64)
        rc = lib().orc_propagate_2(ct.byref(self.c), ct.byref(p), None if keep is None else keep.ctypes.data)
        if rc:
            raise RuntimeError(f"orc_propagate_2 {rc}")

    def run_verlet(self, sp, nsteps, pul):
        p = self.params(sp)
        return lib().orc_run_verlet(ct.byref(self.c), ct.byref(p), nsteps, pul)

    def atom_ekin(self):
        ep, el = ct.c_double(), ct.c_double()
        lib().orc_atom_ekin(ct.byref(self.c), ct.byref(ep), ct.byref(el))
        return ep.value, el.value

    def bead_ekin(self):
        ep, el = ct.c_double(), ct.c_double()
        lib().orc_bead_ekin(ct.byref(self.c), ct.byref(ep), ct.byref(el))
        return ep.value, el.value

    def bead_epot(self, sp):
        p = self.params(sp)
        return lib().orc_bead_epot(ct.byref(self.c), ct.byref(p))


# ---------------------------------------------------------------------------
# RuNNer HDNNP oracle (nene_oracle.cpp)
# ---------------------------------------------------------------------------
class CNN(ct.Structure):
    _fields_ = [("nelem", ct.c_int), ("z", ct.c_void_p), ("maxsf", ct.c_int), ("nsf", ct.c_void_p),
                ("sftype", ct.c_void_p), ("eta", ct.c_void_p), ("rshift", ct.c_void_p), ("lambda_", ct.c_void_p),
                ("zeta", ct.c_void_p), ("rc", ct.c_void_p), ("e1", ct.c_void_p), ("e2", ct.c_void_p),
                ("smin", ct.c_void_p), ("smax", ct.c_void_p), ("savg", ct.c_void_p),
                ("scalesym", ct.c_int), ("centersym", ct.c_int), ("scmin", ct.c_double), ("scmax", ct.c_double),
                ("cutoff_type", ct.c_int), ("cutoff_alpha", ct.c_double), ("nlayers", ct.c_int),
                ("maxnodes", ct.c_int), ("nodes", ct.c_void_p), ("act", ct.c_void_p), ("maxweights", ct.c_int),
                ("weights", ct.c_void_p), ("normnodes", ct.c_int), ("remove_atom_energies", ct.c_int),
                ("atom_energy", ct.c_void_p)]


class NNOracle:
    """compute_nene on the CPU for one bead (positions in A, cell columns in A)."""

    def __init__(self, model):
        f = model.flat()
        self.keep = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in f.items()}
        k = self.keep
        self.model = model
        self.c = CNN()
        c = self.c
        c.nelem, c.maxsf = model.nelem, model.maxsf
        for name in ("z", "nsf", "sftype", "eta", "rshift", "zeta", "rc", "e1", "e2", "smin", "smax", "savg",
                     "nodes", "act", "weights", "atom_energy"):
            setattr(c, name, k[name].ctypes.data)
        c.lambda_ = k["lambda"].ctypes.data
        c.scalesym, c.centersym = int(model.scalesym), int(model.centersym)
        c.scmin, c.scmax = model.scmin, model.scmax
        c.cutoff_type, c.cutoff_alpha = model.cutoff_type, model.cutoff_alpha
        c.nlayers, c.maxnodes, c.maxweights = k["nlayers"], k["maxnodes"], k["maxweights"]
        c.normnodes = int(model.normnodes)
        c.remove_atom_energies = int(bool(model.atom_energy))
        L = lib()
        L.orc_nene_energy_force.argtypes = [ct.POINTER(CNN), ct.c_int] + [ct.c_void_p] * 7
        L.orc_nene_neighbors.argtypes = [ct.c_int, ct.c_void_p, ct.c_void_p, ct.c_int, ct.c_double] + \
            [ct.c_void_p] * 4 + [ct.c_int]

    def energy_force(self, elem, r_ang, simbox, want_G=False):
        """elem: 0-based element index per atom; r_ang (N,3); simbox (3,3) columns."""
        N = len(elem)
        e = np.ascontiguousarray(elem, np.int32)
        r = np.ascontiguousarray(r_ang, np.float64).reshape(N, 3)
        box = np.ascontiguousarray(np.asarray(simbox, np.float64).T)  # column major
        f = np.zeros((N, 3))
        en = ct.c_double()
        G = np.zeros((N, self.model.maxsf)) if want_G else None
        ea = np.zeros(N)
        rc = lib().orc_nene_energy_force(ct.byref(self.c), N, e.ctypes.data, r.ctypes.data, box.ctypes.data,
                                         ct.addressof(en), f.ctypes.data, None if G is None else G.ctypes.data,
                                         ea.ctypes.data)
        if rc:
            raise RuntimeError(f"orc_nene_energy_force {rc}")
        return (en.value, f, G, ea) if want_G else (en.value, f)

    @staticmethod
    def neighbors(r_bohr, lat_rows_bohr, cutoff, periodic=True, max_total=2_000_000):
        N = len(r_bohr)
        xyz = np.ascontiguousarray(r_bohr, np.float64)
        lat = np.ascontiguousarray(lat_rows_bohr, np.float64)
        counts = np.zeros(N, np.int32)
        oj = np.zeros(max_total, np.int32)
        on = np.zeros(3 * max_total, np.int32)
        orr = np.zeros(max_total)
        tot = lib().orc_nene_neighbors(N, xyz.ctypes.data, lat.ctypes.data, int(periodic), cutoff,
                                       counts.ctypes.data, oj.ctypes.data, on.ctypes.data, orr.ctypes.data,
                                       max_total)
        if tot < 0:
            raise RuntimeError("neighbour list larger than max_total")
        return counts, oj[:tot], on[:3 * tot].reshape(-1, 3), orr[:tot]
