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
SOURCES = ["md_oracle.cpp"]

ORC_VERLET, ORC_LANGEVIN, ORC_ANDERSEN, ORC_PILE, ORC_LANGEVIN_CONST = 1001, 1003, 1005, 1006, 1007


def build(force: bool = False) -> Path:
    srcs = [HERE / s for s in SOURCES] + [HERE / "md_oracle.h"]
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(s.stat().st_mtime for s in srcs):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".tmp.so")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", str(tmp)] + [str(HERE / s) for s in SOURCES]
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
        _lib.orc_remove_com_velocity.argtypes = [P(CUniverse)]
    return _lib


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

    def bead_epot(self, sp):
        p = self.params(sp)
        return lib().orc_bead_epot(ct.byref(self.c), ct.byref(p))
