"""Shared helpers for the parity tests: run the oracle trajectory by trajectory and
compare against the engine's flat Fortran-order outputs."""
from __future__ import annotations

import numpy as np

from md_tian2_gb300.engine import Engine, SimParams
from oracle.oracle import OracleUniverse


def make_engine(universes, emt):
    eng = Engine(0)
    eng.read_emt(emt)
    eng.define(universes)
    eng.upload()
    return eng


def oracle_list(universes, emt):
    return [OracleUniverse(u, emt) for u in universes]


def flat(arrs):
    return np.concatenate([np.asarray(a).reshape(-1) for a in arrs])


def max_abs(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b))) if a.size else 0.0


def injected(universes, rng):
    """Per-trajectory deviates in the reference's Fortran order."""
    n3 = [u.natoms * u.nbeads * 3 for u in universes]
    n1 = [u.natoms * u.nbeads for u in universes]
    randy = [rng.normal(size=n) for n in n3]
    zeta = [rng.normal(size=n) for n in n3]
    av = [rng.normal(size=n) for n in n3]
    au = [rng.random(size=n) for n in n1]
    return randy, zeta, av, au
