"""Seeded synthetic workloads with the shapes of the engine's benchmark configurations.

The reference ships pre-thermalised slab libraries and reads them with ``conf merge``
(src/md_init.f90:559-625, 829-877); these generators build equivalent inputs from a
seed instead:

* fcc(111) slabs with hexagonal in-plane cells a1 = (k d, 0, 0),
  a2 = (k d / 2, k d sqrt(3)/2, 0), d = a / sqrt(2), ABC stacking, layer spacing
  a / sqrt(3), 4 layers, bottom 2 frozen, c = 3 a / sqrt(3) + 15 A of vacuum;
* Maxwell-Boltzmann velocities at Tsurf for mobile slab atoms, centre-of-mass removed;
* one H projectile at z = 6 A above the top layer (z = 0), uniform in x, y, with the
  incidence velocity of set_proj_incidence (md_init.f90:861-871, v_z = -v cos(polar)).
The projectile is atom 1, as merge_universes makes it.
"""
from __future__ import annotations

import math

import numpy as np

from . import constants as C
from .io import EMT_KEYS, EmtParams
from .universe import Universe

# EMT parameter sets of the reference's pes/EMT-HAu.pes and pes/EMT-HPt.pes
# (eta2, n0, E0, lambda, V0, kappa, s0), so that the GPU machine needs no reference files.
EMT_TABLE = {
    ("H", "Au"): {
        "H": (5.06612337, 0.13115359, -1.76738026, 8.00198330, 0.21350000, 8.97429324, 0.71031644),
        "Au": (3.16340000, 0.04858000, -3.80000000, 4.12338000, 2.32100000, 5.42918000, 1.64174000),
    },
    ("H", "Pt"): {
        "H": (4.92557652, 0.12090900, -2.11450646, 7.01217816, 0.21350000, 8.85208951, 0.64979500),
        "Pt": (3.37380459, 0.06062800, -5.85000000, 4.19626000, 21.67781225, 6.05575253, 1.57466581),
    },
}
LATTICE_A = {"Au": 4.078, "Pt": 3.92}


def emt_params(proj: str = "H", metal: str = "Au", with_proj: bool = True) -> EmtParams:
    """EMT parameters for the type table [proj, metal] (or [metal] alone)."""
    table = EMT_TABLE[(proj, metal)]
    names = [proj, metal] if with_proj else [metal]
    p = EmtParams(ntypes=len(names), values={k: np.zeros(len(names)) for k in EMT_KEYS},
                  pes=np.full((len(names), len(names)), C.PES_ID_EMT, np.int32))
    for t, n in enumerate(names):
        for k, val in zip(EMT_KEYS, table[n]):
            p.values[k][t] = val
    return p


def fcc111_slab(a: float, k: int, layers: int = 4, nfixed: int = 2, vacuum: float = 15.0):
    """Positions (n, 3), cell (3, 3) with cell vectors as columns, fixed flags (n,)."""
    d = a / math.sqrt(2.0)
    dz = a / math.sqrt(3.0)
    a1 = np.array([d, 0.0, 0.0])
    a2 = np.array([d / 2, d * math.sqrt(3.0) / 2, 0.0])
    shift = (a1 + a2) / 3.0  # ABC stacking offset between consecutive layers
    pos, fixed = [], []
    for l in range(layers):
        for i in range(k):
            for j in range(k):
                p = i * a1 + j * a2 + (l % 3) * shift
                p[2] = -l * dz
                pos.append(p)
                fixed.append(l >= layers - nfixed)
    cell = np.zeros((3, 3))
    cell[:, 0] = k * a1
    cell[:, 1] = k * a2
    cell[:, 2] = [0.0, 0.0, (layers - 1) * dz + vacuum]
    return np.array(pos), cell, np.array(fixed, bool)


def maxwell_boltzmann(rng, masses, mobile, T):
    v = np.zeros((len(masses), 3))
    sd = np.sqrt(C.KB * T / masses[mobile])
    v[mobile] = rng.normal(size=(int(mobile.sum()), 3)) * sd[:, None]
    if mobile.sum() > 0:
        m = masses[mobile][:, None]
        v[mobile] -= (m * v[mobile]).sum(0) / m.sum()
    return v


def h_on_metal(rng, metal: str, k: int, einc: float, polar_deg: float, azimuth_deg: float, Tsurf: float,
               algo_proj=C.PROP_ID_VERLET, algo_latt=C.PROP_ID_VERLET, z0: float = 6.0, nbeads: int = 1) -> Universe:
    """One H/metal(111) trajectory start (projectile first)."""
    pos, cell, fx = fcc111_slab(LATTICE_A[metal], k)
    n = len(pos) + 1
    masses = np.empty(n)
    masses[0] = C.MASS_AMU["H"] * C.AMU2MASS
    masses[1:] = C.MASS_AMU[metal] * C.AMU2MASS
    r = np.zeros((n, 3))
    frac = rng.random(2)
    r[0, :2] = frac[0] * cell[:2, 0] + frac[1] * cell[:2, 1]
    r[0, 2] = z0
    r[1:] = pos
    fixed = np.zeros((n, 3), bool)
    fixed[1:] = fx[:, None]
    v = np.zeros((n, 3))
    v[1:] = maxwell_boltzmann(rng, masses[1:], ~fx, Tsurf)
    vinc = math.sqrt(2.0 * einc / masses[0])
    pol, az = polar_deg * C.DEG2RAD, azimuth_deg * C.DEG2RAD
    v[0] = [vinc * math.sin(pol) * math.cos(az), vinc * math.sin(pol) * math.sin(az), -vinc * math.cos(pol)]
    u = Universe(r=r[:, None, :].copy(), v=v[:, None, :].copy(), m=masses, idx=np.array([1] + [2] * (n - 1), np.int32),
                 is_fixed=fixed[:, None, :].copy(), simbox=cell, names=["H", metal],
                 is_proj=np.array([True, False]), algo=np.array([algo_proj, algo_latt], np.int32))
    return u.force_beads(nbeads) if nbeads > 1 else u


def config1(ntraj: int = 100, seed: int = 1):
    """Plain EMT H/Au(111) 3x3, Einc 2.76 eV, polar 45, azimuth 0, Verlet."""
    rng = np.random.default_rng(seed)
    return [h_on_metal(rng, "Au", 3, 2.76, 45.0, 0.0, 300.0) for _ in range(ntraj)]


def config2(ntraj: int = 4096, seed: int = 2, lattice_algo=C.PROP_ID_LANGEVIN_CONST):
    """Ragged batch: slabs k in {3,4,5,6}, Einc ~ U(0.5,5) eV, polar ~ U(0,60), azimuth
    ~ U(0,360), Langevin (constant friction) on Au, Verlet on H."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ntraj):
        k = int(rng.integers(3, 7))
        out.append(h_on_metal(rng, "Au", k, rng.uniform(0.5, 5.0), rng.uniform(0.0, 60.0), rng.uniform(0.0, 360.0),
                              300.0, C.PROP_ID_VERLET, lattice_algo))
    return out


def config3(ntraj: int = 1024, seed: int = 3, beads=(4, 8, 16, 32)):
    """RPMD H/Pt(111) 4x4, nbeads mixed per trajectory, PILE, normal incidence."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(ntraj):
        nb = int(rng.choice(beads))
        out.append(h_on_metal(rng, "Pt", 4, rng.uniform(0.1, 1.0), 0.0, 0.0, 300.0, C.PROP_ID_PILE, C.PROP_ID_PILE,
                              nbeads=nb))
    return out


# ---------------------------------------------------------------------------
# H on graphene (HDNNP workload)
# ---------------------------------------------------------------------------
def graphene(k: int = 6, a: float = 2.46, c: float = 20.0, ripple: float = 0.05, rng=None):
    """k x k hexagonal graphene supercell (2 atoms per primitive cell) at z = 0 with a
    Gaussian z-ripple; returns positions (n, 3) and cell (columns)."""
    rng = rng or np.random.default_rng(0)
    a1 = np.array([a, 0.0, 0.0])
    a2 = np.array([a / 2, a * math.sqrt(3.0) / 2, 0.0])
    pos = []
    for i in range(k):
        for j in range(k):
            o = i * a1 + j * a2
            pos.append(o)
            pos.append(o + (a1 + a2) / 3.0)
    pos = np.array(pos)
    pos[:, 2] = rng.normal(scale=ripple, size=len(pos))
    cell = np.zeros((3, 3))
    cell[:, 0] = k * a1
    cell[:, 1] = k * a2
    cell[:, 2] = [0.0, 0.0, c]
    return pos, cell


def h_on_graphene(rng, einc: float, Tsurf: float = 300.0, z0: float = 4.0, k: int = 6, algo=C.PROP_ID_VERLET):
    """One H/graphene trajectory start: H first (projectile), normal incidence."""
    pos, cell = graphene(k, rng=rng)
    n = len(pos) + 1
    masses = np.empty(n)
    masses[0] = C.MASS_AMU["H"] * C.AMU2MASS
    masses[1:] = C.MASS_AMU["C"] * C.AMU2MASS
    r = np.zeros((n, 3))
    frac = rng.random(2)
    r[0, :2] = frac[0] * cell[:2, 0] + frac[1] * cell[:2, 1]
    r[0, 2] = z0
    r[1:] = pos
    v = np.zeros((n, 3))
    v[1:] = maxwell_boltzmann(rng, masses[1:], np.ones(n - 1, bool), Tsurf)
    v[0, 2] = -math.sqrt(2.0 * einc / masses[0])
    return Universe(r=r[:, None, :].copy(), v=v[:, None, :].copy(), m=masses, idx=np.array([1] + [2] * (n - 1), np.int32),
                    is_fixed=np.zeros((n, 1, 3), bool), simbox=cell, names=["H", "C"], is_proj=np.array([True, False]),
                    algo=np.array([algo, algo], np.int32))


def config4(ntraj: int = 2048, seed: int = 4):
    """H on 6x6 graphene (72 C + 1 H), Einc ~ U(0.5, 2) eV, Tsurf = 300 K."""
    rng = np.random.default_rng(seed)
    return [h_on_graphene(rng, rng.uniform(0.5, 2.0)) for _ in range(ntraj)]
