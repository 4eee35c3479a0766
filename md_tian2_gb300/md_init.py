"""Trajectory initialisation of the reference (src/md_init.f90), restated on the host for
batches: ``merge_universes`` (projectile + slab, :557-617), ``apply_pip`` (projectile
initial position, :498-553), ``set_proj_incidence`` (incidence energy and angles,
:829-876) and ``force_beads`` (post_process, :630-671).

Random numbers: the reference draws from the compiler's ``random_number``; here a
``numpy.random.Generator`` passed by the caller supplies the uniform and normal deviates in
the same order (one uniform per random pip coordinate, then the incidence energy deviate,
then the azimuth), so a batch is reproducible from its seed.

``apply_pip`` keeps the reference's arithmetic: after drawing direct coordinate k it
multiplies the whole target vector by the sum of the k-th cell vector's components
(:523-525), so the random target lies outside the cell; ``merge_universes`` folds every
centroid back into the cell (:608-613), which puts the projectile at a pseudo-random
in-cell position (not uniform). ``workloads.h_on_metal`` draws a uniform in-plane position
instead, which is what the synthetic benchmarks use.
"""
from __future__ import annotations

import math

import numpy as np

from . import constants as C
from .universe import Universe, invert_matrix


def _centroids(u: Universe) -> np.ndarray:
    return u.r.mean(axis=1)


def apply_pip(proj: Universe, pip, rng) -> Universe:
    """apply_pip, md_init.f90:498-553.  ``pip`` holds three entries, each ``"r"`` (random
    direct coordinate) or a number (Cartesian offset in A); every atom must be a
    projectile."""
    if not np.all(np.asarray(proj.is_proj)[np.asarray(proj.idx) - 1]):
        raise ValueError("Error in apply_pip(): there are lattice atoms affected by apply_pip() subroutine")
    r = proj.r.copy()
    cents = _centroids(proj)
    box = proj.simbox
    target = np.zeros(3)
    for k in range(3):
        if str(pip[k]).strip() == "r":
            target[k] = rng.random()
            target = target * np.sum(box[:, k])
        else:
            try:
                r[:, :, k] += float(pip[k])
            except ValueError:
                raise ValueError(f"Error in apply_pip(): unknown pip format at position {k + 1} of pip array") from None
    for k in range(3):
        fixed = box[k, 0] * target[0] + box[k, 1] * target[1] + box[k, 2] * target[2]
        r[:, :, k] = r[:, :, k] - cents[:, None, k] + fixed
    return Universe(r=r, v=proj.v.copy(), m=proj.m.copy(), idx=proj.idx.copy(), is_fixed=proj.is_fixed.copy(),
                    simbox=proj.simbox.copy(), names=list(proj.names), is_proj=np.array(proj.is_proj),
                    algo=None if proj.algo is None else np.array(proj.algo))


def merge_universes(slab: Universe, proj: Universe, pip=None, rng=None, algo_p=C.PROP_ID_VERLET,
                    algo_l=C.PROP_ID_VERLET) -> Universe:
    """merge_universes, md_init.f90:557-617: the projectile (one atom) first, then the slab
    with its type indices shifted; propagators per type (projectile, lattice); the slab's
    cell; then every atom's centroid folded into the cell by subtracting the integer part
    of its direct coordinates (Fortran int(): truncation toward zero)."""
    err = "Error in merge_universes: "
    if slab.nbeads != proj.nbeads:
        raise ValueError(err + "mxt and merge files differ in number of beads")
    if np.any(np.asarray(slab.is_proj)):
        raise ValueError(err + "mxt file contains projectile atoms")
    if not np.all(np.asarray(proj.is_proj)):
        raise ValueError(err + "merge file contains lattice atoms")
    if proj.natoms > 1:
        raise ValueError(err + "multiple projectiles not implemented for use with merge option")
    if pip is not None:
        proj = apply_pip(proj, pip, rng)
    r = np.concatenate([proj.r, slab.r])
    box = slab.simbox
    ibox = invert_matrix(box)
    cent = np.concatenate([_centroids(proj), _centroids(slab)]) @ ibox.T
    frac = np.einsum("ij,nbj->nbi", ibox, r) - np.trunc(cent)[:, None, :]
    r = np.einsum("ij,nbj->nbi", box, frac)
    return Universe(r=r, v=np.concatenate([proj.v, slab.v]), m=np.concatenate([proj.m, slab.m]),
                    idx=np.concatenate([proj.idx, np.asarray(slab.idx) + int(np.max(proj.idx))]).astype(np.int32),
                    is_fixed=np.concatenate([proj.is_fixed, slab.is_fixed]), simbox=box.copy(),
                    names=list(proj.names) + list(slab.names),
                    is_proj=np.concatenate([np.asarray(proj.is_proj, bool), np.asarray(slab.is_proj, bool)]),
                    algo=np.array([algo_p, algo_l], np.int32))


def set_proj_incidence(u: Universe, einc: float, polar_deg: float, azimuth="r", rng=None, sigma_einc: float = 0.0,
                       sigma_azimuth: float = 0.0) -> Universe:
    """set_proj_incidence, md_init.f90:829-876: the incidence energy drawn from
    N(einc, sigma_einc), the azimuth uniform in [0, 2 pi) (``"r"``) or N(azimuth,
    sigma_azimuth) in degrees; every projectile atom (they lead the atom list) loses its
    centre-of-mass drift over the beads and gains v = sqrt(2 E / m_proj) (sin(polar)
    cos(azi), sin(polar) sin(azi), -cos(polar)), with m_proj the projectiles' total mass."""
    rng = rng or np.random.default_rng()
    e = einc + sigma_einc * rng.standard_normal() if sigma_einc > 0 else einc
    proj_mask = np.asarray(u.is_proj)[np.asarray(u.idx) - 1]
    m_proj = float(np.sum(u.m[proj_mask]))
    if str(azimuth).strip() == "r":
        azi = 2.0 * math.pi * rng.random()
    else:
        a = float(azimuth)
        if sigma_azimuth > 0:
            a = a + sigma_azimuth * rng.standard_normal()
        azi = a * C.DEG2RAD
    pol = polar_deg * C.DEG2RAD
    vinc = math.sqrt(2.0 * e / m_proj)
    vel = np.array([vinc * math.sin(pol) * math.cos(azi), vinc * math.sin(pol) * math.sin(azi), -vinc * math.cos(pol)])
    v = u.v.copy()
    for i in range(u.natoms):
        if not proj_mask[i]:
            break  # projectiles are always at the beginning of the universe
        v[i] = v[i] - v[i].mean(axis=0) + vel  # remove_atomic_com, then the incidence velocity
    return Universe(r=u.r.copy(), v=v, m=u.m.copy(), idx=u.idx.copy(), is_fixed=u.is_fixed.copy(),
                    simbox=u.simbox.copy(), names=list(u.names), is_proj=np.array(u.is_proj),
                    algo=None if u.algo is None else np.array(u.algo))


def force_beads(u: Universe, nbeads: int) -> Universe:
    """post_process's force_beads, md_init.f90:630-671: every bead a copy of bead 1."""
    return u.force_beads(nbeads)
