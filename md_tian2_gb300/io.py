"""Readers for the reference's input formats.

* ``.pes`` blocks (src/md_init.f90:83-154 dispatch, src/pes_emt_mod.f90:49-190 for EMT):
  ``pes emt`` / ``A B proj|latt proj|latt`` / ``key value`` lines / blank line.
  In a two-element block the first 7 parameters belong to A, the next 7 to B.
* ``mxt`` geometry files (src/md_init.f90:346-381): Fortran unformatted sequential,
  4-byte record markers, records (natoms, nbeads, ntypes) and
  (r, v, is_cart, is_fixed, idx, name, is_proj, simbox, isimbox); logicals are 4 bytes.
* POSCAR (src/md_init.f90:195-342) with the optional bead count, mobility flags and
  velocity section, and ``create_repetitions`` (src/universe_mod.f90:120-217).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import constants as C
from .universe import Universe, invert_matrix

EMT_KEYS = ("eta2", "n0", "e0", "lambda", "v0", "kappa", "s0")


class InputError(ValueError):
    """Malformed input; the reference would print and ``stop``."""


@dataclass
class EmtParams:
    """Per-type EMT parameters and the pes matrix (what read_emt fills in)."""

    ntypes: int
    values: dict = field(default_factory=dict)   # key -> np.ndarray(ntypes)
    pes: np.ndarray = None                       # (ntypes, ntypes) int32, pes[i, j]

    def arrays(self):
        return [np.ascontiguousarray(self.values[k], dtype=np.float64) for k in EMT_KEYS]


def _type_index(names, is_proj, name, role):
    want_proj = role == "proj"
    for t, (n, p) in enumerate(zip(names, is_proj)):
        if n == name and bool(p) == want_proj:
            return t
    raise InputError("Error in get_idx_from_name(): make sure you correctly assign element names to "
                     f"projectile and slab in both *.inp and *.pes files ({name} {role})")


def read_pes(path, names, is_proj) -> EmtParams:
    """Parse every ``pes emt`` block of a .pes file for a universe whose types are
    ``names`` (per 1-based type, in order) with projectile flags ``is_proj``."""
    ntypes = len(names)
    out = EmtParams(ntypes=ntypes, values={k: np.full(ntypes, np.inf) for k in EMT_KEYS},
                    pes=np.zeros((ntypes, ntypes), dtype=np.int32))
    lines = Path(path).read_text().splitlines()
    k = 0
    while k < len(lines):
        words = lines[k].split()
        k += 1
        if len(words) == 2 and words[0] == "pes":
            if words[1] != "emt":
                raise InputError(f"unsupported potential in PES file: {words[1]}")
            if k >= len(lines):
                raise InputError("Error in read_emt: need four entries in interaction-defining lines")
            head = lines[k].split()
            k += 1
            if len(head) != 4:
                raise InputError("Error in read_emt: need four entries in interaction-defining lines")
            if head[2] not in ("proj", "latt") or head[3] not in ("proj", "latt"):
                raise InputError("interaction must be defined via 'proj' and 'latt' keywords")
            i1 = _type_index(names, is_proj, head[0], head[2])
            i2 = _type_index(names, is_proj, head[1], head[3])
            if out.pes[i1, i2] != 0:
                raise InputError(f"pes already defined for atoms {head}")
            out.pes[i1, i2] = out.pes[i2, i1] = C.PES_ID_EMT
            counter = 1
            while k < len(lines):
                w = lines[k].split()
                k += 1
                if len(w) == 0:
                    break
                if len(w) != 2:
                    raise InputError("Error in the PES file: PES parameters must consist of key value pairs. "
                                     "A parameter block must be terminated by a blank line.")
                key = w[0].lower()
                if key not in EMT_KEYS:
                    raise InputError(f"Error in the PES file: unknown parameter {w[0]}")
                tgt = i1 if counter <= 7 else i2
                out.values[key][tgt] = float(w[1].replace("d", "e").replace("D", "e"))
                counter += 1
    if np.any(out.pes == 0):
        raise InputError("Error in read_pes(): pes matrix incomplete")
    for t in range(ntypes):
        if out.pes[t, t] == C.PES_ID_EMT:
            for key in EMT_KEYS:
                if not np.isfinite(out.values[key][t]):
                    raise InputError(f"EMT parameter {key} missing for type {names[t]}")
    return out


def _records(buf: bytes):
    """Split a Fortran unformatted sequential file into records."""
    off, recs = 0, []
    while off < len(buf):
        if off + 4 > len(buf):
            raise InputError("truncated record marker")
        (n,) = struct.unpack_from("<i", buf, off)
        if n < 0 or off + 8 + n > len(buf):
            raise InputError("bad record length")
        recs.append(buf[off + 4: off + 4 + n])
        (n2,) = struct.unpack_from("<i", buf, off + 4 + n)
        if n2 != n:
            raise InputError("record markers disagree")
        off += 8 + n
    return recs


def read_mxt(path, masses_amu=None) -> Universe:
    """read_mxt, src/md_init.f90:346-381.  ``masses_amu`` maps element -> amu."""
    recs = _records(Path(path).read_bytes())
    if len(recs) < 2 or len(recs[0]) != 12:
        raise InputError("Error in read_mxt(): cannot read universe type constructor arguments")
    natoms, nbeads, ntypes = struct.unpack("<3i", recs[0])
    b = recs[1]
    n3 = 3 * nbeads * natoms
    need = 8 * n3 * 2 + 4 + 4 * n3 + 4 * natoms + 3 * ntypes + 4 * ntypes + 8 * 18
    if len(b) != need:
        raise InputError(f"Error in read_mxt(): cannot read file (record of {len(b)} bytes, expected {need})")
    o = 0
    r = np.frombuffer(b, "<f8", n3, o).reshape(natoms, nbeads, 3).copy(); o += 8 * n3
    v = np.frombuffer(b, "<f8", n3, o).reshape(natoms, nbeads, 3).copy(); o += 8 * n3
    is_cart = struct.unpack_from("<i", b, o)[0] != 0; o += 4
    fixed = np.frombuffer(b, "<i4", n3, o).reshape(natoms, nbeads, 3) != 0; o += 4 * n3
    idx = np.frombuffer(b, "<i4", natoms, o).copy(); o += 4 * natoms
    names = [b[o + 3 * t: o + 3 * t + 3].decode("ascii").strip() for t in range(ntypes)]; o += 3 * ntypes
    is_proj = np.frombuffer(b, "<i4", ntypes, o) != 0; o += 4 * ntypes
    simbox = np.frombuffer(b, "<f8", 9, o).reshape(3, 3).T.copy(); o += 72   # column major
    if not is_cart:
        r = np.einsum("ij,nbj->nbi", simbox, r)
    masses_amu = masses_amu or C.MASS_AMU
    m = np.array([masses_amu.get(names[i - 1], np.nan) for i in idx]) * C.AMU2MASS
    return Universe(r=r, v=v, m=m, idx=idx.astype(np.int32), is_fixed=fixed.copy(), simbox=simbox,
                    names=names, is_proj=is_proj.copy(), algo=np.full(ntypes, C.PROP_ID_VERLET, np.int32))


def write_mxt(path, u: Universe) -> None:
    """Inverse of read_mxt (Cartesian coordinates), for round-trip tests and dumps
    (the reference's ``output mxt``, src/output_mod.f90:612)."""
    def rec(payload: bytes) -> bytes:
        return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))
    p1 = struct.pack("<3i", u.natoms, u.nbeads, u.ntypes)
    parts = [np.ascontiguousarray(u.r, "<f8").tobytes(), np.ascontiguousarray(u.v, "<f8").tobytes(),
             struct.pack("<i", -1), np.where(u.is_fixed, -1, 0).astype("<i4").tobytes(),
             np.asarray(u.idx, "<i4").tobytes(), "".join(f"{n:<3.3s}" for n in u.names).encode("ascii"),
             np.where(np.asarray(u.is_proj), -1, 0).astype("<i4").tobytes(),
             np.asarray(u.simbox.T, "<f8").tobytes(), np.asarray(invert_matrix(u.simbox).T, "<f8").tobytes()]
    Path(path).write_bytes(rec(p1) + rec(b"".join(parts)))


def create_repetitions(u: Universe, rep=(0, 0)) -> Universe:
    """create_repetitions, src/universe_mod.f90:120-217: the non-projectile atoms are
    repeated (1 + 2 rep[0]) x (1 + 2 rep[1]) times along the first two cell vectors (direct
    offsets -rep..rep, the second index fastest), projectile atoms (those leading the atom
    list) stay first and unmoved, and the first two cell vectors grow by the same factors."""
    r1, r2 = int(rep[0]), int(rep[1])
    if r1 < 0 or r2 < 0:
        raise InputError("Error in create_repetitions: negative repetition")
    if r1 == 0 and r2 == 0:
        return u
    proj_type = np.asarray(u.is_proj, bool)
    nprojs = int(np.sum(proj_type[np.asarray(u.idx) - 1]))
    if not np.all(proj_type[np.asarray(u.idx[:nprojs]) - 1]):
        raise InputError("Error in create_repetitions: projectile atoms must lead the atom list")
    box = np.asarray(u.simbox, float)
    frac = np.einsum("ij,nbj->nbi", invert_matrix(box), u.r)  # direct coordinates
    parts_r, parts = [frac[:nprojs]], {k: [getattr(u, k)[:nprojs]] for k in ("v", "m", "idx", "is_fixed")}
    for i in range(-r1, r1 + 1):
        for j in range(-r2, r2 + 1):
            f = frac[nprojs:].copy()
            f[..., 0] += i
            f[..., 1] += j
            parts_r.append(f)
            for k in parts:
                parts[k].append(getattr(u, k)[nprojs:])
    r = np.einsum("ij,nbj->nbi", box, np.concatenate(parts_r))
    big = box.copy()
    big[:, 0] *= 1 + 2 * r1
    big[:, 1] *= 1 + 2 * r2
    return Universe(r=r, v=np.concatenate(parts["v"]).copy(), m=np.concatenate(parts["m"]).copy(),
                    idx=np.concatenate(parts["idx"]).astype(np.int32), is_fixed=np.concatenate(parts["is_fixed"]).copy(),
                    simbox=big, names=list(u.names), is_proj=np.array(u.is_proj, bool),
                    algo=None if u.algo is None else np.array(u.algo))


def read_poscar(path, nprojectiles: int = 1, masses_amu=None, rep=(0, 0)) -> Universe:
    """read_poscar, src/md_init.f90:195-342: comment line; scaling constant; three cell
    vectors; element names; atom counts, optionally preceded by ``:nbeads:``; coordinate
    system (d/direct or c/cart/cartesian); coordinates, 3 per line or 3 plus mobility
    flags T/F per line (atom-major, bead-minor); optionally a blank line and velocities in
    the same order.  The first ``nprojectiles`` element types are projectiles.  Cartesian
    coordinates are scaled by the constant, velocities are not; the result is Cartesian
    after ``create_repetitions(rep)``.  Masses from ``masses_amu`` (element -> amu)."""
    lines = Path(path).read_text().splitlines()
    err = "Error in read_poscar: "
    if len(lines) < 8:
        raise InputError(err + "file too short")
    try:
        scale = float(lines[1].split()[0])
    except (IndexError, ValueError):
        raise InputError(err + "reading scaling constant") from None
    try:
        cell = np.array([[float(x) for x in lines[2 + k].split()[:3]] for k in range(3)])
    except ValueError:
        raise InputError(err + "reading simulation box") from None
    if cell.shape != (3, 3):
        raise InputError(err + "reading simulation box")
    elements = lines[5].split()
    counts_line = lines[6]
    nbeads = 1
    if ":" in counts_line:
        a, b = counts_line.index(":"), counts_line.rindex(":")
        try:
            nbeads = int(counts_line[a + 1:b])
        except ValueError:
            raise InputError(err + "reading number of beads") from None
        if nbeads < 1:
            raise InputError(err + "reading number of beads")
        counts_line = counts_line[b + 1:]
    try:
        natoms = [int(x) for x in counts_line.split()]
    except ValueError:
        raise InputError(err + "reading number of atoms") from None
    if len(natoms) != len(elements) or any(n <= 0 for n in natoms):
        raise InputError(err + "number of atoms could not be read")
    csys = lines[7].strip().lower()
    if csys not in ("d", "direct", "c", "cart", "cartesian"):
        raise InputError(err + "reading coordinate system type (cartesian/direct)")
    N = sum(natoms)
    nrow = N * nbeads
    body = lines[8:8 + nrow]
    if len(body) < nrow:
        raise InputError(err + "reading coordinates")
    nwords = len(body[0].split())
    if nwords not in (3, 6):
        raise InputError(err + "cannot read coordinate section")
    r = np.zeros((N, nbeads, 3))
    fixed = np.zeros((N, nbeads, 3), bool)
    for row, line in enumerate(body):
        w = line.split()
        if len(w) != nwords:
            raise InputError(err + "reading atom coordinates and mobility flags")
        i, b = divmod(row, nbeads)
        r[i, b] = [float(x) for x in w[:3]]
        if nwords == 6:
            fixed[i, b] = [x == "F" for x in w[3:]]
    v = np.zeros_like(r)
    rest = lines[8 + nrow:]
    if rest and rest[0].strip() == "":
        vals = [float(x) for l in rest[1:] for x in l.split()]
        if len(vals) < 3 * nrow:
            raise InputError(err + "cannot read initial atom velocities")
        v = np.array(vals[:3 * nrow]).reshape(N, nbeads, 3)
    elif rest and rest[0].strip():
        raise InputError(err + "cannot read initial atom velocities. Did you specify all species in the *.inp file?")
    box = cell.T * scale  # simbox(:, k) = k-th vector
    if csys.startswith("c"):
        r = r * scale
    else:
        r = np.einsum("ij,nbj->nbi", box, r)
    masses_amu = masses_amu or C.MASS_AMU
    idx = np.concatenate([[k + 1] * n for k, n in enumerate(natoms)]).astype(np.int32)
    m = np.array([masses_amu.get(elements[i - 1], np.nan) for i in idx]) * C.AMU2MASS
    is_proj = np.arange(len(elements)) < nprojectiles
    u = Universe(r=r, v=v, m=m, idx=idx, is_fixed=fixed, simbox=box, names=elements, is_proj=is_proj,
                 algo=np.full(len(elements), C.PROP_ID_VERLET, np.int32))
    return create_repetitions(u, rep)
