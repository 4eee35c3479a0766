"""Readers for the reference's input formats.

* ``.pes`` blocks (src/md_init.f90:83-154 dispatch, src/pes_emt_mod.f90:49-190 for EMT):
  ``pes emt`` / ``A B proj|latt proj|latt`` / ``key value`` lines / blank line.
  In a two-element block the first 7 parameters belong to A, the next 7 to B.
* ``mxt`` geometry files (src/md_init.f90:346-381): Fortran unformatted sequential,
  4-byte record markers, records (natoms, nbeads, ntypes) and
  (r, v, is_cart, is_fixed, idx, name, is_proj, simbox, isimbox); logicals are 4 bytes.
* POSCAR (src/md_init.f90:195-342), the subset without repetitions.
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
