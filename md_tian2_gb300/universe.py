"""Host-side mirror of the reference's ``type universe`` (src/universe_mod.f90:38-67).

Arrays keep the reference's memory order: Fortran ``r(3, nbeads, natoms)`` is stored as
a C-contiguous numpy array of shape ``(natoms, nbeads, 3)``, which is the same bytes.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import constants as C


def invert_matrix(a: np.ndarray) -> np.ndarray:
    """Direct 3x3 inverse, src/useful_things.f90:296-321 (``a`` indexed a[row, col])."""
    A = lambda i, j: a[i - 1, j - 1]  # noqa: E731
    det = (A(1, 1) * A(2, 2) * A(3, 3) - A(1, 1) * A(2, 3) * A(3, 2) - A(1, 2) * A(2, 1) * A(3, 3)
           + A(1, 2) * A(2, 3) * A(3, 1) + A(1, 3) * A(2, 1) * A(3, 2) - A(1, 3) * A(2, 2) * A(3, 1))
    if det < C.TOLERANCE:
        raise ValueError("Error in invert_matrix: matrix is singular")
    d = 1.0 / det
    b = np.empty((3, 3))
    b[0, 0] = +d * (A(2, 2) * A(3, 3) - A(2, 3) * A(3, 2))
    b[1, 0] = -d * (A(2, 1) * A(3, 3) - A(2, 3) * A(3, 1))
    b[2, 0] = +d * (A(2, 1) * A(3, 2) - A(2, 2) * A(3, 1))
    b[0, 1] = -d * (A(1, 2) * A(3, 3) - A(1, 3) * A(3, 2))
    b[1, 1] = +d * (A(1, 1) * A(3, 3) - A(1, 3) * A(3, 1))
    b[2, 1] = -d * (A(1, 1) * A(3, 2) - A(1, 2) * A(3, 1))
    b[0, 2] = +d * (A(1, 2) * A(2, 3) - A(1, 3) * A(2, 2))
    b[1, 2] = -d * (A(1, 1) * A(2, 3) - A(1, 3) * A(2, 1))
    b[2, 2] = +d * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1))
    return b


@dataclass
class Universe:
    """One trajectory's atoms: the fields of ``type universe`` the hot path reads."""

    r: np.ndarray                 # (N, nb, 3)  positions, A
    v: np.ndarray                 # (N, nb, 3)  velocities, A/fs
    m: np.ndarray                 # (N,)        masses, eV fs^2 / A^2
    idx: np.ndarray               # (N,)        1-based type index
    is_fixed: np.ndarray          # (N, nb, 3)  bool
    simbox: np.ndarray            # (3, 3)      cell vectors as columns (simbox[:, k] = a_k)
    names: list = field(default_factory=list)    # per type
    is_proj: np.ndarray = None    # (ntypes,) bool
    algo: np.ndarray = None       # (ntypes,) propagator ids

    @property
    def natoms(self) -> int:
        return self.r.shape[0]

    @property
    def nbeads(self) -> int:
        return self.r.shape[1]

    @property
    def ntypes(self) -> int:
        return len(self.names)

    @property
    def isimbox(self) -> np.ndarray:
        return invert_matrix(self.simbox)

    def copy(self) -> "Universe":
        return Universe(self.r.copy(), self.v.copy(), self.m.copy(), self.idx.copy(), self.is_fixed.copy(),
                        self.simbox.copy(), list(self.names), None if self.is_proj is None else self.is_proj.copy(),
                        None if self.algo is None else self.algo.copy())

    def force_beads(self, nb: int) -> "Universe":
        """post_process's bead replication, src/md_init.f90:630-671."""
        rep = lambda a: np.repeat(a[:, :1, :], nb, axis=1).copy()  # noqa: E731
        return Universe(rep(self.r), rep(self.v), self.m.copy(), self.idx.copy(), rep(self.is_fixed),
                        self.simbox.copy(), list(self.names), None if self.is_proj is None else self.is_proj.copy(),
                        None if self.algo is None else self.algo.copy())
