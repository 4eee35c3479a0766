"""The HDNNP arm's FLOP convention counts geometry (every image within the cutoff), so its
pairs and triplets (r_ij, r_ik, r_jk inside the cutoff) must not depend on where the atoms
sit in the periodic frame: unchanged when atoms move by lattice vectors, and every pair
counted from both of its atoms.  (The EMT arm counts the reference's minimum-image pairs,
the pairs its kernels compute; on a skewed cell rounding fractional coordinates is not
frame invariant, in the reference either.)"""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402
from md_tian2_gb300 import workloads as W  # noqa: E402


def _shifted(us, seed):
    rng = np.random.default_rng(seed)
    out = []
    for u in us:
        v = W.Universe(**{k: getattr(u, k) for k in ("r", "v", "m", "idx", "is_fixed", "simbox", "names", "is_proj",
                                                      "algo")})
        v.r = u.r.copy()
        n = rng.integers(-2, 3, size=(u.natoms, 3)).astype(float)
        v.r[:, 0, :] += n @ np.asarray(u.simbox, float).T
        out.append(v)
    return out


def test_hdnnp_triplets_do_not_depend_on_the_periodic_frame():
    us = W.config4(2, seed=4)
    pairs, trip = bench._valid_triplets(us, 6.5, 2)
    pairs2, trip2 = bench._valid_triplets(_shifted(us, 1), 6.5, 2)
    assert (pairs, trip) == (pairs2, trip2)
    assert pairs % 2 == 0
    # graphene at a 6.5 A cutoff: about 45 neighbours and 550 triplets (j < k) per atom
    n = sum(u.natoms for u in us)
    assert 40 < pairs / n < 50 and 450 < trip / n < 650
