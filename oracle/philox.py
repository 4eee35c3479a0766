"""Counter-based generator of the engine's thermostats, restated in numpy.

TEST INFRASTRUCTURE ONLY: the checker of the device deviate streams (tests/ only).

The reference draws its Langevin, PILE and Andersen noise from the compiler's
``random_number`` and turns it into N(0,1) deviates by Box-Muller in FP64
(src/useful_things.f90:121-173).  The engine instead keys a Philox4x32-10 block
(Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11) by
(seed, trajectory, step, slot, stream), so every deviate is reproducible without state.
This module restates that generator from the paper, vectorised over counters, and the
two maps the device applies to a block: a uniform on [0, 1) from 53 bits (x >> 5, y >> 6)
and a Box-Muller normal in FP32 from the 24-bit uniforms (x >> 8) + 1 and z >> 8.
"""
from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: (n, 4) uint32 counters, key: (k0, k1) -> (n, 4) uint32 blocks (SC'11, Fig. 2,
    ten rounds, Weyl key schedule)."""
    c = [np.asarray(ctr[:, i], np.uint64) for i in range(4)]
    k0, k1 = int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c = [hi1 ^ c[1] ^ np.uint64(k0), lo1, hi0 ^ c[3] ^ np.uint64(k1), lo0]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return np.stack(c, axis=1).astype(np.uint32)


def blocks(seed, traj, step, stream, n):
    """The blocks of slots 0..n-1: counter (step, slot, stream, traj), key (seed lo, seed hi)."""
    ctr = np.zeros((n, 4), np.uint32)
    ctr[:, 0] = step
    ctr[:, 1] = np.arange(n, dtype=np.uint64).astype(np.uint32)
    ctr[:, 2] = stream
    ctr[:, 3] = traj
    return philox4x32_10(ctr, (seed & 0xFFFFFFFF, seed >> 32))


def uniforms(seed, traj, step, stream, n):
    b = blocks(seed, traj, step, stream, n).astype(np.uint64)
    v = ((b[:, 0] >> np.uint64(5)) << np.uint64(26)) | (b[:, 1] >> np.uint64(6))
    return (v.astype(np.float64) + 1.0) * 2.0 ** -53 - 2.0 ** -53


def normals(seed, traj, step, stream, n):
    b = blocks(seed, traj, step, stream, n)
    u1 = ((b[:, 0] >> 8) + 1).astype(np.float32) * np.float32(2.0 ** -24)
    u2 = (b[:, 2] >> 8).astype(np.float32) * np.float32(2.0 ** -24)
    r = np.sqrt(np.float32(-2.0) * np.log(u1))
    return (r * np.cos(np.float32(2.0 * np.pi) * u2.astype(np.float64)).astype(np.float32)).astype(np.float64)
