"""Restatement of the reference's trajectory observables, the checker of the device-side
tracking (mdt_traj_observables).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker; the product
(md_tian2_gb300) never imports it.

collect_trajectory_characteristics (src/trajectory_info.f90:47-75), called once per MD
step with the step's positions and velocities (N, nbeads, 3):
- check_for_lowest_position (:136-145): the projectile centroid position with the lowest z;
- check_for_closest_approach (:80-132): the minimum image (direct coordinates minus
  anint) of the centroid distances from atom 1 (the projectile) to atoms 2..N; the first
  step reaching the smallest value;
- check_for_bounce (:243-250): a turning point whenever the sign of the projectile
  centroid's z velocity differs from the previous one (moving down at the start).
"""
from __future__ import annotations

import numpy as np

HUGE = np.finfo(np.float64).max  # default_real, src/constants.f90:101


class TrajectoryInfo:
    def __init__(self, simbox):
        self.box = np.asarray(simbox, float)
        self.ibox = np.linalg.inv(self.box)
        self.turn, self.up, self.cl, self.clstep = 0, False, HUGE, 0
        self.low = np.full(3, HUGE)
        self.dist = {}  # closest approach of each step

    def __call__(self, k, r, v):
        c = r.mean(axis=1)
        if c[0, 2] < self.low[2]:
            self.low = c[0].copy()
        d = c[0] - c[1:]
        f = d @ self.ibox.T
        f -= np.round(f)
        dist = np.sqrt(np.sum((f @ self.box.T) ** 2, axis=1)).min()
        self.dist[k] = dist
        if dist < self.cl:
            self.cl, self.clstep = dist, k
        down = v[0].mean(axis=0)[2] < 0
        if down == self.up:
            self.turn += 1
            self.up = not down
