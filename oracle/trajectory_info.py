"""Restatement of the reference's trajectory observables, the checker of the device-side
tracking (mdt_traj_observables, mdt_traj_bounces).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker; the product
(md_tian2_gb300) never imports it.

collect_trajectory_characteristics (src/trajectory_info.f90:47-75), called once per MD
step with the step's positions, velocities and forces (N, nbeads, 3):
- check_for_lowest_position (:136-145): the projectile centroid position with the lowest z;
- check_for_closest_approach (:80-132): the minimum image (direct coordinates minus
  anint) of the centroid distances from atom 1 (the projectile) to atoms 2..N; the first
  step reaching the smallest value; the nearest atom of this step (first index on ties);
  the adsorption flag with its hysteresis (below adsorption_start: adsorbed, above
  adsorption_end: not adsorbed);
- check_for_proj_surf_interaction (:140-148): steps with a non-zero projectile force;
- check_for_bounce (:152-250): r = unit vector from the projectile to its nearest atom
  (minimum image), v, F = unit centroid velocity and force of the projectile; while the
  nearest atom stays the same, the crossings of r.v with r.F and with v.F and the + to -
  sign changes of r.v are counted (not when r.F = 0); a change of the nearest atom closes
  the segment, adding min(three counts) to the bounces (finalize_bounces, :252-256, also
  called once by output_scatter before the record is written); a turning point whenever
  the sign of the projectile centroid's z velocity differs from the previous one (moving
  down at the start).
"""
from __future__ import annotations

import numpy as np

HUGE = np.finfo(np.float64).max  # default_real, src/constants.f90:101


def _normalize(x):
    with np.errstate(invalid="ignore", divide="ignore"):
        return x / np.sqrt(np.sum(x * x))


class TrajectoryInfo:
    def __init__(self, simbox, adsorption=(HUGE, HUGE), step=0.1):
        self.box = np.asarray(simbox, float)
        self.ibox = np.linalg.inv(self.box)
        self.turn, self.up, self.cl, self.clstep = 0, False, HUGE, 0
        self.low = np.full(3, HUGE)
        self.dist = {}  # closest approach of each step
        self.ads_start, self.ads_end = adsorption
        self.step = step
        self.adsorbed = False
        self.bounces = 0
        self.rv = [HUGE, HUGE]
        self.rF = [HUGE, HUGE]
        self.vF = [HUGE, HUGE]
        self.partner_change = 1
        self.rFcut = self.vFcut = self.ptm = 0
        self.last_idx = None
        self.inter_steps = 0

    def _image(self, d):
        f = d @ self.ibox.T
        f -= np.round(f)
        return f @ self.box.T

    def __call__(self, k, r, v, f=None):
        c = r.mean(axis=1)
        if c[0, 2] < self.low[2]:
            self.low = c[0].copy()
        dvec = self._image(c[0] - c[1:])
        dd = np.sqrt(np.sum(dvec ** 2, axis=1))
        near = int(np.argmin(dd)) + 1  # first index of the minimum, 0-based atom index
        dist = dd[near - 1]
        self.dist[k] = dist
        if dist < self.cl:
            self.cl, self.clstep = dist, k
        if not self.adsorbed and dist < self.ads_start:
            self.adsorbed = True
        if self.adsorbed and dist > self.ads_end:
            self.adsorbed = False
        if f is not None:
            if np.any(f[0] != 0):
                self.inter_steps += 1
            self._bounce(k, c, near, v, f)
        down = v[0].mean(axis=0)[2] < 0
        if down == self.up:
            self.turn += 1
            self.up = not down

    def _bounce(self, k, c, near, v, f):
        rr = _normalize(self._image(c[near] - c[0]))
        vv = _normalize(v[0].mean(axis=0))
        ff = _normalize(f[0].mean(axis=0))
        last, this = (k + 1) % 2, k % 2
        self.rv[this] = float(np.dot(rr, vv))
        self.rF[this] = float(np.dot(rr, ff))
        self.vF[this] = float(np.dot(vv, ff))
        if self.last_idx is None:
            self.last_idx = near
        rv, rF, vF = self.rv, self.rF, self.vF
        if self.last_idx != near:
            self.bounces += min(self.ptm, self.rFcut, self.vFcut)
            self.partner_change = -self.partner_change
            self.rFcut = self.vFcut = self.ptm = 0
        elif rF[this] != 0:
            if rv[last] > rF[last] and rv[this] < rF[this]:
                self.rFcut += 1
            elif rv[last] < rF[last] and rv[this] > rF[this]:
                self.rFcut += 1
            if rv[last] > vF[last] and rv[this] < vF[this]:
                self.vFcut += 1
            elif rv[last] < vF[last] and rv[this] > vF[this]:
                self.vFcut += 1
            if rv[last] > 0 and rv[this] < 0:
                self.ptm += 1
        self.last_idx = near

    def final_bounces(self):
        """bounces as output_scatter leaves them (after its finalize_bounces call)."""
        return self.bounces + min(self.ptm, self.rFcut, self.vFcut)

    def interaction_time(self):
        return self.inter_steps * self.step
