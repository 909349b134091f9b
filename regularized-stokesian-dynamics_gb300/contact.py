"""Host-side contact forces between near-touching spheres: a stand-in for
the reference's DEM contact engine (the `DEM` branch of main.f90, which
hands contact forces to the hydrodynamic step as external forces Fe and
runs on the host; it is not part of the GPU path).

The force is a short-range repulsion along the line of centres, of the form
Bossis and Brady used for dense Stokesian dynamics (J. Chem. Phys. 80,
5141, 1984): for a surface gap h, F = F0 exp(-h / delta), and for an overlap
(h < 0) F = F0 (1 - h / delta), continuous at contact.  With the
dimensionless units of the step (mu_f = 1/pi, radius 1, shear rate 1) the
Stokes drag scale 6 pi mu_f a^2 gammadot is 6, and F0 is given in multiples
of it.

Neighbours come from a list of pairs within 2a + skin, rebuilt every
`rebuild` steps; each step takes the minimum image of every listed pair in
the current Lees-Edwards lattice (skew = strain mod 1), so the list stays
valid while the particles move less than skin / 2.
"""
from __future__ import annotations

import numpy as np

from . import configs


class SoftContact:
    def __init__(self, N, L, a=1.0, f0=100.0, delta=0.01, skin=0.3, rebuild=20, gamma=1.0):
        self.N, self.L, self.a = N, float(L), float(a)
        self.F0 = f0 * 6.0 * a * a * gamma  # 6 pi mu_f a^2 gammadot with mu_f = 1/pi
        self.delta, self.skin, self.rebuild, self.gamma = float(delta), float(skin), int(rebuild), float(gamma)
        self.count = 0
        self.i = self.j = None
        self.min_gap = np.inf

    def _skew(self, T):
        s = (self.gamma * T) % 1.0
        return s

    def forces(self, conf, T):
        """Fe (6N: forces, then zero torques) for the configuration at time T."""
        pos = np.asarray(conf, dtype=np.float64).reshape(self.N, 3)
        skew = self._skew(T)
        if self.i is None or self.count % self.rebuild == 0:
            i, j, _ = configs._pairs_within(pos, self.L, skew, 2 * self.a + self.skin)
            self.i, self.j = np.asarray(i), np.asarray(j)
        self.count += 1
        Fe = np.zeros(6 * self.N)
        if len(self.i) == 0:
            return Fe
        LR, LI = configs._sheared_lattice(self.L, skew)
        d = configs.sheared_min_image(pos[self.j] - pos[self.i], LR, LI)
        r = np.sqrt(np.einsum("ij,ij->i", d, d))
        h = r - 2 * self.a
        self.min_gap = float(h.min())
        act = h < 10 * self.delta
        if not act.any():
            return Fe
        hh, dd, rr = h[act], d[act], r[act]
        f = np.where(hh >= 0, self.F0 * np.exp(-hh / self.delta), self.F0 * (1.0 - hh / self.delta))
        fv = (f / rr)[:, None] * dd  # on j, away from i
        F = np.zeros((self.N, 3))
        np.add.at(F, self.j[act], fv)
        np.add.at(F, self.i[act], -fv)
        Fe[:3 * self.N] = F.ravel()
        return Fe
