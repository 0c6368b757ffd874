"""Analytic spherical background models used to build basis tables.

A model supplies density rho(r), enclosed mass M(r), potential Phi(r) and
dPhi/dr with G = 1.  The Hernquist profile follows
``exptool/models/hernquist.py:86-110`` (Phi = -M/(r+a), dPhi/dr = M/(r+a)^2);
the truncated variant renormalises the mass inside ``rtrunc`` to ``mass`` so
that it matches a particle sample drawn with an exact r < rtrunc cut.
"""
from __future__ import annotations

import numpy as np


class TruncatedHernquist:
    """Hernquist sphere cut at ``rtrunc`` and rescaled to total mass ``mass``.

    rho(r) = mass/f * a / (2 pi r (r+a)^3)  for r < rtrunc, f = (rt/(rt+a))^2.
    Phi(r) = mass/f * (-1/(r+a) + a/(rt+a)^2)  inside (the shell term removes
    the mass beyond rt), and -mass/r outside.
    """

    def __init__(self, a: float = 1.0, mass: float = 1.0, rtrunc: float = 100.0):
        self.a = float(a)
        self.mass = float(mass)
        self.rt = float(rtrunc)
        self.f = (self.rt / (self.rt + self.a)) ** 2
        self.norm = self.mass / self.f

    def density(self, r):
        r = np.asarray(r, dtype=np.float64)
        a = self.a
        out = self.norm * a / (2.0 * np.pi * r * (r + a) ** 3)
        return np.where(r <= self.rt * (1.0 + 1e-12), out, 0.0)

    def enclosed_mass(self, r):
        r = np.asarray(r, dtype=np.float64)
        m = self.norm * (r / (r + self.a)) ** 2
        return np.where(r <= self.rt * (1.0 + 1e-12), m, self.mass)

    def potential(self, r):
        r = np.asarray(r, dtype=np.float64)
        a, rt = self.a, self.rt
        inside = self.norm * (-1.0 / (r + a) + a / (rt + a) ** 2)
        return np.where(r <= rt * (1.0 + 1e-12), inside, -self.mass / np.maximum(r, 1e-300))

    def dpotential(self, r):
        """dPhi/dr."""
        r = np.asarray(r, dtype=np.float64)
        inside = self.norm / (r + self.a) ** 2
        return np.where(r <= self.rt * (1.0 + 1e-12), inside, self.mass / np.maximum(r, 1e-300) ** 2)


class SphericalExponential:
    """Spherical stand-in for an exponential disc of scale length ``a``.

    rho(r) = mass e^{-r/a} / (4 pi a^2 r), M(r) = mass (1 - (1 + r/a) e^{-r/a}),
    Phi(r) = -mass (1 - e^{-r/a}) / r.  Used as the background model of the
    spherical basis from which the cylindrical (EOF) tables are built.
    """

    def __init__(self, a: float = 1.0, mass: float = 1.0):
        self.a = float(a)
        self.mass = float(mass)

    def density(self, r):
        r = np.asarray(r, dtype=np.float64)
        return self.mass * np.exp(-r / self.a) / (4.0 * np.pi * self.a ** 2 * r)

    def enclosed_mass(self, r):
        x = np.asarray(r, dtype=np.float64) / self.a
        return self.mass * (1.0 - (1.0 + x) * np.exp(-x))

    def potential(self, r):
        r = np.asarray(r, dtype=np.float64)
        x = r / self.a
        return -self.mass * (-np.expm1(-x)) / r

    def dpotential(self, r):
        r = np.asarray(r, dtype=np.float64)
        x = r / self.a
        # d/dr[-(1-e^{-x})/r] = (1-e^{-x})/r^2 - e^{-x}/(a r)
        return self.mass * ((-np.expm1(-x)) / r ** 2 - np.exp(-x) / (self.a * r))
