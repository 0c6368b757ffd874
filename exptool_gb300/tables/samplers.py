"""Seeded synthetic particle samplers for the spherical and disc workloads.

All draws use ``numpy.random.default_rng(seed)`` (PCG64) in a fixed order so
the GPU path and the oracle consume identical arrays.
"""
from __future__ import annotations

import numpy as np


def hernquist_sample(n: int, seed: int, a: float = 1.0, rmax: float = 100.0,
                     mass_total: float = 1.0):
    """Hernquist sphere truncated at r < rmax, equal masses mass_total/n.

    Draw order: u ~ U[0, u_max) with u_max = (rmax/(rmax+a))^2 (exact truncation,
    no rejection), r = a sqrt(u)/(1 - sqrt(u)); then cos(theta) ~ U[-1, 1];
    then phi ~ U[0, 2 pi).  Returns x, y, z, m as float64 arrays.
    """
    rng = np.random.default_rng(seed)
    umax = (rmax / (rmax + a)) ** 2
    u = rng.uniform(0.0, umax, n)
    su = np.sqrt(u)
    r = a * su / (1.0 - su)
    c = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - c * c))
    x = r * s * np.cos(phi)
    y = r * s * np.sin(phi)
    z = r * c
    m = np.full(n, mass_total / max(n, 1))
    return x, y, z, m


def _invert_exp_cdf(u):
    """Solve 1 - (1+x) e^-x = u for x by Newton iteration (vectorised)."""
    x = np.where(u < 0.5, np.sqrt(2.0 * u), -np.log1p(-u) + 1.0)
    for _ in range(80):
        f = 1.0 - (1.0 + x) * np.exp(-x) - u
        fp = x * np.exp(-x)
        step = f / np.maximum(fp, 1e-300)
        x = np.maximum(x - step, 1e-12)
        if np.max(np.abs(step), initial=0.0) < 1e-15 * max(1.0, float(np.max(x, initial=1.0))):
            break
    return x


def disc_cylindrical(n: int, seed: int, a: float = 1.0, h: float = 0.1,
                     rmax: float = 20.0, zmax: float = 2.0):
    """Exponential disc (surface density ~ e^{-R/a}, sech^2(z/h) layers)
    truncated at R < rmax, |z| < zmax.

    Draw order: u ~ U[0, u_max) and R solves 1-(1+R/a)e^{-R/a} = u; then
    v ~ U(-tanh(zmax/h), tanh(zmax/h)) and z = h artanh(v); then phi ~ U[0, 2pi).
    Returns R, z, phi.
    """
    rng = np.random.default_rng(seed)
    umax = 1.0 - (1.0 + rmax / a) * np.exp(-rmax / a)
    u = rng.uniform(0.0, umax, n)
    R = _invert_exp_cdf(u) * a
    vmax = np.tanh(zmax / h)
    v = rng.uniform(-vmax, vmax, n)
    z = h * np.arctanh(v)
    phi = rng.uniform(0.0, 2.0 * np.pi, n)
    return R, z, phi


def disc_sample(n: int, seed: int, a: float = 1.0, h: float = 0.1, rmax: float = 20.0,
                zmax: float = 2.0, mass_total: float = 1.0):
    """Cartesian x, y, z, m of :func:`disc_cylindrical` with equal masses."""
    R, z, phi = disc_cylindrical(n, seed, a, h, rmax, zmax)
    return R * np.cos(phi), R * np.sin(phi), z, np.full(n, mass_total / max(n, 1))
