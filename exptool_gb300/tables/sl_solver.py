"""Sturm-Liouville spherical basis generator and SLGridSph cache writer.

exptool only *reads* SL basis tables (``exptool/utils/halo_methods.py:96-169``)
built elsewhere by EXP; this module builds them.  For a spherical background
(rho0, Phi0) the potential/density pairs are

    Phi_nl(r) = u_nl(r) Phi0(r) / sqrt(mu_nl),   4 pi rho_nl = u_nl 4 pi rho0 sqrt(mu_nl)

which is exactly how the reference consumes the table (``spheresl.py:106-160``:
pot = ef * p0 / sqrt(ev), dens = ef * sqrt(ev) * d0 with d0 = 4 pi rho0).  Putting
Phi_nl into Poisson's equation gives the self-adjoint problem

    -(p u')' + q u = mu w u,   p = r^2 Phi0^2,  w = -4 pi r^2 Phi0 rho0,
                               q = l(l+1) Phi0^2 + w

with Robin conditions from regularity at the centre (Phi_nl ~ r^l) and the
vacuum solution outside (Phi_nl ~ r^-(l+1)).  The problem is discretised with
linear finite elements in t = ln r (lumped mass), reduced to a symmetric
tridiagonal matrix, and the lowest ``nmax`` eigenpairs are taken.  The
normalisation is int w u_n u_m dr = delta_nm, which makes the pairs biorthogonal
in the sense int Phi_n 4 pi rho_m r^2 dr = -delta_nm, the convention under which
the reference's accumulation factor -4 pi (``spheresl.py:585``) is exact.

For l = 0 the lowest eigenfunction is u = const with mu = 1 (Phi_00 is the
background itself); the test suite checks this.
"""
from __future__ import annotations

import os
import struct

import numpy as np
from scipy.interpolate import CubicSpline
from scipy.linalg import eigh_tridiagonal


class SLBasis:
    """Eigenfunctions u_nl on a fine ln r grid, with evaluation helpers."""

    def __init__(self, model, lmax: int, nmax: int, rmin: float, rmax: float,
                 nfine: int = 16001):
        self.model = model
        self.lmax = int(lmax)
        self.nmax = int(nmax)
        self.rmin = float(rmin)
        self.rmax = float(rmax)
        t = np.linspace(np.log(rmin), np.log(rmax), int(nfine))
        self.t = t
        h = t[1] - t[0]
        r = np.exp(t)
        phi = model.potential(r)
        rho = model.density(r)
        w_t = -4.0 * np.pi * r ** 3 * phi * rho          # W = r w  (weight in t)
        if np.any(w_t <= 0):
            raise ValueError("SL weight must be positive on [rmin, rmax]")
        rm = np.exp(0.5 * (t[1:] + t[:-1]))
        p_mid = rm * model.potential(rm) ** 2               # P = p / r at element midpoints
        hw = np.full(t.size, h)
        hw[0] = hw[-1] = 0.5 * h
        bdiag = w_t * hw
        p_a = r[0] * phi[0] ** 2
        p_b = r[-1] * phi[-1] ** 2
        g_a = r[0] * model.dpotential(r[0]) / phi[0]         # r Phi0'/Phi0
        g_b = r[-1] * model.dpotential(r[-1]) / phi[-1]

        self.ev = np.zeros((self.lmax + 1, self.nmax))
        self.u = np.zeros((self.lmax + 1, self.nmax, t.size))
        for l in range(self.lmax + 1):
            q_t = l * (l + 1) * r * phi ** 2 + w_t
            d = q_t * hw
            d[:-1] += p_mid / h
            d[1:] += p_mid / h
            e = -p_mid / h
            alpha_a = l - g_a
            alpha_b = -(l + 1) - g_b
            d[0] += p_a * alpha_a
            d[-1] -= p_b * alpha_b
            sb = np.sqrt(bdiag)
            cd = d / bdiag
            ce = e / (sb[:-1] * sb[1:])
            mu, y = eigh_tridiagonal(cd, ce, select="i",
                                     select_range=(0, self.nmax - 1))
            u = y / sb[:, None]
            for n in range(self.nmax):
                col = u[:, n]
                amax = np.max(np.abs(col))
                first = np.argmax(np.abs(col) > 0.1 * amax)
                if col[first] < 0:
                    u[:, n] = -col
            self.ev[l] = mu
            self.u[l] = u.T
        self._splines = {}

    def _spline(self, l):
        if l not in self._splines:
            self._splines[l] = CubicSpline(self.t, self.u[l], axis=1)
        return self._splines[l]

    def u_at(self, l, r):
        """u_nl(r) for all n: shape (nmax, len(r))."""
        return self._spline(l)(np.log(np.asarray(r, dtype=np.float64)))

    def pot_and_dpot(self, l, r):
        """Phi_nl(r) and dPhi_nl/dr for all n: each (nmax, len(r))."""
        r = np.asarray(r, dtype=np.float64)
        sp = self._spline(l)
        t = np.log(r)
        u = sp(t)
        du_dt = sp(t, 1)
        phi0 = self.model.potential(r)
        dphi0 = self.model.dpotential(r)
        inv = 1.0 / np.sqrt(self.ev[l])[:, None]
        pot = u * phi0 * inv
        dpot = (du_dt * phi0 / r + u * dphi0) * inv
        return pot, dpot

    def dens(self, l, r):
        """rho_nl(r) (true density, 4 pi rho = nabla^2 Phi): (nmax, len(r))."""
        r = np.asarray(r, dtype=np.float64)
        u = self._spline(l)(np.log(r))
        return u * self.model.density(r) * np.sqrt(self.ev[l])[:, None]


def xi_grid(numr: int, rmin: float, rmax: float, cmap: int, scale: float):
    """The table abscissa exactly as ``halo_methods.init_table`` forms it
    (``exptool/utils/halo_methods.py:186-212``): xi_i = xmin + dxi*i."""
    if cmap == 1:
        xmin = (rmin / scale - 1.0) / (rmin / scale + 1.0)
        xmax = (rmax / scale - 1.0) / (rmax / scale + 1.0)
    elif cmap == 2:
        xmin = np.log(rmin)
        xmax = np.log(rmax)
    else:
        xmin = rmin
        xmax = rmax
    dxi = (xmax - xmin) / (numr - 1)
    xi = np.array([xmin + dxi * i for i in range(numr)])
    if cmap == 1:
        r = (1.0 + xi) / (1.0 - xi) * scale
    elif cmap == 2:
        r = np.exp(xi)
    else:
        r = xi.copy()
    return xi, r


def write_model_file(path: str, model, rmin: float, rmax: float, npts: int = 4000,
                     title: str = "model"):
    """Write an ``R D M P`` model table with five header lines, the layout
    ``halo_methods.read_sph_model_table`` reads (``genfromtxt(comments='!',
    skip_header=5)``, ``exptool/utils/halo_methods.py:56-62``)."""
    r = np.geomspace(rmin, rmax, npts)
    d = model.density(r)
    m = model.enclosed_mass(r)
    p = model.potential(r)
    with open(path, "w") as f:
        f.write(f"! {title}\n")
        f.write("! columns: radius density enclosed_mass potential\n")
        f.write("! G = 1\n")
        f.write("!\n")
        f.write(f"{npts}\n")
        for row in zip(r, d, m, p):
            f.write("%.17e %.17e %.17e %.17e\n" % row)


def write_sl_cache(path: str, basis: SLBasis, numr: int, cmap: int, scale: float,
                   rmin: float | None = None, rmax: float | None = None):
    """Write an SLGridSph-layout cache (``halo_methods.py:132-162``): header
    uint32 lmax,nmax,numr,cmap; float64 rmin,rmax,scale; then per l: uint32 l,
    nmax eigenvalues, nmax x numr eigenfunction samples on the xi grid."""
    rmin = basis.rmin if rmin is None else rmin
    rmax = basis.rmax if rmax is None else rmax
    _, r = xi_grid(numr, rmin, rmax, cmap, scale)
    r = np.clip(r, basis.rmin, basis.rmax)
    with open(path, "wb") as f:
        f.write(struct.pack("<4I", basis.lmax, basis.nmax, numr, cmap))
        f.write(struct.pack("<3d", rmin, rmax, scale))
        for l in range(basis.lmax + 1):
            f.write(struct.pack("<I", l))
            f.write(np.asarray(basis.ev[l], dtype="<f8").tobytes())
            ef = basis.u_at(l, r)
            f.write(np.ascontiguousarray(ef, dtype="<f8").tobytes())


def make_hernquist_sl(directory: str, lmax: int = 4, nmax: int = 10, numr: int = 2000,
                      rmin: float = 1e-3, rmax: float = 100.0, cmap: int = 2,
                      scale: float = 1.0, a: float = 1.0, rtrunc: float = 100.0,
                      tag: str = "hernquist"):
    """Build a Hernquist SL basis and write ``SLGridSph.cache.<tag>`` and
    ``SLGridSph.model.<tag>`` into ``directory``; returns the two paths."""
    from .models import TruncatedHernquist
    os.makedirs(directory, exist_ok=True)
    model = TruncatedHernquist(a=a, rtrunc=rtrunc)
    basis = SLBasis(model, lmax, nmax, rmin, rmax)
    cache = os.path.join(directory, f"SLGridSph.cache.{tag}")
    modelf = os.path.join(directory, f"SLGridSph.model.{tag}")
    write_sl_cache(cache, basis, numr, cmap, scale)
    write_model_file(modelf, model, rmin * 0.5, rmax, title=f"truncated Hernquist a={a} rt={rtrunc}")
    return cache, modelf
