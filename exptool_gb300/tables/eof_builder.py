"""Cylindrical empirical-orthogonal-function (EOF) basis builder.

exptool reads EmpCylSL cache files (``exptool/basis/eof.py:98-313``) but notes
that they "are currently constructed elsewhere" (``eof.py:94-95``).  This module
constructs them in the same spirit as EmpCylSL:

1. a spherical Sturm-Liouville basis Phi_nl(r) Y_lm with a high lmax is built
   for a Hernquist background of scale ``ascale`` (its power-law envelope keeps
   the SL weight well scaled out to the table edge, which an exponential
   profile does not);
2. for each azimuthal order m the second-moment matrix
   C_ij = sum_p m_p psi_i(x_p) psi_j(x_p) of those functions over a seeded disc
   sample is diagonalised; the ``norder`` leading eigenvectors define the EOFs;
3. potential, -dPhi/dR, -dPhi/dz and density of each EOF are tabulated on the
   mapped (X, Y) grid that ``eof.set_table_params`` (``eof.py:316-347``)
   defines, and written in the old-style 76-byte-header layout
   (``eof.py:163-181, 261-308``).

Two engines build the same tables.  ``engine="gpu"`` (the default) evaluates
every basis function at the sample and at the table nodes with one CUDA kernel
per m (``xt_eof_basis``: Legendre recurrence, spline of u_nl(ln r), forces and
density in FP64) and forms the second-moment matrix and the tabulation as FP64
products on the device; only the small symmetric eigenproblems and the spline
coefficients are computed on the host.  ``engine="numpy"`` is the host
restatement, kept as the reference the GPU engine is tested against.

Force tables hold forces (``rforce = -dPhi/dR``, ``zforce = -dPhi/dz``): the sign
``potential.Fields.return_forces_cart`` assumes (``potential.py:487-494``).  The
angular factor is the same ``factorial_return`` normalisation the spherical code
uses (``spheresl.py:823-863``), so the reference's -4 pi accumulation factor is
the biorthogonality constant of these tables too.  Sine tables equal the cosine
tables for m >= 1 (the disc is axisymmetric).  Only even (l - m) terms enter,
so every EOF is even in z.
"""
from __future__ import annotations

import struct

import numpy as np
from scipy.special import gammaln

from .models import TruncatedHernquist
from .samplers import disc_cylindrical
from .sl_solver import SLBasis


def _factorial(lmax):
    f = np.zeros((lmax + 1, lmax + 1))
    for l in range(lmax + 1):
        for m in range(l + 1):
            f[l, m] = np.sqrt((0.5 * l + 0.25) / np.pi * np.exp(gammaln(1.0 + l - m) - gammaln(1.0 + l + m)))
            if m:
                f[l, m] *= np.sqrt(2.0)
    return f


def _legendre_m(lmax, m, c):
    """Normalised fact_lm P_l^m(c) and its theta derivative for l = m..lmax.

    Uses the normalised three-term recurrence (stable for large l) with the
    Condon-Shortley phase, the convention of ``spheresl.legendre_R``
    (``spheresl.py:664-700``).  Returns arrays of shape (lmax+1, len(c)); rows
    l < m are zero.
    """
    c = np.asarray(c, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, (1.0 - c) * (1.0 + c)))
    nl = lmax + 2
    Y = np.zeros((nl + 1, c.size))
    # normalised sectoral term  N_mm P_mm, N_lm = sqrt((2l+1)/(4pi) (l-m)!/(l+m)!)
    ymm = np.full(c.size, np.sqrt(1.0 / (4.0 * np.pi)))
    for k in range(1, m + 1):
        ymm = -np.sqrt((2.0 * k + 1.0) / (2.0 * k)) * s * ymm
    Y[m] = ymm
    if m + 1 <= nl:
        Y[m + 1] = np.sqrt(2.0 * m + 3.0) * c * ymm
    for l in range(m + 2, nl + 1):
        a = np.sqrt((4.0 * l * l - 1.0) / (l * l - m * m))
        b = np.sqrt(((l - 1.0) ** 2 - m * m) / (4.0 * (l - 1.0) ** 2 - 1.0))
        Y[l] = a * (c * Y[l - 1] - b * Y[l - 2])
    if m > 0:
        Y *= np.sqrt(2.0)
    # theta derivative from  sin(t) dP_l^m/dt = l c P_l^m - (l+m) P_{l-1}^m
    # written for normalised functions: dY_l/dt = [l c Y_l - sqrt((2l+1)/(2l-1) (l^2-m^2)) Y_{l-1}] / s
    dY = np.zeros_like(Y)
    safe = s > 1e-12
    for l in range(m, nl):
        prev = Y[l - 1] if l - 1 >= m else np.zeros(c.size)
        coef = np.sqrt((2.0 * l + 1.0) / (2.0 * l - 1.0) * (l * l - m * m)) if l > m else 0.0
        num = l * c * Y[l] - coef * prev
        dY[l] = np.where(safe, num / np.where(safe, s, 1.0), 0.0)
    return Y[: lmax + 1], dY[: lmax + 1]


def table_grid(numx, numy, rmin, rmax, ascale, hscale, cmap):
    """Node coordinates (R, z) of the (numx+1) x (numy+1) table, following
    ``eof.set_table_params`` (``eof.py:316-347``) for the abscissae."""
    rtable = np.sqrt(0.5) * rmax

    def r_to_xi(r):
        if cmap == 1:
            return (r / ascale - 1.0) / (r / ascale + 1.0)
        if cmap == 2:
            return np.log(r)
        return r

    def z_to_y(z):
        return (z / (np.abs(z) + 1.0e-8)) * np.arcsinh(np.abs(z / hscale))

    xmin = r_to_xi(rmin * ascale)
    xmax = r_to_xi(rtable * ascale)
    dx = (xmax - xmin) / numx
    ymin = z_to_y(-rtable * ascale)
    ymax = z_to_y(rtable * ascale)
    dy = (ymax - ymin) / numy
    X = xmin + dx * np.arange(numx + 1)
    Y = ymin + dy * np.arange(numy + 1)
    if cmap == 1:
        R = (1.0 + X) / (1.0 - X) * ascale
    elif cmap == 2:
        R = np.exp(X)
    else:
        R = X
    z = hscale * np.sinh(Y)
    return R, z


class EOFTables:
    """Built EOF tables: arrays (mmax+1, norder, numx+1, numy+1)."""

    def __init__(self, mmax=6, norder=18, numx=256, numy=256, rmin=0.001, rmax=30.0,
                 ascale=1.0, hscale=0.1, cmap=1, lmax_sph=32, nmax_sph=14,
                 nsample=100000, seed=12345, disc_h=0.1, disc_rmax=20.0, disc_zmax=2.0, engine="gpu"):
        if engine not in ("gpu", "numpy"):
            raise ValueError(f"engine must be 'gpu' or 'numpy', not {engine!r}")
        self.mmax, self.norder, self.numx, self.numy = mmax, norder, numx, numy
        self.rmin, self.rmax, self.ascale, self.hscale, self.cmap = rmin, rmax, ascale, hscale, cmap
        r_lo = 0.5 * rmin * ascale
        r_hi = 1.05 * rmax * ascale
        model = TruncatedHernquist(a=ascale, rtrunc=r_hi)
        self.sl = SLBasis(model, lmax_sph, nmax_sph, r_lo, r_hi, nfine=12001)
        Rn, zn = table_grid(numx, numy, rmin, rmax, ascale, hscale, cmap)
        RR, ZZ = np.meshgrid(Rn, zn, indexing="ij")
        Rs, zs, _ = disc_cylindrical(nsample, seed, a=ascale, h=disc_h, rmax=disc_rmax, zmax=disc_zmax)
        shape = (mmax + 1, norder, numx + 1, numy + 1)
        self.pot = np.zeros(shape)
        self.rforce = np.zeros(shape)
        self.zforce = np.zeros(shape)
        self.dens = np.zeros(shape)
        self.eigvals = np.zeros((mmax + 1, norder))
        nodes_R = RR.ravel()
        nodes_z = ZZ.ravel()
        if engine == "gpu":
            self._build_gpu(nodes_R, nodes_z, Rs, zs, lmax_sph, nsample)
            return
        cache_nodes = self._radial_cache(nodes_R, nodes_z, lmax_sph)
        cache_samp = self._radial_cache(Rs, zs, lmax_sph)
        for m in range(mmax + 1):
            psi_s, _, _, _ = self._functions(m, cache_samp, lmax_sph, need_derivs=False)
            C = psi_s @ psi_s.T / nsample
            V = self._eigvecs(m, C)
            psi_n, dR_n, dz_n, rho_n = self._functions(m, cache_nodes, lmax_sph, need_derivs=True)
            V = self._orient(V, V.T @ psi_n)
            self.pot[m] = (V.T @ psi_n).reshape(norder, numx + 1, numy + 1)
            self.rforce[m] = (-(V.T @ dR_n)).reshape(norder, numx + 1, numy + 1)
            self.zforce[m] = (-(V.T @ dz_n)).reshape(norder, numx + 1, numy + 1)
            self.dens[m] = (V.T @ rho_n).reshape(norder, numx + 1, numy + 1)

    def _eigvecs(self, m, C):
        """The norder leading eigenvectors of the second-moment matrix
        (columns), eigenvalues kept in self.eigvals[m]."""
        w, V = np.linalg.eigh(C)
        order = np.argsort(w)[::-1][:self.norder]
        self.eigvals[m] = w[order]
        return V[:, order]

    def _orient(self, V, pot):
        """Deterministic sign: the potential of each EOF at the midplane node
        of largest magnitude is negative."""
        V = V.copy()
        for k in range(self.norder):
            ref = np.asarray(pot[k]).reshape(self.numx + 1, self.numy + 1)[:, (self.numy + 1) // 2]
            j = int(np.argmax(np.abs(ref)))
            if ref[j] > 0:
                V[:, k] = -V[:, k]
        return V

    def _build_gpu(self, nodes_R, nodes_z, Rs, zs, lmax, nsample):
        """Basis functions by the xt_eof_basis kernel, second moments and
        tabulation as FP64 products on the device."""
        import torch
        from scipy.interpolate import CubicSpline
        from .. import _lib, device as dev
        lib = _lib.load()
        sl = self.sl
        knots = dev.to_dev(sl.t)
        nseg = sl.t.size - 1
        coef = np.empty((lmax + 1, nseg, sl.nmax, 4))
        for l in range(lmax + 1):
            coef[l] = np.transpose(CubicSpline(sl.t, sl.u[l], axis=1).c, (1, 2, 0))
        coef_d = dev.to_dev(coef)
        ise = dev.to_dev(1.0 / np.sqrt(sl.ev[:lmax + 1]))
        se = dev.to_dev(np.sqrt(sl.ev[:lmax + 1]))

        def points(R, z):
            r = np.maximum(np.sqrt(R * R + z * z), sl.rmin)
            return [dev.to_dev(a) for a in (R, z, sl.model.potential(r), sl.model.dpotential(r),
                                             sl.model.density(r))]

        P_n, P_s = points(nodes_R, nodes_z), points(Rs, zs)
        norder, nx, ny = self.norder, self.numx + 1, self.numy + 1

        def basis(m, P, derivs):
            nf = ((lmax - m) // 2 + 1) * sl.nmax
            npt = P[0].numel()
            outs = [torch.empty((nf, npt), dtype=torch.float64, device=P[0].device) for _ in range(4 if derivs else 1)]
            ptr = [dev.dptr(o) for o in outs] + [None] * (4 - len(outs))
            _lib.check(lib.xt_eof_basis(m, lmax, sl.nmax, nseg, dev.dptr(knots), dev.dptr(coef_d), dev.dptr(ise),
                                        dev.dptr(se), *(dev.dptr(a) for a in P), float(sl.rmin), npt,
                                        int(bool(derivs)), *ptr, dev.stream_ptr()), "xt_eof_basis")
            return outs

        for m in range(self.mmax + 1):
            (psi_s,) = basis(m, P_s, False)
            C = dev.to_host(psi_s @ psi_s.T / nsample)
            del psi_s
            V = self._eigvecs(m, C)
            psi_n, dR_n, dz_n, rho_n = basis(m, P_n, True)
            Vt = dev.to_dev(np.ascontiguousarray(V.T))
            V = self._orient(V, dev.to_host(Vt @ psi_n))
            Vt = dev.to_dev(np.ascontiguousarray(V.T))
            self.pot[m] = dev.to_host(Vt @ psi_n).reshape(norder, nx, ny)
            self.rforce[m] = (-dev.to_host(Vt @ dR_n)).reshape(norder, nx, ny)
            self.zforce[m] = (-dev.to_host(Vt @ dz_n)).reshape(norder, nx, ny)
            self.dens[m] = dev.to_host(Vt @ rho_n).reshape(norder, nx, ny)
            del psi_n, dR_n, dz_n, rho_n

    def _radial_cache(self, R, z, lmax):
        r = np.sqrt(R * R + z * z)
        r = np.maximum(r, self.sl.rmin)
        c = z / r
        pots, dpots, dens = [], [], []
        for l in range(lmax + 1):
            p, dp = self.sl.pot_and_dpot(l, r)
            pots.append(p)
            dpots.append(dp)
            dens.append(self.sl.dens(l, r))
        return dict(R=R, z=z, r=r, c=c, pot=pots, dpot=dpots, dens=dens)

    def _functions(self, m, cache, lmax, need_derivs):
        R, z, r, c = cache["R"], cache["z"], cache["r"], cache["c"]
        Y, dY = _legendre_m(lmax, m, c)
        psis, dRs, dzs, rhos = [], [], [], []
        for l in range(m, lmax + 1, 2):
            p = cache["pot"][l]
            psis.append(p * Y[l])
            if need_derivs:
                dp = cache["dpot"][l]
                # d/dR and d/dz of Phi(r) Y(theta): dr/dR = R/r, dtheta/dR = z/r^2,
                # dr/dz = z/r, dtheta/dz = -R/r^2
                dRs.append(dp * (R / r) * Y[l] + p * dY[l] * (z / r ** 2))
                dzs.append(dp * (z / r) * Y[l] - p * dY[l] * (R / r ** 2))
                rhos.append(cache["dens"][l] * Y[l])
        psi = np.concatenate(psis, axis=0)
        if not need_derivs:
            return psi, None, None, None
        return (psi, np.concatenate(dRs, axis=0), np.concatenate(dzs, axis=0),
                np.concatenate(rhos, axis=0))

    def write(self, path, dens=True, tnow=0.0, cylmass=1.0):
        """Old-style EmpCylSL cache: 7 x uint32 (mmax numx numy nmax norder dens
        cmap), 6 x float64 (rmin rmax ascale hscale cylmass tnow), then for
        each m, n: pot, rforce, zforce[, dens] blocks of (numx+1)(numy+1)
        float64, cosine terms for m = 0..mmax then sine terms for m = 1..mmax."""
        with open(path, "wb") as f:
            f.write(struct.pack("<7I", self.mmax, self.numx, self.numy, self.norder,
                                self.norder, 1 if dens else 0, self.cmap))
            f.write(struct.pack("<6d", self.rmin, self.rmax, self.ascale, self.hscale,
                                cylmass, tnow))
            for part in ("cos", "sin"):
                m0 = 0 if part == "cos" else 1
                for m in range(m0, self.mmax + 1):
                    for n in range(self.norder):
                        blocks = [self.pot, self.rforce, self.zforce] + ([self.dens] if dens else [])
                        for arr in blocks:
                            f.write(np.ascontiguousarray(arr[m, n], dtype="<f8").tobytes())


def make_disc_eof(path, **kw):
    """Build and write an EOF cache for the exponential disc; returns tables."""
    dens = kw.pop("dens", True)
    t = EOFTables(**kw)
    t.write(path, dens=dens)
    return t
