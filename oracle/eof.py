"""Oracle: cylindrical EOF expansion (``exptool/basis/eof.py``), vectorised
over particles.  TEST INFRASTRUCTURE (see package docstring)."""
from __future__ import annotations

import numpy as np

from .sl import r_to_xi


def z_to_y(z, hscale):
    """``compatibility.z_to_y`` (``compatibility.py:83-91``)."""
    return (z / (np.abs(z) + 1.0e-8)) * np.arcsinh(np.abs(z / hscale))


def eof_params(path):
    """Old-style header of ``eof.eof_params`` (``eof.py:163-181``)."""
    with open(path, "rb") as f:
        a = np.fromfile(f, dtype="<u4", count=7)
        b = np.fromfile(f, dtype="<f8", count=6)
    mmax, numx, numy, nmax, norder, dens, cmap = (int(v) for v in a)
    rmin, rmax, ascale, hscale, cylmass, tnow = (float(v) for v in b)
    return rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens


def parse_eof(path):
    """``eof.parse_eof`` (``eof.py:224-313``), old-style header: returns
    potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS."""
    rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof_params(path)
    shape = (mmax + 1, norder, numx + 1, numy + 1)
    arrs = [np.zeros(shape) for _ in range(8)]
    nb = (numx + 1) * (numy + 1)
    with open(path, "rb") as f:
        f.seek(76)
        for part, m0 in ((0, 0), (4, 1)):
            for i in range(m0, mmax + 1):
                for j in range(norder):
                    for k in range(4 if dens == 1 else 3):
                        arrs[part + k][i, j] = np.fromfile(f, dtype="<f8", count=nb).reshape(numx + 1, numy + 1)
    return tuple(arrs)


def set_table_params(RMAX=20.0, RMIN=0.001, ASCALE=0.01, HSCALE=0.001, NUMX=128, NUMY=64, CMAP=0):
    """``eof.set_table_params`` (``eof.py:316-347``)."""
    Rtable = np.sqrt(0.5) * RMAX
    XMIN = float(r_to_xi(RMIN * ASCALE, CMAP, ASCALE))
    XMAX = float(r_to_xi(Rtable * ASCALE, CMAP, ASCALE))
    dX = (XMAX - XMIN) / NUMX
    YMIN = float(z_to_y(-Rtable * ASCALE, HSCALE))
    YMAX = float(z_to_y(Rtable * ASCALE, HSCALE))
    dY = (YMAX - YMIN) / NUMY
    return XMIN, XMAX, dX, YMIN, YMAX, dY


def return_bins(r, z, rmin=0, dR=0, zmin=0, dZ=0, numx=0, numy=0, ASCALE=0.01, HSCALE=0.001, CMAP=0):
    """``eof.return_bins`` (``eof.py:354-427``).  Lower clamps set ix, X (and
    iy, Y) to 0; the upper clamps set only ix (iy) — the X (Y) assignment that
    follows tests the already-clamped index and never fires, so X > numx-1 is
    linearly extrapolated."""
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    z = np.atleast_1d(np.asarray(z, dtype=np.float64))
    X = (r_to_xi(r, CMAP, ASCALE) - rmin) / dR
    Y = (z_to_y(z, HSCALE) - zmin) / dZ
    with np.errstate(invalid="ignore"):
        ix = np.trunc(X)
        iy = np.trunc(Y)
    ix = np.where(np.isfinite(ix), ix, 0).astype(np.int64)
    iy = np.where(np.isfinite(iy), iy, 0).astype(np.int64)
    ix = np.where(ix < 0, 0, ix)
    X = np.where(X < 0, 0.0, X)
    ix = np.where(ix >= numx, numx - 1, ix)
    iy = np.where(iy < 0, 0, iy)
    Y = np.where(Y < 0, 0.0, Y)
    iy = np.where(iy >= numy, numy - 1, iy)
    return X, Y, ix, iy


def _weights(X, Y, ix, iy):
    delx0 = ix + 1.0 - X
    dely0 = iy + 1.0 - Y
    delx1 = X - ix
    dely1 = Y - iy
    return delx0 * dely0, delx1 * dely0, delx0 * dely1, delx1 * dely1


def _interp(T, ix, iy, c):
    """Bilinear gather of T[..., ix(+1), iy(+1)] -> (..., N) (``eof.py:430-457``)."""
    c00, c10, c01, c11 = c
    return T[..., ix, iy] * c00 + T[..., ix + 1, iy] * c10 + T[..., ix, iy + 1] * c01 + T[..., ix + 1, iy + 1] * c11


def accumulate(x, y, z, mass, potC, potS, MMAX, NMAX, XMIN, dX, YMIN, dY, NUMX, NUMY, ASCALE, HSCALE, CMAP,
               chunk=65536):
    """``eof.accumulate`` (``eof.py:492-640``) without the VAR branch:
    returns (accum_cos, accum_sin), each (MMAX+1, NMAX).  The ``no_odd`` mask
    the reference builds is never applied (:544-549), so it is not an input."""
    norm = -4.0 * np.pi
    acc_c = np.zeros((MMAX + 1, NMAX))
    acc_s = np.zeros((MMAX + 1, NMAX))
    mo = np.arange(0.0, MMAX + 1.0)
    for s in range(0, x.size, chunk):
        sl = slice(s, s + chunk)
        r = (x[sl] ** 2.0 + y[sl] ** 2.0 + 1.0e-10) ** 0.5
        phi = np.arctan2(y[sl], x[sl])
        X, Y, ix, iy = return_bins(r, z[sl], XMIN, dX, YMIN, dY, NUMX, NUMY, ASCALE, HSCALE, CMAP)
        c = _weights(X, Y, ix, iy)
        vc = _interp(potC[:MMAX + 1, :NMAX], ix, iy, c) * mass[sl]
        vs = _interp(potS[:MMAX + 1, :NMAX], ix, iy, c) * mass[sl]
        ang = phi[None, :] * mo[:, None]
        acc_c += np.sum((norm * np.cos(ang))[:, None, :] * vc, axis=2)
        acc_s += np.sum((norm * np.sin(ang))[:, None, :] * vs, axis=2)
    return acc_c, acc_s


def accumulated_eval_particles(x, y, z, accum_cos, accum_sin, potC, rforceC, zforceC, potS, rforceS, zforceS,
                               rmin, dR, zmin, dZ, numx, numy, MMAX, NMAX, ASCALE, HSCALE, CMAP,
                               m1=0, m2=1000, densC=None, densS=None, chunk=32768):
    """``eof.accumulated_eval_particles`` (``eof.py:989-1144``): returns
    p0, p, fr, fp, fz, R (with densities: p0, p, d0, d, fr, fp, fz, R).  The
    m = 0 potential (and density) moves to p0 (d0) and p (d) restarts (:1128-1138)."""
    n = x.size
    R = (x * x + y * y + 1.0e-10) ** 0.5
    PHI = np.arctan2(y, x)
    density = densC is not None
    outs = {k: np.zeros(n) for k in ("p0", "p", "fr", "fp", "fz", "d0", "d")}
    for s in range(0, n, chunk):
        sl = slice(s, s + chunk)
        X, Y, ix, iy = return_bins(R[sl], z[sl], rmin, dR, zmin, dZ, numx, numy, ASCALE, HSCALE, CMAP)
        c = _weights(X, Y, ix, iy)
        phi = PHI[sl]
        p = np.zeros(phi.size)
        fr, fp, fz, d = np.zeros_like(p), np.zeros_like(p), np.zeros_like(p), np.zeros_like(p)
        p0 = np.zeros_like(p)
        d0 = np.zeros_like(p)
        for mm in range(MMAX + 1):
            if mm > m2 or mm < m1:
                continue
            ccos = np.cos(phi * mm)
            ssin = np.sin(phi * mm)
            fac = accum_cos[mm][:, None] * ccos
            pc = _interp(potC[mm, :NMAX], ix, iy, c)
            p += np.sum(fac * pc, axis=0)
            fr += np.sum(fac * _interp(rforceC[mm, :NMAX], ix, iy, c), axis=0)
            fz += np.sum(fac * _interp(zforceC[mm, :NMAX], ix, iy, c), axis=0)
            if density:
                d += np.sum(fac * _interp(densC[mm, :NMAX], ix, iy, c), axis=0)
            fac = accum_cos[mm][:, None] * ssin
            fp += np.sum(fac * mm * pc, axis=0)
            if mm > 0:
                fac = accum_sin[mm][:, None] * ssin
                ps = _interp(potS[mm, :NMAX], ix, iy, c)
                p += np.sum(fac * ps, axis=0)
                fr += np.sum(fac * _interp(rforceS[mm, :NMAX], ix, iy, c), axis=0)
                fz += np.sum(fac * _interp(zforceS[mm, :NMAX], ix, iy, c), axis=0)
                if density:
                    d += np.sum(fac * _interp(densS[mm, :NMAX], ix, iy, c), axis=0)
                fac = -accum_sin[mm][:, None] * ccos
                fp += np.sum(fac * mm * ps, axis=0)
            if mm == 0:
                p0 = p.copy()
                p[:] = 0.0
                if density:
                    d0 = d.copy()
                    d[:] = 0.0
        for k, v in (("p0", p0), ("p", p), ("fr", fr), ("fp", fp), ("fz", fz), ("d0", d0), ("d", d)):
            outs[k][sl] = v
    if density:
        return outs["p0"], outs["p"], outs["d0"], outs["d"], outs["fr"], outs["fp"], outs["fz"], R
    return outs["p0"], outs["p"], outs["fr"], outs["fp"], outs["fz"], R


def force_eval(r, z, phi, accum_cos, accum_sin, potC, rforceC, zforceC, potS, rforceS, zforceS,
               rmin=0, dR=0, zmin=0, dZ=0, numx=0, numy=0, MMAX=6, NMAX=18, ASCALE=0.0, HSCALE=0.0, CMAP=0,
               no_odd=False, perturb=False):
    """``eof.force_eval`` (``eof.py:756-870``), vectorised over points.  The odd-m
    mask is |cos(pi/2 m)| (about 6e-17 for odd m, not 0), as in :822-826.
    Returns (fr+fr0, fp, fz+fz0, p+p0, p0), or with perturb
    (fr, fp, fz, p, p0, fr0, fz0)."""
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    z = np.atleast_1d(np.asarray(z, dtype=np.float64))
    phi = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    ac = accum_cos[:MMAX + 1, :NMAX]
    as_ = accum_sin[:MMAX + 1, :NMAX]
    X, Y, ix, iy = return_bins(r, z, rmin, dR, zmin, dZ, numx, numy, ASCALE, HSCALE, CMAP)
    c = _weights(X, Y, ix, iy)
    morder = np.arange(1.0, MMAX + 1.0)[:, None, None]           # (MMAX, 1, 1)
    ccos = np.cos(phi[None, None, :] * morder)
    ssin = np.sin(phi[None, None, :] * morder)
    mask = np.abs(np.cos((np.pi / 2.0) * morder)) if no_odd else np.ones_like(morder)
    pC = _interp(potC[1:MMAX + 1, :NMAX], ix, iy, c)
    pS = _interp(potS[1:MMAX + 1, :NMAX], ix, iy, c)
    fac = ac[1:, :, None] * ccos
    p = np.sum(mask * fac * pC, axis=(0, 1))
    fr = np.sum(mask * fac * _interp(rforceC[1:MMAX + 1, :NMAX], ix, iy, c), axis=(0, 1))
    fz = np.sum(mask * fac * _interp(zforceC[1:MMAX + 1, :NMAX], ix, iy, c), axis=(0, 1))
    p0 = np.sum(ac[0][:, None] * _interp(potC[0, :NMAX], ix, iy, c), axis=0)
    fr0 = np.sum(ac[0][:, None] * _interp(rforceC[0, :NMAX], ix, iy, c), axis=0)
    fz0 = np.sum(ac[0][:, None] * _interp(zforceC[0, :NMAX], ix, iy, c), axis=0)
    fac = ac[1:, :, None] * ssin
    fp = np.sum(mask * fac * morder * pC, axis=(0, 1))
    fac = as_[1:, :, None] * ssin
    p = p + np.sum(mask * fac * pS, axis=(0, 1))
    fr = fr + np.sum(mask * fac * _interp(rforceS[1:MMAX + 1, :NMAX], ix, iy, c), axis=(0, 1))
    fz = fz + np.sum(mask * fac * _interp(zforceS[1:MMAX + 1, :NMAX], ix, iy, c), axis=(0, 1))
    fac = -as_[1:, :, None] * ccos
    fp = fp + np.sum(mask * fac * morder * pS, axis=(0, 1))
    if perturb:
        return fr, fp, fz, p, p0, fr0, fz0
    return fr + fr0, fp, fz + fz0, p + p0, p0


def accumulated_eval(r, z, phi, accum_cos, accum_sin, potC, rforceC, zforceC, densC, potS, rforceS, zforceS,
                     densS, rmin=0, dR=0, zmin=0, dZ=0, numx=0, numy=0, MMAX=6, NMAX=18, ASCALE=0.0,
                     HSCALE=0.0, CMAP=0, no_odd=False):
    """``eof.accumulated_eval`` (``eof.py:874-929``), vectorised over points:
    returns p0, p, fr, fp, fz, d0, d with p, d the totals over m."""
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    z = np.atleast_1d(np.asarray(z, dtype=np.float64))
    phi = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    X, Y, ix, iy = return_bins(r, z, rmin, dR, zmin, dZ, numx, numy, ASCALE, HSCALE, CMAP)
    c = _weights(X, Y, ix, iy)
    n = r.size
    p, fr, fz, fp, d = (np.zeros(n) for _ in range(5))
    p0 = np.zeros(n)
    d0 = np.zeros(n)
    for mm in range(MMAX + 1):
        if (mm % 2) != 0 and no_odd:
            continue
        ccos = np.cos(phi * mm)
        ssin = np.sin(phi * mm)
        fac = accum_cos[mm][:, None] * ccos
        pc = _interp(potC[mm, :NMAX], ix, iy, c)
        p += np.sum(fac * pc, axis=0)
        fr += np.sum(fac * _interp(rforceC[mm, :NMAX], ix, iy, c), axis=0)
        fz += np.sum(fac * _interp(zforceC[mm, :NMAX], ix, iy, c), axis=0)
        d += np.sum(fac * _interp(densC[mm, :NMAX], ix, iy, c), axis=0)
        fac = accum_cos[mm][:, None] * ssin
        fp += np.sum(fac * mm * pc, axis=0)
        if mm > 0:
            fac = accum_sin[mm][:, None] * ssin
            ps = _interp(potS[mm, :NMAX], ix, iy, c)
            p += np.sum(fac * ps, axis=0)
            fr += np.sum(fac * _interp(rforceS[mm, :NMAX], ix, iy, c), axis=0)
            fz += np.sum(fac * _interp(zforceS[mm, :NMAX], ix, iy, c), axis=0)
            d += np.sum(fac * _interp(densS[mm, :NMAX], ix, iy, c), axis=0)
            fac = -accum_sin[mm][:, None] * ccos
            fp += np.sum(fac * mm * ps, axis=0)
        if mm == 0:
            p0 = p.copy()
            d0 = d.copy()
    return p0, p, fr, fp, fz, d0, d


def load_table(path):
    """Parse an EOF cache into the dict used by the oracle tests."""
    potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS = parse_eof(path)
    rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof_params(path)
    XMIN, XMAX, dX, YMIN, YMAX, dY = set_table_params(RMAX=rmax, RMIN=rmin, ASCALE=ascale, HSCALE=hscale,
                                                      NUMX=numx, NUMY=numy, CMAP=cmap)
    return dict(potC=potC, rforceC=rforceC, zforceC=zforceC, densC=densC, potS=potS, rforceS=rforceS,
                zforceS=zforceS, densS=densS, rmin=rmin, rmax=rmax, numx=numx, numy=numy, mmax=mmax,
                norder=norder, ascale=ascale, hscale=hscale, cmap=cmap, dens=dens, XMIN=XMIN, XMAX=XMAX,
                dX=dX, YMIN=YMIN, YMAX=YMAX, dY=dY)
