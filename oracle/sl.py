"""Oracle: spherical Sturm-Liouville expansion (``exptool/basis/spheresl.py``,
``exptool/utils/halo_methods.py``, ``exptool/basis/compatibility.py``),
vectorised over particles.  TEST INFRASTRUCTURE (see package docstring)."""
from __future__ import annotations

import numpy as np
from scipy import interpolate
from scipy.special import gammaln


# ---------------------------------------------------------------- tables
def read_cached_table(path):
    """SL cache reader, layout of ``halo_methods.read_cached_table``
    (``halo_methods.py:96-169``)."""
    with open(path, "rb") as f:
        a = np.fromfile(f, dtype="<u4", count=4)
        lmax, nmax, numr, cmap = (int(v) for v in a)
        rmin, rmax, scale = (float(v) for v in np.fromfile(f, dtype="<f8", count=3))
        ltable = np.zeros(lmax + 1)
        ev = np.ones((lmax + 1, nmax))
        ef = np.ones((lmax + 1, nmax, numr))
        for l in range(lmax + 1):
            ltable[l] = np.fromfile(f, dtype="<u4", count=1)[0]
            ev[l] = np.fromfile(f, dtype="<f8", count=nmax)
            ef[l] = np.fromfile(f, dtype="<f8", count=nmax * numr).reshape(nmax, numr)
    return lmax, nmax, numr, cmap, rmin, rmax, scale, ltable, ev, ef


def init_table(modelfile, numr, rmin, rmax, cmap=0, scale=1.0):
    """``halo_methods.init_table`` (``halo_methods.py:178-220``) with the cmap=2
    ``log`` defect (:195) resolved to ``np.log``."""
    A = np.genfromtxt(modelfile, comments="!", skip_header=5)
    R1, D1, P1 = A[:, 0], A[:, 1], A[:, 3]
    fac0 = 4.0 * np.pi
    if cmap == 1:
        xmin = (rmin / scale - 1.0) / (rmin / scale + 1.0)
        xmax = (rmax / scale - 1.0) / (rmax / scale + 1.0)
    elif cmap == 2:
        xmin, xmax = np.log(rmin), np.log(rmax)
    else:
        xmin, xmax = rmin, rmax
    dxi = (xmax - xmin) / (numr - 1)
    pfunc = interpolate.splrep(R1, P1, s=0)
    dfunc = interpolate.splrep(R1, fac0 * D1, s=0)
    xi = np.array([xmin + dxi * i for i in range(numr)])
    r = xi_to_r(xi, cmap, scale)
    p0 = np.array([interpolate.splev(v, pfunc, der=0) for v in r], dtype=np.float64)
    d0 = np.array([interpolate.splev(v, dfunc, der=0) for v in r], dtype=np.float64)
    return xi, r, p0, d0


# ---------------------------------------------------------------- maps
def r_to_xi(r, cmap, scale):
    """``compatibility.r_to_xi`` (``compatibility.py:16-49``)."""
    r = np.asarray(r, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        if cmap == 1:
            out = (r / scale - 1.0) / (r / scale + 1.0)
        elif cmap == 2:
            out = np.log(r)
        else:
            out = r.copy()
    return np.where(r < 0.0, 0.0, out)


def xi_to_r(xi, cmap, scale):
    """``compatibility.xi_to_r`` (``compatibility.py:54-62``)."""
    if cmap == 1:
        return (1.0 + xi) / (1.0 - xi) * scale
    if cmap == 2:
        return np.exp(xi)
    return xi


def d_xi_to_r(xi, cmap, scale):
    """``compatibility.d_xi_to_r`` (``compatibility.py:65-80``)."""
    if cmap == 1:
        return 0.5 * (1.0 - xi) * (1.0 - xi) / scale
    if cmap == 2:
        return np.exp(-xi)
    return np.ones_like(xi)


# ---------------------------------------------------------------- Legendre
def legendre_R(lmax, x):
    """``spheresl.legendre_R`` (``spheresl.py:664-700``) for an array of x:
    returns (lmax+1, lmax+1, N); non-finite entries set to 0."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    p = np.zeros((lmax + 1, lmax + 1, x.size))
    p[0, 0] = 1.0
    pll = np.ones_like(x)
    with np.errstate(invalid="ignore", over="ignore"):
        if lmax > 0:
            somx2 = np.sqrt((1.0 - x) * (1.0 + x))
            fact = 1.0
            for m in range(1, lmax + 1):
                pll = pll * (-fact * somx2)
                p[m, m] = pll
                fact += 2.0
        for m in range(lmax):
            pl2 = p[m, m].copy()
            p[m + 1, m] = x * (2.0 * m + 1) * pl2
            pl1 = x * (2.0 * m + 1) * pl2
            for l in range(m + 2, lmax + 1):
                pll = (x * (2 * l - 1) * pl1 - (l + m - 1) * pl2) / (l - m)
                p[l, m] = pll
                pl2 = pl1
                pl1 = pll
    p[~np.isfinite(p)] = 0.0
    return p


def dlegendre_R(lmax, x):
    """``spheresl.dlegendre_R`` (``spheresl.py:706-770``): P and dP/dx with x
    clamped to +-(1-1e-8) for the derivative only."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    p = legendre_R(lmax, x)
    dp = np.zeros_like(p)
    MINEPS = 1.0e-8
    with np.errstate(invalid="ignore"):
        near = (1.0 - np.abs(x)) < MINEPS
    xc = np.where(near, np.where(x > 0, 1.0 - MINEPS, -(1.0 - MINEPS)), x)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        somx2 = 1.0 / (xc * xc - 1.0)
        for l in range(1, lmax + 1):
            for m in range(l):
                dp[l, m] = somx2 * (xc * l * p[l, m] - (l + m) * p[l - 1, m])
            dp[l, l] = somx2 * xc * l * p[l, l]
    dp[~np.isfinite(dp)] = 0.0
    return p, dp


def factorial_return(lmax):
    """``spheresl.factorial_return`` (``spheresl.py:823-863``)."""
    f = np.zeros((lmax + 1, lmax + 1))
    for l in range(lmax + 1):
        for m in range(l + 1):
            f[l, m] = np.sqrt((0.5 * l + 0.25) / np.pi * np.exp(gammaln(1.0 + l - m) - gammaln(1.0 + l + m)))
            if m != 0:
                f[l, m] *= np.sqrt(2.0)
    return f


# ---------------------------------------------------------------- radial functions
def _radial_bins(r, xi, cmap, scale, rmin, rmax, numr):
    """Mapping, clamp and index of ``get_halo_*`` (``spheresl.py:121-143``),
    with the cmap=2 bounds (undefined globals xmin/xmax at :128-130) taken as
    log(rmin), log(rmax)."""
    x = r_to_xi(r, cmap, scale)
    if cmap == 1:
        x = np.where(x < -1.0, -1.0, x)
        x = np.where(x >= 1.0, 1.0 - 1.0e-08, x)
    if cmap == 2:
        lo, hi = np.log(rmin), np.log(rmax)
        x = np.where(x < lo, lo, x)
        x = np.where(x > hi, hi, x)
    dxi = xi[1] - xi[0]
    with np.errstate(invalid="ignore"):
        indx = np.floor((x - np.min(xi)) / dxi)
    indx = np.where(np.isfinite(indx), indx, 0).astype(np.int64)
    indx = np.clip(indx, 0, numr - 2)
    x1 = (xi[indx + 1] - x) / dxi
    x2 = (x - xi[indx]) / dxi
    return x, indx, x1, x2, dxi


def halo_pot_matrix(r, lmax, nmax, ev, ef, xi, p0, cmap, scale, rmin, rmax):
    """``get_halo_pot_matrix`` (``spheresl.py:301-335``): (N, lmax+1, nmax)."""
    numr = p0.shape[0]
    x, i, x1, x2, _ = _radial_bins(np.atleast_1d(r), xi, cmap, scale, rmin, rmax, numr)
    e = ef[:lmax + 1, :nmax]
    sev = np.sqrt(ev[:lmax + 1, :nmax])
    efl = (x1[:, None, None] * np.moveaxis(e[:, :, i], 2, 0) + x2[:, None, None] * np.moveaxis(e[:, :, i + 1], 2, 0))
    return efl / sev * (x1 * p0[i] + x2 * p0[i + 1])[:, None, None]


def halo_dens_force_pot(r, lmax, nmax, ev, ef, xi, d0, p0, cmap, scale, rmin, rmax):
    """``get_halo_dens_pot_force`` (``spheresl.py:106-160``): returns
    (dens, force, pot), each (N, lmax+1, nmax).  For indx == 0 the force
    stencil uses rows 0,1,2 with the unshifted x2 (:147-150)."""
    numr = p0.shape[0]
    x, i, x1, x2, dxi = _radial_bins(np.atleast_1d(r), xi, cmap, scale, rmin, rmax, numr)
    fac = d_xi_to_r(x, cmap, scale) / dxi
    e = ef[:lmax + 1, :nmax]
    ev_ = ev[:lmax + 1, :nmax]
    sev = np.sqrt(ev_)

    def g(k):
        return np.moveaxis(e[:, :, k], 2, 0)

    X1, X2 = x1[:, None, None], x2[:, None, None]
    lerp = X1 * g(i) + X2 * g(i + 1)
    dens = lerp * sev * (x1 * d0[i] + x2 * d0[i + 1])[:, None, None]
    pot = lerp / sev * (x1 * p0[i] + x2 * p0[i + 1])[:, None, None]
    j = np.where(i == 0, 1, i)
    force = fac[:, None, None] * ((X2 - 0.5) * g(j - 1) * p0[j - 1][:, None, None]
                                  - 2.0 * X2 * g(j) * p0[j][:, None, None]
                                  + (X2 + 0.5) * g(j + 1) * p0[j + 1][:, None, None]) / sev
    return dens, force, pot


def _rows(lmax):
    """(l, m, row) of the expcoef layout: l-major, m = 0 one row, m > 0 a
    (cos, sin) pair (``spheresl.py:618-654``)."""
    out = []
    loff = 0
    for l in range(lmax + 1):
        moff = 0
        for m in range(l + 1):
            out.append((l, m, loff + moff))
            moff += 1 if m == 0 else 2
        loff += 2 * l + 1
    return out


# ---------------------------------------------------------------- accumulation
def compute_coefficients_solitary(x, y, z, mass, table, no_odd=False):
    """``compute_coefficients_solitary`` (``spheresl.py:567-656``), vectorised:
    returns expcoef ((lmax+1)^2, nmax)."""
    lmax, nmax, numr, cmap, rmin, rmax, scale, ev, ef, xi, p0 = (
        table[k] for k in ("lmax", "nmax", "numr", "cmap", "rmin", "rmax", "scale", "ev", "ef", "xi", "p0"))
    fac0 = -4.0 * np.pi
    r = np.sqrt(x * x + y * y + z * z)
    r = np.where(np.isnan(r) | (r < 1.0e-10), 1.0e-10, r)
    costh = z / r
    phi = np.arctan2(y, x)
    legs = legendre_R(lmax, costh)
    potd = halo_pot_matrix(r, lmax, nmax, ev, ef, xi, p0, cmap, scale, rmin, rmax)
    fact = factorial_return(lmax)
    ec = np.zeros((lmax * (lmax + 2) + 1, nmax))
    for l, m, row in _rows(lmax):
        if (l % 2) != 0 and no_odd:
            continue
        fac = fact[l, m] * legs[l, m]
        fac4 = potd[:, l, :] * (fac * fac0)[:, None]
        if m == 0:
            ec[row] = np.sum(fac4 * mass[:, None], axis=0)
        else:
            ec[row] = np.sum(np.cos(phi * m)[:, None] * fac4 * mass[:, None], axis=0)
            ec[row + 1] = np.sum(np.sin(phi * m)[:, None] * fac4 * mass[:, None], axis=0)
    return ec


# ---------------------------------------------------------------- evaluation
def all_eval_particles(x, y, z, expcoef, table, L1=-1000, L2=1000, NO_ODD=False):
    """``all_eval_particles`` (``spheresl.py:1240-1362``), vectorised.  Keeps the
    reference's den1 m = 0 factor ``legs[1][m]`` (:1323) and densfac 0.25*pi
    (:1351).  Returns den0, den1, pot0, pot1, potr, pott, potp, rr."""
    lmax, nmax = table["lmax"], table["nmax"]
    r = np.sqrt(x * x + y * y + z * z)
    rr = np.sqrt(x * x + y * y)
    phi = np.arctan2(y, x)
    with np.errstate(invalid="ignore", divide="ignore"):
        costh = z / r
    dend, dpot, potd = halo_dens_force_pot(r, lmax, nmax, table["ev"], table["ef"], table["xi"], table["d0"],
                                           table["p0"], table["cmap"], table["scale"], table["rmin"], table["rmax"])
    legs, dlegs = dlegendre_R(lmax, costh)
    fact = factorial_return(lmax)
    ec = expcoef
    f00 = fact[0, 0]
    den0 = np.sum(f00 * ec[0] * dend[:, 0, :], axis=1)
    pot0 = np.sum(f00 * ec[0] * potd[:, 0, :], axis=1)
    potr = np.sum(f00 * ec[0] * dpot[:, 0, :], axis=1)
    n = x.size
    den1, pot1, pott, potp = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n)
    for l, m, row in _rows(lmax):
        if l == 0:
            continue
        if l > L2 or l < L1:
            continue
        if NO_ODD and (l % 2) != 0:
            continue
        f = fact[l, m]
        if m == 0:
            den1 += np.sum(f * legs[1, m][:, None] * ec[row] * dend[:, l], axis=1)
            pot1 += np.sum(f * legs[l, m][:, None] * ec[row] * potd[:, l], axis=1)
            potr += np.sum(f * legs[l, m][:, None] * ec[row] * dpot[:, l], axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * ec[row] * potd[:, l], axis=1)
        else:
            cosm = np.cos(phi * m)[:, None]
            sinm = np.sin(phi * m)[:, None]
            ang = ec[row] * cosm + ec[row + 1] * sinm
            den1 += np.sum(f * legs[l, m][:, None] * dend[:, l] * ang, axis=1)
            pot1 += np.sum(f * legs[l, m][:, None] * potd[:, l] * ang, axis=1)
            potr += np.sum(f * legs[l, m][:, None] * dpot[:, l] * ang, axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * potd[:, l] * ang, axis=1)
            potp += np.sum(f * legs[l, m][:, None] * potd[:, l] * m * (-ec[row] * sinm + ec[row + 1] * cosm), axis=1)
    densfac = 0.25 * np.pi
    return den0 * densfac, den1 * densfac, pot0, pot1, potr, pott, potp, rr


def all_eval(r, costh, phi, expcoef, table, lmax=None, nmax=None, no_odd=False):
    """``all_eval`` (``spheresl.py:987-1102``), vectorised over points: den1
    includes the l = 0 density; densfac 0.25/pi.  lmax/nmax truncate the
    expansion (the reference's row truncation at :1019 keeps lmax+1 rows, which
    cannot index the l > 0 rows it then reads; (lmax+1)^2 rows are kept here)."""
    lmax = table["lmax"] if lmax is None else lmax
    nmax = table["nmax"] if nmax is None else nmax
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    costh = np.atleast_1d(np.asarray(costh, dtype=np.float64))
    phi = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    ec = expcoef[:(lmax + 1) ** 2, :nmax]
    dend, dpot, potd = halo_dens_force_pot(r, lmax, nmax, table["ev"], table["ef"], table["xi"], table["d0"],
                                           table["p0"], table["cmap"], table["scale"], table["rmin"], table["rmax"])
    legs, dlegs = dlegendre_R(lmax, costh)
    fact = factorial_return(lmax)
    f00 = fact[0, 0]
    den0 = np.sum(f00 * ec[0] * dend[:, 0], axis=1)
    pot0 = np.sum(f00 * ec[0] * potd[:, 0], axis=1)
    potr = np.sum(f00 * ec[0] * dpot[:, 0], axis=1)
    den1 = den0.copy()
    n = r.size
    pot1, pott, potp = np.zeros(n), np.zeros(n), np.zeros(n)
    for l, m, row in _rows(lmax):
        if l == 0 or ((l % 2) != 0 and no_odd):
            continue
        f = fact[l, m]
        if m == 0:
            den1 += np.sum(f * legs[l, m][:, None] * (ec[row] * dend[:, l]), axis=1)
            pot1 += np.sum(f * legs[l, m][:, None] * (ec[row] * potd[:, l]), axis=1)
            potr += np.sum(f * legs[l, m][:, None] * (ec[row] * dpot[:, l]), axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * (ec[row] * potd[:, l]), axis=1)
        else:
            cosm = np.cos(phi * m)[:, None]
            sinm = np.sin(phi * m)[:, None]
            den1 += np.sum(f * legs[l, m][:, None] * (ec[row] * dend[:, l] * cosm + ec[row + 1] * dend[:, l] * sinm), axis=1)
            pot1 += np.sum(f * legs[l, m][:, None] * (ec[row] * potd[:, l] * cosm + ec[row + 1] * potd[:, l] * sinm), axis=1)
            potr += np.sum(f * legs[l, m][:, None] * (ec[row] * dpot[:, l] * cosm + ec[row + 1] * dpot[:, l] * sinm), axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * (ec[row] * potd[:, l] * cosm + ec[row + 1] * potd[:, l] * sinm), axis=1)
            potp += np.sum(f * legs[l, m][:, None] * m * (-ec[row] * potd[:, l] * sinm + ec[row + 1] * potd[:, l] * cosm), axis=1)
    densfac = 0.25 / np.pi
    return den0 * densfac, den1 * densfac, pot0, pot1, potr, pott, potp


def force_eval(r, costh, phi, expcoef, table, lmax=None, nmax=None, no_odd=False, correct_m=False):
    """``force_eval`` (``spheresl.py:1107-1234``), vectorised over points.  The
    azimuthal factors are cos(l phi), sin(l phi) (row l of ``morder``,
    :1173,1185-1190,1222-1225) as in the reference; ``correct_m=True`` uses
    cos(m phi), sin(m phi) instead (the ``all_eval`` convention).  Returns
    potr, pott, potp, pot1, pot0."""
    lmax = table["lmax"] if lmax is None else lmax
    nmax = table["nmax"] if nmax is None else nmax
    r = np.atleast_1d(np.asarray(r, dtype=np.float64))
    costh = np.atleast_1d(np.asarray(costh, dtype=np.float64))
    phi = np.atleast_1d(np.asarray(phi, dtype=np.float64))
    ec = expcoef[:(lmax + 1) * (lmax + 1), :nmax]
    dend, dpot, potd = halo_dens_force_pot(r, lmax, nmax, table["ev"], table["ef"], table["xi"], table["d0"],
                                           table["p0"], table["cmap"], table["scale"], table["rmin"], table["rmax"])
    legs, dlegs = dlegendre_R(lmax, costh)
    fact = factorial_return(lmax)
    f00 = fact[0, 0]
    pot0 = np.sum(f00 * ec[0] * potd[:, 0], axis=1)
    potr = np.sum(f00 * ec[0] * dpot[:, 0], axis=1)
    n = r.size
    pot1, pott, potp = np.zeros(n), np.zeros(n), np.zeros(n)
    for l, m, row in _rows(lmax):
        if l == 0 or ((l % 2) != 0 and no_odd):
            continue
        f = fact[l, m]
        if m == 0:
            pot1 += np.sum(f * legs[l, m][:, None] * (ec[row] * potd[:, l]), axis=1)
            potr += np.sum(f * legs[l, m][:, None] * (ec[row] * dpot[:, l]), axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * (ec[row] * potd[:, l]), axis=1)
        else:
            k = m if correct_m else l
            cosm = np.cos(phi * k)[:, None]
            sinm = np.sin(phi * k)[:, None]
            pot1 += np.sum(f * legs[l, m][:, None] * (ec[row] * potd[:, l] * cosm + ec[row + 1] * potd[:, l] * sinm), axis=1)
            potr += np.sum(f * legs[l, m][:, None] * (ec[row] * dpot[:, l] * cosm + ec[row + 1] * dpot[:, l] * sinm), axis=1)
            pott += np.sum(f * dlegs[l, m][:, None] * (ec[row] * potd[:, l] * cosm + ec[row + 1] * potd[:, l] * sinm), axis=1)
            potp += np.sum(f * legs[l, m][:, None] * m * (-ec[row] * potd[:, l] * sinm + ec[row + 1] * potd[:, l] * cosm), axis=1)
    return potr, pott, potp, pot1, pot0


def load_table(sph_file, model_file):
    """Read an SL cache + model file into the dict the functions above take."""
    lmax, nmax, numr, cmap, rmin, rmax, scale, lt, ev, ef = read_cached_table(sph_file)
    xi, rarr, p0, d0 = init_table(model_file, numr, rmin, rmax, cmap, scale)
    return dict(lmax=lmax, nmax=nmax, numr=numr, cmap=cmap, rmin=rmin, rmax=rmax, scale=scale,
                ev=ev, ef=ef, xi=xi, p0=p0, d0=d0)
