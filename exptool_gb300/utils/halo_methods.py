"""SL cache / model-table readers with the interface of
``exptool/utils/halo_methods.py``.

Host-side file parsing and the FITPACK spline set-up of the model table; the
results are uploaded once per table to the GPU by ``exptool_gb300.device``.
"""
from __future__ import annotations

import numpy as np
from scipy import interpolate

from ..basis.compatibility import xi_to_r


def read_sph_model_table(modelfile):
    """``R D M P`` columns after five header lines (halo_methods.py:56-62)."""
    A = np.genfromtxt(modelfile, comments="!", skip_header=5)
    return A[:, 0], A[:, 1], A[:, 2], A[:, 3]


def parse_slgrid(file, verbose=0):
    """Header of an SL cache (halo_methods.py:65-93)."""
    with open(file, "rb") as f:
        a = np.fromfile(f, dtype="<u4", count=4)
        b = np.fromfile(f, dtype="<f8", count=3)
    lmax, nmax, numr, cmap = (int(v) for v in a)
    rmin, rmax, scale = (float(v) for v in b)
    if verbose > 0:
        print("LMAX=", lmax, "NMAX=", nmax, "NUMR=", numr, "CMAP=", cmap, "RMIN=", rmin, "RMAX=", rmax,
              "SCALE=", scale)
    return lmax, nmax, numr, cmap, rmin, rmax, scale


def read_cached_table(file, verbose=0, retall=True):
    """SL cache reader (halo_methods.py:96-169): uint32 lmax nmax numr cmap,
    float64 rmin rmax scale, then per l: uint32 l, nmax eigenvalues and
    nmax x numr eigenfunction samples."""
    with open(file, "rb") as f:
        a = np.fromfile(f, dtype="<u4", count=4)
        if a.size != 4:
            raise ValueError(f"{file}: truncated SL cache header")
        lmax, nmax, numr, cmap = (int(v) for v in a)
        b = np.fromfile(f, dtype="<f8", count=3)
        if b.size != 3:
            raise ValueError(f"{file}: truncated SL cache header")
        rmin, rmax, scale = (float(v) for v in b)
        ltable = np.zeros(lmax + 1)
        evtable = np.ones((lmax + 1, nmax))
        eftable = np.ones((lmax + 1, nmax, numr))
        for l in range(lmax + 1):
            lv = np.fromfile(f, dtype="<u4", count=1)
            ev = np.fromfile(f, dtype="<f8", count=nmax)
            ef = np.fromfile(f, dtype="<f8", count=nmax * numr)
            if lv.size != 1 or ev.size != nmax or ef.size != nmax * numr:
                raise ValueError(f"{file}: truncated SL cache at l={l}")
            ltable[l] = lv[0]
            evtable[l] = ev
            eftable[l] = ef.reshape(nmax, numr)
    if retall:
        return lmax, nmax, numr, cmap, rmin, rmax, scale, ltable, evtable, eftable
    return ltable, evtable, eftable


def init_table(modelfile, numr, rmin, rmax, cmap=0, scale=1.0, spline=True):
    """Model potential p0 and 4 pi rho0 d0 on the table abscissa
    (halo_methods.py:178-220); the cmap=2 branch uses ``np.log`` (the
    reference's bare ``log`` at :195 is undefined)."""
    R1, D1, M1, P1 = read_sph_model_table(modelfile)
    fac0 = 4.0 * np.pi
    if cmap == 1:
        xmin = (rmin / scale - 1.0) / (rmin / scale + 1.0)
        xmax = (rmax / scale - 1.0) / (rmax / scale + 1.0)
    elif cmap == 2:
        xmin, xmax = np.log(rmin), np.log(rmax)
    else:
        xmin, xmax = rmin, rmax
    dxi = (xmax - xmin) / (numr - 1)
    xi = np.array([xmin + dxi * i for i in range(numr)])
    r = np.asarray(xi_to_r(xi, cmap, scale), dtype=np.float64)
    if spline:
        pfunc = interpolate.splrep(R1, P1, s=0)
        dfunc = interpolate.splrep(R1, fac0 * D1, s=0)
        p0 = np.asarray(interpolate.splev(r, pfunc, der=0), dtype=np.float64)
        d0 = np.asarray(interpolate.splev(r, dfunc, der=0), dtype=np.float64)
    else:
        idx = np.array([np.abs(rv - R1).argmin() for rv in r])
        p0 = P1[idx].astype(np.float64)
        d0 = fac0 * D1[idx].astype(np.float64)
    return xi, r, p0, d0
