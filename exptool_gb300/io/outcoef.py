"""EXP coefficient time series (``outcoef.*`` files) with the interface of
``exptool/io/outcoef.py``: ``OutCoef(filename)`` sets ``.basis``
('SphereSL' or 'Cylinder'), ``.T`` (times) and ``.coefs``:

* SphereSL: ``coefs[t, lm, n]``, lm unrolled l-major with (cos, sin) pairs
  for m > 0 (outcoef.py:264-336);
* Cylinder: ``coefs[t, cos/sin, m, n]``, sin of m = 0 zero (outcoef.py:339-411).

Four layouts, told apart as the reference does (outcoef.py:79-130):

* new SphereSL (first u32 202004386) and new Cylinder (202004387): per
  record the magic, a u32 length, a YAML header with at least time, lmax /
  mmax and nmax, then the coefficients (SphereSL: per n, (lmax+1)^2 values;
  Cylinder: per m, nmax cos values and, for m > 0, nmax sin values);
* old SphereSL (64-byte label containing 'Sphere SL'; then time, scale (f8),
  nmax, lmax (u32), then per n the (lmax+1)^2 values);
* old Cylinder (time (f8), mmax, nmax (u32), then per m cos and sin as above);
  old files hold as many whole records as fit in the file size.

Fixed-size layouts are read with one structured read of the whole file
instead of the reference's per-record loop; YAML headers go through
exptool_gb300.io.yaml_lite (PyYAML is not a dependency).
"""
from __future__ import annotations

import os
import struct

import numpy as np

from . import yaml_lite

MAGIC_SL = 202004386
MAGIC_CYL = 202004387


class EOF_Object(object):
    """Carrier of one cylindrical coefficient set (outcoef.py:27-38)."""
    time = None
    dump = None
    comp = None
    nbodies = None
    mmax = None
    nmax = None
    eof_file = None
    cos = None
    sin = None


def _cyl_order(mmax, nmax):
    """Gather indices: (2, mmax+1, nmax) coefficient -> offset in a record's
    value block (per m: cos, then sin for m > 0), or -1 for sin of m = 0."""
    idx = -np.ones((2, mmax + 1, nmax), dtype=np.int64)
    at = 0
    for m in range(mmax + 1):
        idx[0, m] = np.arange(at, at + nmax)
        at += nmax
        if m > 0:
            idx[1, m] = np.arange(at, at + nmax)
            at += nmax
    return idx


def _gather_cyl(vals, mmax, nmax):
    idx = _cyl_order(mmax, nmax)
    out = np.zeros((vals.shape[0], 2, mmax + 1, nmax))
    ok = idx >= 0
    out[:, ok] = vals[:, idx[ok]]
    return out


def read_old_cylinder(path):
    """Old Cylinder layout (outcoef.py:134-196; eof.py:2230-2293)."""
    size = os.path.getsize(path)
    with open(path, "rb") as f:
        head = f.read(16)
    _t, mmax, nmax = struct.unpack("<dII", head)
    nval = (2 * mmax + 1) * nmax
    rec = np.dtype([("t", "<f8"), ("mmax", "<u4"), ("nmax", "<u4"), ("v", "<f8", (nval,))])
    nout = int(size / (8 * nval + 4 * 2 + 8))
    data = np.fromfile(path, dtype=rec, count=nout)
    return data["t"].astype(np.float64), _gather_cyl(data["v"].reshape(nout, nval), mmax, nmax)


def read_old_spheresl(path):
    """Old SphereSL layout (outcoef.py:199-261; spheresl.py:1636-1696)."""
    size = os.path.getsize(path)
    with open(path, "rb") as f:
        head = f.read(64 + 16 + 8)
    _time, _scale, nmax, lmax = struct.unpack("<ddII", head[64:88])
    nlm = lmax * (lmax + 2) + 1
    rec = np.dtype([("label", "S64"), ("t", "<f8"), ("scale", "<f8"), ("nmax", "<u4"), ("lmax", "<u4"),
                    ("v", "<f8", (nmax, nlm))])
    nout = int(size / (8 * nlm * nmax + 4 * 2 + 8 * 2 + 64))
    data = np.fromfile(path, dtype=rec, count=nout)
    return data["t"].astype(np.float64), np.ascontiguousarray(np.transpose(data["v"], (0, 2, 1)))


def _yaml_records(path, spherical):
    """(header dict, value offset) of each record of a new-style file."""
    buf = np.fromfile(path, dtype=np.uint8)
    pos, out = 0, []
    while pos < buf.size:
        _magic, nlen = struct.unpack_from("<II", buf, pos)
        text = bytes(buf[pos + 8:pos + 8 + nlen]).split(b"\x00")[0].decode()
        D = yaml_lite.load(text)
        out.append((D, pos + 8 + nlen))
        if spherical:
            nval = (D["lmax"] * (D["lmax"] + 2) + 1) * D["nmax"]
        else:
            nval = (2 * D["mmax"] + 1) * D["nmax"]
        pos = pos + 8 + nlen + 8 * nval
    return buf, out


def read_new_spheresl(path):
    """New SphereSL layout (outcoef.py:264-336)."""
    buf, recs = _yaml_records(path, True)
    if not recs:
        return np.zeros(0), np.zeros((0, 1, 0))
    L, N = recs[0][0]["lmax"], recs[0][0]["nmax"]
    nlm = L * (L + 2) + 1
    T = np.array([D["time"] for D, _o in recs], dtype=np.float64)
    coefs = np.zeros((len(recs), nlm, N))
    for t, (D, off) in enumerate(recs):
        v = np.frombuffer(buf, dtype="<f8", count=nlm * D["nmax"], offset=off).reshape(D["nmax"], nlm)
        coefs[t, :, :D["nmax"]] = v.T
    return T, coefs


def read_new_cylinder(path):
    """New Cylinder layout (outcoef.py:339-411)."""
    buf, recs = _yaml_records(path, False)
    if not recs:
        return np.zeros(0), np.zeros((0, 2, 1, 0))
    M, N = recs[0][0]["mmax"], recs[0][0]["nmax"]
    T = np.array([D["time"] for D, _o in recs], dtype=np.float64)
    coefs = np.zeros((len(recs), 2, M + 1, N))
    for t, (D, off) in enumerate(recs):
        nval = (2 * D["mmax"] + 1) * D["nmax"]
        v = np.frombuffer(buf, dtype="<f8", count=nval, offset=off)[None, :]
        coefs[t] = _gather_cyl(v, D["mmax"], D["nmax"])[0]
    return T, coefs


class OutCoef(object):
    """Reader of EXP coefficient time series (outcoef.py:41-537)."""

    def __init__(self, filename):
        self.coeffile = filename
        with open(filename, "rb") as f:
            head = f.read(64)
        (cmagic,) = struct.unpack("<I", head[:4])
        if cmagic == MAGIC_SL:
            self.basis = "SphereSL"
            print("OutCoef: reading SphereSL coefficients . . .")
            self.T, self.coefs = read_new_spheresl(filename)
        elif cmagic == MAGIC_CYL:
            self.basis = "Cylinder"
            print("OutCoef: reading Cylinder coefficients . . .")
            self.T, self.coefs = read_new_cylinder(filename)
        elif b"Sphere SL" in head:
            self.basis = "SphereSL"
            print("OutCoef: reading OLD SphereSL coefficients . . .")
            print("CAUION. These coefficients have a different normalisation scheme.")
            self.T, self.coefs = read_old_spheresl(filename)
        else:
            self.basis = "Cylinder"
            print("OutCoef: reading OLD Cylinder coefficients . . .")
            self.T, self.coefs = read_old_cylinder(filename)

    def _repackage_cylindrical_coefficients(self):
        """self.C[m]['cos'|'sin'][n] = time series (outcoef.py:414-441)."""
        _nt, _cs, numm, numn = self.coefs.shape
        self.C = {m: {c: {n: self.coefs[:, ic, m, n] for n in range(numn)} for ic, c in enumerate(["cos", "sin"])}
                  for m in range(numm)}

    def _repackage_cylindrical_coefficients_compatibility(self):
        """{time: EOF_Object} (outcoef.py:443-485)."""
        numt, _cs, numm, numn = self.coefs.shape
        out = {}
        for t in range(numt):
            E = EOF_Object()
            E.time = self.T[t]
            E.mmax = numm - 1
            E.nmax = numn
            E.filename = "[redacted]"
            E.comp = "star"
            E.nbodies = 0.0
            E.eof_file = "[redacted]"
            E.cos = np.array(self.coefs[t, 0])
            E.sin = np.array(self.coefs[t, 1])
            out[E.time] = E
        return out

    def _repackage_spherical_coefficients(self):
        """self.C[l][m]['cos'|'sin'][n] = time series (outcoef.py:487-537)."""
        _nt, numl2, numn = self.coefs.shape
        numl = int(np.sqrt(numl2))
        self.C = {}
        for l in range(numl):
            self.C[l] = {}
            for m in range(l + 1):
                if m > 0:
                    self.C[l][m] = {"cos": {n: self.coefs[:, l * l + 2 * m - 1, n] for n in range(numn)},
                                    "sin": {n: self.coefs[:, l * l + 2 * m, n] for n in range(numn)}}
                else:
                    self.C[l][m] = {"cos": {n: self.coefs[:, l * l, n] for n in range(numn)}}


class CylCoefs(object):
    """outcoef.CylCoefs (outcoef.py:540-589).  The reference stores the time
    array in ``numt`` and its ``normalise`` / ``total_order_*`` then fail;
    here ``numt`` is the same time array and the three methods use the
    number of times and the read coefficients."""

    def __init__(self, filename):
        self.CylCoefs = OutCoef(filename)
        self.numt = self.CylCoefs.T
        self.mmax = self.CylCoefs.coefs.shape[2]
        self.norder = self.CylCoefs.coefs.shape[3]

    def normalise(self):
        c = self.CylCoefs.coefs
        self.CylNormCoefs = c / c[:, 0, 0, 0][:, None, None, None]

    def total_order_power(self):
        c = self.CylCoefs.coefs
        return np.sum(c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1], axis=2)

    def total_order_amplitude(self):
        return np.sqrt(self.total_order_power())


# ------------------------------------------------------------------ writers
def write_new_spheresl(path, times, coefs, extra=None):
    """New SphereSL file from coefs[t, lm, n]."""
    nt, nlm, N = coefs.shape
    L = int(round(np.sqrt(nlm))) - 1
    with open(path, "wb") as f:
        for t in range(nt):
            head = f"lmax: {L}\nnmax: {N}\ntime: {float(times[t]):.17e}\n" + "".join(
                f"{k}: {v}\n" for k, v in (extra or {}).items())
            hb = head.encode()
            f.write(struct.pack("<II", MAGIC_SL, len(hb)))
            f.write(hb)
            f.write(np.ascontiguousarray(coefs[t].T, dtype="<f8").tobytes())


def write_new_cylinder(path, times, coefs, extra=None):
    """New Cylinder file from coefs[t, cos/sin, m, n]."""
    nt, _cs, M1, N = coefs.shape
    idx = _cyl_order(M1 - 1, N)
    with open(path, "wb") as f:
        for t in range(nt):
            head = f"mmax: {M1 - 1}\nnmax: {N}\ntime: {float(times[t]):.17e}\n" + "".join(
                f"{k}: {v}\n" for k, v in (extra or {}).items())
            hb = head.encode()
            f.write(struct.pack("<II", MAGIC_CYL, len(hb)))
            f.write(hb)
            v = np.zeros((2 * M1 - 1) * N)
            ok = idx >= 0
            v[idx[ok]] = coefs[t][ok]
            f.write(v.astype("<f8").tobytes())


def write_old_spheresl(path, times, coefs, scale=1.0, label=b"Sphere SL"):
    nt, nlm, N = coefs.shape
    L = int(round(np.sqrt(nlm))) - 1
    with open(path, "wb") as f:
        for t in range(nt):
            f.write(label.ljust(64, b"\x00")[:64])
            f.write(struct.pack("<ddII", float(times[t]), scale, N, L))
            f.write(np.ascontiguousarray(coefs[t].T, dtype="<f8").tobytes())


def write_old_cylinder(path, times, coefs):
    nt, _cs, M1, N = coefs.shape
    idx = _cyl_order(M1 - 1, N)
    with open(path, "wb") as f:
        for t in range(nt):
            f.write(struct.pack("<dII", float(times[t]), M1 - 1, N))
            v = np.zeros((2 * M1 - 1) * N)
            ok = idx >= 0
            v[idx[ok]] = coefs[t][ok]
            f.write(v.astype("<f8").tobytes())
