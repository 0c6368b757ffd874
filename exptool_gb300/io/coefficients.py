"""Coefficient and field files of exptool, byte-compatible.

Three formats, each a leading int32 dump count followed by fixed-size
records (the layouts are the files' contract, so they match the reference
byte for byte; each record is read and written here as one NumPy structured
record):

* SL coefficients (spheresl.sl_coefficients_to_file / save_sl_coefficients /
  restore_sl_coefficients, spheresl.py:1390-1488): time f4, filename S100,
  comp S8, nbodies i4, sph_file S100, model_file S100, lmax i4, nmax i4,
  expcoef f8[(lmax+1)^2 * nmax]  (324-byte header).
* EOF coefficients (eof.eof_coefficients_to_file / save_eof_coefficients /
  restore_eof_coefficients, eof.py:1646-1760): time f4, filename S100,
  comp S8, nbodies i4, eof_file S100, mmax i4, nmax i4,
  cos f8[(mmax+1) nmax], sin f8[(mmax+1) nmax]  (224-byte header).
* A whole Fields instance (potential.Fields.save_field, potential.py:738-963,
  and potential.restore_field, :968-1042): one record, no dump count.
"""
from __future__ import annotations

import os
from collections import OrderedDict

import numpy as np


def _sl_dtype(lmax, nmax):
    return np.dtype([("time", "<f4"), ("filename", "S100"), ("comp", "S8"), ("nbodies", "<i4"),
                     ("sph_file", "S100"), ("model_file", "S100"), ("lmax", "<i4"), ("nmax", "<i4"),
                     ("expcoef", "<f8", ((lmax + 1) * (lmax + 1) * nmax,))])


def _eof_dtype(mmax, nmax):
    return np.dtype([("time", "<f4"), ("filename", "S100"), ("comp", "S8"), ("nbodies", "<i4"),
                     ("eof_file", "S100"), ("mmax", "<i4"), ("nmax", "<i4"),
                     ("cos", "<f8", ((mmax + 1) * nmax,)), ("sin", "<f8", ((mmax + 1) * nmax,))])


SL_HEADER = _sl_dtype(0, 0).itemsize              # 324 bytes before expcoef
EOF_HEADER = _eof_dtype(0, 0).itemsize            # 224 bytes before cos, sin


def _cv(v, dt):
    """Scalar converted exactly as np.array([v], dtype=dt) converts it (None
    becomes b'None' for strings and nan for floats, as in the reference files)."""
    return np.array([v], dtype=dt)[0]


def _append_record(path, rec, verbose=0, what=""):
    """Increment the leading dump count and write `rec` after the previous
    dumps (all dumps of a file have the same size)."""
    if not os.path.exists(path):
        with open(path, "wb") as f:
            np.array([0], dtype="<i4").tofile(f)
    with open(path, "rb+") as f:
        n = int(np.fromfile(f, dtype="<i4", count=1)[0]) + 1
        f.seek(0)
        np.array([n], dtype="<i4").tofile(f)
        if verbose:
            print(f"{what}: coefficient file currently has {n:d} dumps.")
        f.seek(4 + (n - 1) * rec.dtype.itemsize)
        rec.tofile(f)
    return n


# ---------------------------------------------------------------- SL
def sl_record(obj):
    lmax, nmax = int(obj.lmax), int(obj.nmax)
    rec = np.zeros(1, dtype=_sl_dtype(lmax, nmax))
    rec["time"] = _cv(obj.time, "<f4")
    rec["filename"] = _cv(getattr(obj, "filename", None), "S100")
    rec["comp"] = _cv(obj.comp, "S8")
    rec["nbodies"] = _cv(obj.nbodies, "<i4")
    rec["sph_file"] = _cv(obj.sph_file, "S100")
    rec["model_file"] = _cv(obj.model_file, "S100")
    rec["lmax"], rec["nmax"] = lmax, nmax
    rec["expcoef"][0] = np.asarray(obj.expcoef, dtype=np.float64).reshape(-1)
    return rec


def sl_coefficients_to_file(f, obj):
    """Write one SL dump at the current position of open file `f`."""
    sl_record(obj).tofile(f)


def save_sl_coefficients(outfile, obj, verbose=0):
    _append_record(outfile, sl_record(obj), verbose, "spheresl.save_sl_coefficients")


def extract_sl_coefficients(f, make):
    """Read one SL dump from open file `f` into a new `make()` object."""
    head = np.fromfile(f, dtype=_sl_dtype(0, 0), count=1)     # the 324-byte header
    if head.size != 1:
        raise EOFError("truncated SL coefficient file")
    lmax, nmax = int(head["lmax"][0]), int(head["nmax"][0])
    coef = np.fromfile(f, dtype="<f8", count=(lmax + 1) * (lmax + 1) * nmax)
    o = make()
    o.time = head["time"][0]
    o.filename, o.comp = head["filename"][0], head["comp"][0]
    o.nbodies = head["nbodies"][0]
    o.sph_file, o.model_file = head["sph_file"][0], head["model_file"][0]
    o.lmax, o.nmax = head["lmax"][0], head["nmax"][0]
    o.expcoef = coef.reshape((lmax + 1) * (lmax + 1), nmax)
    return o


def restore_sl_coefficients(infile, make):
    """(last dump, {round(time, 3): dump}) of an SL coefficient file."""
    with open(infile, "rb") as f:
        n = int(np.fromfile(f, dtype="<i4", count=1)[0])
        out, last = {}, None
        for _ in range(n):
            last = extract_sl_coefficients(f, make)
            out[np.round(last.time, 3)] = last
    return last, out


# ---------------------------------------------------------------- EOF
def eof_record(obj):
    mmax, nmax = int(obj.mmax), int(obj.nmax)
    rec = np.zeros(1, dtype=_eof_dtype(mmax, nmax))
    rec["time"] = _cv(obj.time, "<f4")
    rec["filename"] = _cv(getattr(obj, "filename", None), "S100")
    rec["comp"] = _cv(obj.comp, "S8")
    rec["nbodies"] = _cv(obj.nbodies, "<i4")
    rec["eof_file"] = _cv(obj.eof_file, "S100")
    rec["mmax"], rec["nmax"] = mmax, nmax
    rec["cos"][0] = np.asarray(obj.cos, dtype=np.float64).reshape(-1)
    rec["sin"][0] = np.asarray(obj.sin, dtype=np.float64).reshape(-1)
    return rec


def eof_coefficients_to_file(f, obj):
    eof_record(obj).tofile(f)


def save_eof_coefficients(outfile, obj, verbose=0):
    _append_record(outfile, eof_record(obj), verbose, "eof.save_eof_coefficients")


def extract_eof_coefficients(f, make):
    head = np.fromfile(f, dtype=_eof_dtype(0, 0), count=1)
    if head.size != 1:
        raise EOFError("truncated EOF coefficient file")
    mmax, nmax = int(head["mmax"][0]), int(head["nmax"][0])
    k = (mmax + 1) * nmax
    cs = np.fromfile(f, dtype="<f8", count=2 * k)
    if cs.size != 2 * k:
        raise EOFError("truncated EOF coefficient file")
    o = make()
    o.time = head["time"][0]
    o.filename, o.comp = head["filename"][0], head["comp"][0]
    o.nbodies = head["nbodies"][0]
    o.eof_file = head["eof_file"][0]
    o.mmax, o.nmax = head["mmax"][0], head["nmax"][0]
    o.cos = cs[:k].reshape(mmax + 1, nmax)
    o.sin = cs[k:].reshape(mmax + 1, nmax)
    return o


def restore_eof_coefficients(infile, make):
    """(last dump, OrderedDict{time: dump}); a truncated trailing dump is
    skipped, as the reference's per-dump try/except does."""
    with open(infile, "rb") as f:
        n = int(np.fromfile(f, dtype="<i4", count=1)[0])
        out, last = OrderedDict(), None
        for _ in range(n):
            try:
                o = extract_eof_coefficients(f, make)
            except EOFError:
                continue
            last = o
            out[o.time] = o
    return last, out


# ---------------------------------------------------------------- Fields
def _field_dtype(mmax, norder, numx, numy, numr, lmax, nmax):
    tab = (mmax + 1) * norder * (numx + 1) * (numy + 1)
    return np.dtype([
        ("files", "S100", (4,)), ("flags", "<i4", (6,)), ("time", "<f4"),
        ("eof_i", "<i4", (6,)), ("eof_f", "<f4", (11,)),
        ("cos", "<f8", ((mmax + 1) * norder,)), ("sin", "<f8", ((mmax + 1) * norder,)),
        ("potC", "<f8", (tab,)), ("rforceC", "<f8", (tab,)), ("zforceC", "<f8", (tab,)), ("densC", "<f8", (tab,)),
        ("potS", "<f8", (tab,)), ("rforceS", "<f8", (tab,)), ("zforceS", "<f8", (tab,)), ("densS", "<f8", (tab,)),
        ("sl_f", "<f4", (7,)), ("sl_i", "<i4", (4,)),
        ("xi", "<f8", (numr,)), ("p0", "<f8", (numr,)), ("d0", "<f8", (numr,)), ("ltable", "<f8", (lmax + 1,)),
        ("ev", "<f8", ((lmax + 1) * nmax,)), ("ef", "<f8", ((lmax + 1) * nmax * numr,)),
        ("expcoef", "<f8", ((lmax + 1) * (lmax + 1) * nmax,))])


def field_record(F):
    """One save_field record of a prepared Fields instance (tables and
    coefficients as the instance holds them)."""
    mmax, norder, numx, numy = int(F.mmax), int(F.norder), int(F.numx), int(F.numy)
    numr, lmax, nmax = int(F.numrhalo), int(F.lmaxhalo), int(F.nmaxhalo)
    rec = np.zeros(1, dtype=_field_dtype(mmax, norder, numx, numy, numr, lmax, nmax))
    rec["files"][0] = [_cv(v, "S100") for v in (F.filename, F.eof_file, F.sph_file, F.model_file)]
    rec["flags"][0] = [_cv(v, "<i4") for v in (F.nhalo, F.transform, F.no_odd, F.centering, F.mutual_center,
                                               F.verbose)]
    rec["time"] = _cv(getattr(F, "time", None), "<f4")
    rec["eof_i"][0] = [numx, numy, mmax, norder, int(F.cmapdisk), int(F.densdisk)]
    rec["eof_f"][0] = [F.rmindisk, F.rmaxdisk, F.ascale, F.hscale, F.XMIN, F.dX, F.YMIN, F.dY, F.xcen_disk,
                       F.ycen_disk, F.zcen_disk]
    rec["cos"][0] = np.asarray(F.EOF.cos, dtype=np.float64).reshape(-1)
    rec["sin"][0] = np.asarray(F.EOF.sin, dtype=np.float64).reshape(-1)
    for k in ("potC", "rforceC", "zforceC", "densC", "potS", "rforceS", "zforceS", "densS"):
        v = getattr(F, k)
        rec[k][0] = 0.0 if v is None else np.asarray(v, dtype=np.float64).reshape(-1)
    rec["sl_f"][0] = [F.halofac, F.rminhalo, F.rmaxhalo, F.scalehalo, F.xcen_halo, F.ycen_halo, F.zcen_halo]
    rec["sl_i"][0] = [numr, int(F.cmaphalo), lmax, nmax]
    rec["xi"][0], rec["p0"][0], rec["d0"][0] = F.xihalo, F.p0halo, F.d0halo
    rec["ltable"][0] = np.asarray(F.ltablehalo, dtype=np.float64).reshape(-1)
    rec["ev"][0] = np.asarray(F.evtablehalo, dtype=np.float64).reshape(-1)
    rec["ef"][0] = np.asarray(F.eftablehalo, dtype=np.float64).reshape(-1)
    rec["expcoef"][0] = np.asarray(F.SL.expcoef, dtype=np.float64).reshape(-1)
    return rec


def read_field_record(filename):
    """The single record of a save_field file, sized from its own headers."""
    with open(filename, "rb") as f:
        head = np.fromfile(f, dtype=[("files", "S100", (4,)), ("flags", "<i4", (6,)), ("time", "<f4"),
                                     ("eof_i", "<i4", (6,))], count=1)
        numx, numy, mmax, norder = (int(v) for v in head["eof_i"][0][:4])
        tab = (mmax + 1) * norder * (numx + 1) * (numy + 1)
        off = head.dtype.itemsize + 11 * 4 + 2 * (mmax + 1) * norder * 8 + 8 * tab * 8 + 7 * 4
        f.seek(off)
        numr, cmap, lmax, nmax = (int(v) for v in np.fromfile(f, dtype="<i4", count=4))
        f.seek(0)
        rec = np.fromfile(f, dtype=_field_dtype(mmax, norder, numx, numy, numr, lmax, nmax), count=1)
    if rec.size != 1:
        raise EOFError("truncated field file")
    return rec[0]
