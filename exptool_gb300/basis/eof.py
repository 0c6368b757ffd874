"""Cylindrical EOF expansion on the GPU, with the call signatures of
``exptool/basis/eof.py``.

Cache parsing is host-side I/O; accumulation and evaluation run in the CUDA
library.  ``precision='f32'`` selects the mixed path.

Behaviour that differs from the reference where the reference cannot run:
* ``compute_coefficients`` moves particles with NaN positions to the origin
  (the reference intends this but fails at ``if nanvals > 0`` on numpy >= 2,
  eof.py:1194, and would edit ``.xpos`` while accumulating ``.data``);
* ``compute_forces`` / ``find_forces_multi`` honour m1/m2 and work for any
  ``nprocs`` (the reference's multi-process branch crashes, eof.py:1523).
"""
from __future__ import annotations

import os

import numpy as np
import torch

from .. import _lib
from .. import device as dev
from ..io.particle import positions
from .compatibility import r_to_xi, z_to_y


class EOF_Object(object):
    """Coefficient container (eof.py:1627-1636)."""
    time = None
    dump = None
    comp = None
    nbodies = None
    mmax = None
    nmax = None
    eof_file = None
    cos = None
    sin = None
    filename = None


# ---------------------------------------------------------------- cache files
HMAGIC = 0xC0A57A1


def eof_params(file, verbose=0):
    """Cache header (eof.py:98-200): returns rmin, rmax, numx, numy, mmax,
    norder, ascale, hscale, cmap, dens.  New-style (YAML) headers need PyYAML."""
    with open(file, "rb") as f:
        tmagic = np.fromfile(f, dtype="<i4", count=1)
        if tmagic.size == 1 and int(tmagic[0]) == HMAGIC:
            ssize = int(np.fromfile(f, dtype="<i4", count=1)[0])
            buf = f.read(ssize)
            try:
                import yaml
            except ImportError as e:
                raise RuntimeError("new-style EOF cache headers need PyYAML") from e
            data = yaml.safe_load(buf)
            cmap = data.get("cmap", data.get("cmapr"))
            vals = (data["rmin"], data["rmax"], data["numx"], data["numy"], data["mmax"], data["norder"],
                    data["ascl"], data["hscl"], cmap, data["dens"])
        else:
            f.seek(0)
            a = np.fromfile(f, dtype="<u4", count=7)
            b = np.fromfile(f, dtype="<f8", count=6)
            if a.size != 7 or b.size != 6:
                raise ValueError(f"{file}: truncated EOF cache header")
            mmax, numx, numy, nmax, norder, dens, cmap = (int(v) for v in a)
            rmin, rmax, ascale, hscale, cylmass, tnow = (float(v) for v in b)
            vals = (rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens)
    if verbose:
        print("eof.eof_params: RMIN={0},RMAX={1},NUMX={2},NUMY={3},MMAX={4},NORDER={5},ASCALE={6},HSCALE={7},"
              "CMAP={8},DENS={9}".format(*vals))
    return vals


def _data_offset(file):
    with open(file, "rb") as f:
        tmagic = np.fromfile(f, dtype="<i4", count=1)
        if tmagic.size == 1 and int(tmagic[0]) == HMAGIC:
            ssize = int(np.fromfile(f, dtype="<i4", count=1)[0])
            return 8 + ssize
    return 76


def parse_eof(file, verbose=0):
    """Cache tables (eof.py:224-313): potC, rforceC, zforceC, densC, potS,
    rforceS, zforceS, densS, each (mmax+1, norder, numx+1, numy+1)."""
    rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof_params(file, verbose=verbose)
    nb = (numx + 1) * (numy + 1)
    nblk = 4 if dens == 1 else 3
    raw = np.fromfile(file, dtype="<f8", offset=_data_offset(file))
    need = ((mmax + 1) + mmax) * norder * nblk * nb
    if raw.size < need:
        raise ValueError(f"{file}: truncated EOF cache ({raw.size} of {need} values)")
    shape = (mmax + 1, norder, numx + 1, numy + 1)
    out = [np.zeros(shape) for _ in range(8)]
    cosb = raw[:(mmax + 1) * norder * nblk * nb].reshape(mmax + 1, norder, nblk, numx + 1, numy + 1)
    sinb = raw[(mmax + 1) * norder * nblk * nb:need].reshape(mmax, norder, nblk, numx + 1, numy + 1)
    for k in range(3):
        out[k][:] = cosb[:, :, k]
        out[4 + k][1:] = sinb[:, :, k]
    if dens == 1:
        out[3][:] = cosb[:, :, 3]
        out[7][1:] = sinb[:, :, 3]
    return tuple(out)


def set_table_params(RMAX=20.0, RMIN=0.001, ASCALE=0.01, HSCALE=0.001, NUMX=128, NUMY=64, CMAP=0):
    """Scaled table bounds (eof.py:316-347): XMIN, XMAX, dX, YMIN, YMAX, dY."""
    Rtable = np.sqrt(0.5) * RMAX
    XMIN = float(r_to_xi(RMIN * ASCALE, CMAP, ASCALE))
    XMAX = float(r_to_xi(Rtable * ASCALE, CMAP, ASCALE))
    dX = (XMAX - XMIN) / NUMX
    YMIN = float(z_to_y(-Rtable * ASCALE, HSCALE))
    YMAX = float(z_to_y(Rtable * ASCALE, HSCALE))
    dY = (YMAX - YMIN) / NUMY
    return XMIN, XMAX, dX, YMIN, YMAX, dY


# ---------------------------------------------------------------- table caches
def table_from_file(eof_file) -> dev.CylTable:
    key = ("cyl-file", dev.file_key(eof_file))

    def make():
        tabs = parse_eof(eof_file)
        rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof_params(eof_file)
        XMIN, XMAX, dX, YMIN, YMAX, dY = set_table_params(RMAX=rmax, RMIN=rmin, ASCALE=ascale, HSCALE=hscale,
                                                          NUMX=numx, NUMY=numy, CMAP=cmap)
        return dev.CylTable(mmax, norder, numx, numy, cmap, dens, XMIN, dX, YMIN, dY, ascale, hscale, *tabs)

    return dev.TABLES.get(key, make)


def table_from_arrays(MMAX, NMAX, numx, numy, CMAP, XMIN, dX, YMIN, dY, ASCALE, HSCALE, potC, rforceC=None,
                      zforceC=None, potS=None, rforceS=None, zforceS=None, densC=None, densS=None) -> dev.CylTable:
    arrs = [potC, rforceC, zforceC, potS, rforceS, zforceS, densC, densS]
    present = tuple(a is not None for a in arrs)
    fp = dev.fingerprint(*[a for a in arrs if a is not None])
    key = ("cyl-arrays", fp, present, int(MMAX), int(NMAX), int(numx), int(numy), int(CMAP), float(XMIN), float(dX),
           float(YMIN), float(dY), float(ASCALE), float(HSCALE))

    def make():
        dens = densC is not None and densS is not None
        return dev.CylTable(MMAX, NMAX, numx, numy, CMAP, dens, XMIN, dX, YMIN, dY, ASCALE, HSCALE, potC, rforceC,
                            zforceC, densC if dens else None, potS, rforceS, zforceS, densS if dens else None)

    return dev.TABLES.get(key, make)


def field_for(table, cos, sin, mmax_use=-1, nmax_use=-1, density=False, precision="f64") -> dev.CylField:
    if isinstance(cos, torch.Tensor):
        return table.prepare(cos, sin, mmax_use, nmax_use, density, precision)
    c = np.asarray(cos, dtype=np.float64)
    s = np.asarray(sin, dtype=np.float64)
    key = (dev.fingerprint(c, s), int(mmax_use), int(nmax_use), bool(density), precision)
    return table.field_cache.get(key, lambda: table.prepare(c, s, mmax_use, nmax_use, density, precision))


# ---------------------------------------------------------------- accumulation
def accumulate(ParticleInstance, potC, potS, MMAX, NMAX, XMIN, dX, YMIN, dY, NUMX, NUMY, ASCALE, HSCALE, CMAP,
               verbose=0, no_odd=False, VAR=0, precision="f64"):
    """eof.accumulate (eof.py:492-640): returns (accum_cos, accum_sin), each
    (MMAX+1, NMAX).  ``no_odd`` is accepted and, as in the reference, not
    applied (its mask is never used, eof.py:544-549).  ``VAR`` sub-sampling
    (unseeded jackknife draws) is not supported."""
    if VAR:
        raise NotImplementedError("VAR jackknife partitions are not part of the GPU path")
    pC = np.asarray(potC)[:MMAX + 1, :NMAX]
    pS = np.asarray(potS)[:MMAX + 1, :NMAX]
    table = table_from_arrays(MMAX, NMAX, NUMX, NUMY, CMAP, XMIN, dX, YMIN, dY, ASCALE, HSCALE, pC, potS=pS)
    return _accumulate_host(table, positions(ParticleInstance, allow_device=True), precision, nan_to_origin=False)


def _accumulate_host(table, xyzm, precision, nan_to_origin):
    """(cos, sin) NumPy arrays: the sorted pipeline where the table fits it
    (particle arrays in page-locked host memory are read in place, and the
    last kernel writes the coefficients into page-locked memory), else the
    particle-order deposit and one copy out."""
    if table.sorted_ok():
        coef = table.accumulate_sorted(*(dev.kernel_input(a) for a in xyzm), precision=precision,
                                       nan_to_origin=nan_to_origin, host=True)
        return coef[0], coef[1]
    x, y, z, m = (dev.to_dev(a) for a in xyzm)
    if nan_to_origin:
        bad = torch.isnan(x) | torch.isnan(y) | torch.isnan(z)
        x, y, z = (torch.where(bad, torch.zeros_like(a), a) for a in (x, y, z))
    c, s = table.accumulate(x, y, z, m, precision=precision)
    return tuple(dev.fetch_many([c, s]))


def make_coefficients_multi(ParticleInstance, nprocs, potC, potS, mmax, norder, XMIN, dX, YMIN, dY, numx, numy,
                            ascale, hscale, cmap, verbose=0, no_odd=False, VAR=False, precision="f64"):
    """eof.make_coefficients_multi (eof.py:1415-1455): one GPU pass (nprocs is
    accepted for signature compatibility)."""
    return accumulate(ParticleInstance, potC, potS, mmax, norder, XMIN, dX, YMIN, dY, numx, numy, ascale, hscale,
                      cmap, verbose=verbose, no_odd=no_odd, VAR=VAR, precision=precision)


def compute_coefficients(PSPInput, eof_file, verbose=1, no_odd=False, nprocs_max=-1, VAR=False, nanblock=False,
                         precision="f64"):
    """eof.compute_coefficients (eof.py:1158-1260): returns an EOF_Object with
    .cos/.sin of shape (mmax+1, norder)."""
    if VAR:
        raise NotImplementedError("VAR jackknife partitions are not part of the GPU path")
    x, y, z, m = positions(PSPInput, allow_device=True)
    if verbose and not isinstance(x, torch.Tensor) and np.isnan(np.sum(x) + np.sum(y) + np.sum(z)):
        print("eof.compute_coefficients: NaN values found in output file {}.".format(getattr(PSPInput, "filename", "")))
    table = table_from_file(eof_file)
    out = EOF_Object()
    out.time = getattr(PSPInput, "time", None)
    out.filename = getattr(PSPInput, "filename", None)
    out.comp = getattr(PSPInput, "comp", None)
    out.nbodies = m.size
    out.eof_file = eof_file
    out.mmax = table.mmax
    out.nmax = table.norder
    # particles with a NaN coordinate are placed at the origin on the device
    # (eof.py:1189-1204) unless nanblock
    out.cos, out.sin = _accumulate_host(table, (x, y, z, m), precision, nan_to_origin=not nanblock)
    return out


def compute_coefficients_and_forces(PSPInput, eof_file, verbose=1, m1=0, m2=1000, nanblock=False, precision="f64"):
    """compute_coefficients followed by compute_forces on the same particles
    (eof.py:1158-1317) as one GPU pipeline: per-particle set-up is done once
    and particles are sorted by table cell on the device.  Returns
    (EOF_Object, (p0, p, fr, fp, fz, R)).  Particles with a NaN coordinate
    are placed at the origin (unless nanblock) for both passes."""
    x, y, z, m = positions(PSPInput, allow_device=True)
    n = int(m.numel()) if isinstance(m, torch.Tensor) else int(m.size)
    table = table_from_file(eof_file)
    # Particle arrays already on the device (snapshots read with device=True)
    # are used in place.  Particle arrays in page-locked host memory are read by the binning
    # kernel in place (the host -> device traffic overlaps its work); other
    # inputs are copied to the device first.  R is written by the binning
    # kernel straight into page-locked host memory; the other five results
    # are evaluated one part of the particles at a time and each part is
    # copied into page-locked host memory while the next is evaluated; the
    # coefficients follow in one copy, with one synchronisation.  Particles
    # with a NaN coordinate are placed at the origin on the device.
    # one page-locked block holds the coefficients, p0 p fr fp fz and R; the
    # returned arrays are views of it
    nc = (table.mmax + 1) * table.norder
    blk = torch.empty(2 * nc + 6 * n, dtype=torch.float64, pin_memory=True)
    base = blk.data_ptr()
    coef, _ = table.accumulate_eval_blocks(*(dev.kernel_input(a) for a in (x, y, z, m)), precision=precision,
                                           m1=m1, m2=m2, nan_to_origin=not nanblock,
                                           r_out=base + 8 * (2 * nc + 5 * n), res_out=base + 16 * nc)
    dev.copy_and_sync([(base, coef.data_ptr(), 16 * nc)])
    h = blk.numpy()
    host = [h[:nc].reshape(table.mmax + 1, table.norder), h[nc:2 * nc].reshape(table.mmax + 1, table.norder)]
    host += [h[2 * nc + k * n:2 * nc + (k + 1) * n] for k in range(6)]
    out = EOF_Object()
    out.time = getattr(PSPInput, "time", None)
    out.filename = getattr(PSPInput, "filename", None)
    out.comp = getattr(PSPInput, "comp", None)
    out.nbodies = n
    out.eof_file = eof_file
    out.mmax = table.mmax
    out.nmax = table.norder
    out.cos, out.sin = host[0], host[1]
    return out, tuple(host[2:])


# ---------------------------------------------------------------- evaluation
def accumulated_eval_particles(Particles, accum_cos, accum_sin, potC=0, rforceC=0, zforceC=0, potS=0, rforceS=0,
                               zforceS=0, rmin=0, dR=0, zmin=0, dZ=0, numx=0, numy=0, MMAX=6, NMAX=18, ASCALE=0.0,
                               HSCALE=0.0, CMAP=0, m1=0, m2=1000, verbose=1, density=False, eof_file="",
                               precision="f64"):
    """eof.accumulated_eval_particles (eof.py:989-1144): returns
    p0, p, fr, fp, fz, R (density: p0, p, d0, d, fr, fp, fz, R)."""
    if eof_file != "":
        table = table_from_file(eof_file)
    else:
        # the reference loops m <= MMAX over full coefficient rows (NMAX unused, eof.py:1093-1126)
        sl = (slice(0, int(MMAX) + 1),)
        nfull = np.asarray(potC).shape[1]
        table = table_from_arrays(MMAX, nfull, numx, numy, CMAP, rmin, dR, zmin, dZ, ASCALE, HSCALE,
                                  np.asarray(potC)[sl], np.asarray(rforceC)[sl], np.asarray(zforceC)[sl],
                                  np.asarray(potS)[sl], np.asarray(rforceS)[sl], np.asarray(zforceS)[sl])
        accum_cos = np.asarray(accum_cos)[sl]
        accum_sin = np.asarray(accum_sin)[sl]
    if density and not table.dens:
        if verbose > 0:
            print("eof.accumulated_eval_particles: cannot compute density (functions not specified). moving on "
                  "without...")
        density = False
    d = Particles.data
    zsrc = Particles.zpos if hasattr(Particles, "zpos") and Particles.zpos is not None else d["z"]
    if not density and table.sorted_ok():
        # binning, counting sort by table cell, field and evaluation in cell
        # order; particle arrays in page-locked host memory are read in place
        c, s = dev.coef_pair(accum_cos, accum_sin, table.mmax + 1, table.norder)
        n = int(np.asarray(d["x"]).size) if not isinstance(d["x"], torch.Tensor) else int(d["x"].numel())
        # one page-locked block for the results: R written into it by the
        # binning kernel, p0 p fr fp fz copied in part by part (3/8, 5/8 of
        # the particles) behind the evaluation; one wait
        blk = torch.empty(6 * n, dtype=torch.float64, pin_memory=True)
        table.eval_sorted(*(dev.kernel_input(a) for a in (d["x"], d["y"], zsrc)), c, s, precision=precision,
                          m1=m1, m2=m2, r_out=blk.data_ptr() + 40 * n, res_out=blk.data_ptr())
        dev.copy_and_sync([])
        h = blk.numpy()
        return tuple(h[k * n:(k + 1) * n] for k in range(6))
    field = field_for(table, accum_cos, accum_sin, density=density, precision=precision)
    x = dev.to_dev(d["x"])
    y = dev.to_dev(d["y"])
    z = dev.to_dev(zsrc)
    outs = table.eval_points(field, x, y, z, _lib.XT_CYL_ACCUMULATED_EVAL_PARTICLES, _lib.XT_COORD_CART, m1=m1, m2=m2,
                             want=[1, 1, 1, 1, 1, 1, int(density), int(density)])
    p0, p, fr, fp, fz, R, d0, dd = dev.to_host_many(list(outs))
    if density:
        return p0, p, d0, dd, fr, fp, fz, R
    return p0, p, fr, fp, fz, R


def compute_forces(PSPInput, EOF_Object, verbose=1, nprocs=-1, m1=0, m2=1000, density=False, precision="f64"):
    """eof.compute_forces (eof.py:1263-1317)."""
    return accumulated_eval_particles(PSPInput, EOF_Object.cos, EOF_Object.sin, m1=m1, m2=m2, verbose=verbose,
                                      density=density, eof_file=EOF_Object.eof_file, precision=precision)


def _pts(*vals):
    arrs = [np.atleast_1d(np.asarray(v, dtype=np.float64)) for v in vals]
    n = max(a.size for a in arrs)
    arrs = [np.broadcast_to(a, (n,)).copy() if a.size != n else a for a in arrs]
    return arrs, all(np.ndim(v) == 0 for v in vals)


def force_eval(r, z, phi, accum_cos, accum_sin, potC, rforceC, zforceC, potS, rforceS, zforceS, rmin=0, dR=0, zmin=0,
               dZ=0, numx=0, numy=0, fac=1.0, MMAX=6, NMAX=18, ASCALE=0.0, HSCALE=0.0, CMAP=0, no_odd=False,
               perturb=False, precision="f64"):
    """eof.force_eval (eof.py:756-870): returns (fr+fr0, fp, fz+fz0, p+p0, p0)
    or with perturb (fr, fp, fz, p, p0, fr0, fz0).  r, z, phi may be arrays."""
    MM = int(MMAX)
    NN = int(NMAX)
    full_m = np.asarray(potC).shape[0] - 1
    full_n = np.asarray(potC).shape[1]
    table = table_from_arrays(full_m, full_n, numx, numy, CMAP, rmin, dR, zmin, dZ, ASCALE, HSCALE, potC, rforceC,
                              zforceC, potS, rforceS, zforceS)
    field = field_for(table, accum_cos, accum_sin, mmax_use=min(MM, full_m), nmax_use=min(NN, full_n),
                      precision=precision)
    (ra, za, pa), scalar = _pts(r, z, phi)
    outs = table.eval_points(field, dev.to_dev(ra), dev.to_dev(za), dev.to_dev(pa), _lib.XT_CYL_FORCE_EVAL,
                             _lib.XT_COORD_CYL, mmax_use=min(MM, full_m), no_odd=no_odd, perturb=perturb)
    k = 7 if perturb else 5
    res = [dev.to_host(t) for t in outs[:k]]
    return tuple(float(v[0]) for v in res) if scalar else tuple(res)


def accumulated_eval(r, z, phi, accum_cos, accum_sin, potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS,
                     rmin=0, dR=0, zmin=0, dZ=0, numx=0, numy=0, fac=1.0, MMAX=6, NMAX=18, ASCALE=0.0, HSCALE=0.0,
                     CMAP=0, no_odd=False, precision="f64"):
    """eof.accumulated_eval (eof.py:874-929): returns p0, p, fr, fp, fz, d0, d
    (p and d summed over all m, p0 and d0 their m = 0 parts)."""
    # m <= MMAX over full coefficient rows, as eof.py:900-927 (NMAX unused)
    MM = int(MMAX)
    sl = (slice(0, MM + 1),)
    NN = np.asarray(potC).shape[1]
    table = table_from_arrays(MM, NN, numx, numy, CMAP, rmin, dR, zmin, dZ, ASCALE, HSCALE,
                              np.asarray(potC)[sl], np.asarray(rforceC)[sl], np.asarray(zforceC)[sl],
                              np.asarray(potS)[sl], np.asarray(rforceS)[sl], np.asarray(zforceS)[sl],
                              np.asarray(densC)[sl], np.asarray(densS)[sl])
    field = field_for(table, np.asarray(accum_cos)[sl], np.asarray(accum_sin)[sl], density=True,
                      precision=precision)
    (ra, za, pa), scalar = _pts(r, z, phi)
    outs = table.eval_points(field, dev.to_dev(ra), dev.to_dev(za), dev.to_dev(pa), _lib.XT_CYL_ACCUMULATED_EVAL,
                             _lib.XT_COORD_CYL, no_odd=no_odd)
    res = [dev.to_host(t) for t in outs[:7]]
    return tuple(float(v[0]) for v in res) if scalar else tuple(res)


# ---------------------------------------------------------------- coefficient files
def eof_coefficients_to_file(f, EOF_Object):
    """eof.eof_coefficients_to_file (eof.py:1646-1671)."""
    from ..io import coefficients
    coefficients.eof_coefficients_to_file(f, EOF_Object)


def save_eof_coefficients(outfile, EOF_Object, verbose=0):
    """eof.save_eof_coefficients (eof.py:1675-1709)."""
    from ..io import coefficients
    coefficients.save_eof_coefficients(outfile, EOF_Object, verbose)


def restore_eof_coefficients(infile):
    """eof.restore_eof_coefficients (eof.py:1712-1739): (last dump,
    OrderedDict{time: EOF_Object})."""
    from ..io import coefficients
    return coefficients.restore_eof_coefficients(infile, EOF_Object)


def extract_eof_coefficients(f):
    """eof.extract_eof_coefficients (eof.py:1743-1760)."""
    from ..io import coefficients
    return coefficients.extract_eof_coefficients(f, EOF_Object)


# ---------------------------------------------------------------- EXP coefficient time series
def read_binary_eof_coefficients(coeffile):
    """eof.read_binary_eof_coefficients (eof.py:2230-2293): old-layout EXP
    Cylinder coefficients -> (times, coefs[t, cos/sin, m, n])."""
    from ..io import outcoef
    return outcoef.read_old_cylinder(coeffile)


def read_binary_eof_coefficients_dict(coeffile):
    """eof.read_binary_eof_coefficients_dict (eof.py:2296-2360): {time: EOF_Object}."""
    from ..io import outcoef
    T, c = outcoef.read_old_cylinder(coeffile)
    out = {}
    for t in range(T.size):
        E = EOF_Object()
        E.time = T[t]
        E.mmax, E.nmax = c.shape[2] - 1, c.shape[3]
        E.filename = "[redacted]"
        E.comp = "star"
        E.nbodies = 0.0
        E.eof_file = "[redacted]"
        E.cos = np.array(c[t, 0])
        E.sin = np.array(c[t, 1])
        out[E.time] = E
    return out


def compute_coefficients_series(files, comp, eof_file, outfile=None, precision="f64", reader="psp"):
    """Coefficients of component `comp` in each snapshot file (PSP, or SPL
    main files with reader='spl'): (times, coefs[t, cos/sin, m, n]), the next
    file read while the GPU accumulates the current one.  With `outfile`,
    also written as an EXP Cylinder coefficient file
    (exptool_gb300.io.outcoef.write_new_cylinder)."""
    from ..io import outcoef, series
    table = table_from_file(eof_file)
    T, cs = series.coefficient_series(
        files, comp, lambda x, y, z, m: torch.stack(table.accumulate(x, y, z, m, precision=precision)), reader)
    c = series.stack_to_host(cs)
    if outfile is not None:
        outcoef.write_new_cylinder(outfile, T, c)
    return T, c
