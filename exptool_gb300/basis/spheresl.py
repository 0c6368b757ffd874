"""Spherical Sturm-Liouville expansion on the GPU, with the call signatures of
``exptool/basis/spheresl.py``.

Every function here marshals NumPy inputs to the device and calls the CUDA
library (``include/exptool_gb300.h``); outputs come back as NumPy arrays owned
by the caller.  Tables are uploaded once per (file, size, mtime) or per array
content and reused.  ``precision='f32'`` selects the mixed path (FP32
per-particle arithmetic, FP64 reductions); the default ``'f64'`` is the drop-in.

Behaviour that differs from the reference where the reference cannot run:
* cmap = 2 clamps use log(rmin), log(rmax) (the reference reads undefined
  globals ``xmin``/``xmax``, spheresl.py:128-130);
* ``eval_particles`` honours l1/l2 for any ``nprocs`` (the reference's
  multi-process branch crashes, spheresl.py:507);
* ``all_eval`` truncated to lmax keeps (lmax+1)^2 coefficient rows (the
  reference keeps lmax+1 rows and then indexes past them, spheresl.py:1019).
"""
from __future__ import annotations

import numpy as np
import torch

from .. import _lib
from .. import device as dev
from ..io.particle import positions
from ..utils import halo_methods


class SL_Object(object):
    """Coefficient container (spheresl.py:1377-1386)."""
    time = None
    dump = None
    comp = None
    nbodies = None
    lmax = None
    nmax = None
    sph_file = None
    model_file = None
    expcoef = None
    filename = None


# ---------------------------------------------------------------- table caches
def table_from_files(sph_file, mod_file) -> dev.SphTable:
    key = ("sph-files", dev.file_key(sph_file), dev.file_key(mod_file))

    def make():
        lmax, nmax, numr, cmap, rmin, rmax, scale, lt, ev, ef = halo_methods.read_cached_table(sph_file)
        xi, r, p0, d0 = halo_methods.init_table(mod_file, numr, rmin, rmax, cmap, scale)
        return dev.SphTable(lmax, nmax, numr, cmap, rmin, rmax, scale, xi, p0, d0, ev, ef)

    return dev.TABLES.get(key, make)


def table_from_arrays(xi, p0, d0, cmap, scale, evtable, eftable) -> dev.SphTable:
    xi = np.asarray(xi, dtype=np.float64)
    ev = np.asarray(evtable, dtype=np.float64)
    ef = np.asarray(eftable, dtype=np.float64)
    key = ("sph-arrays", dev.fingerprint(xi, p0, d0, ev, ef), int(cmap), float(scale))

    def make():
        lmax = ev.shape[0] - 1
        nmax = ev.shape[1]
        if int(cmap) == 2:
            rmin, rmax = float(np.exp(xi[0])), float(np.exp(xi[-1]))
        else:
            rmin, rmax = float(xi[0]), float(xi[-1])
        return dev.SphTable(lmax, nmax, xi.size, int(cmap), rmin, rmax, float(scale), xi, p0, d0, ev, ef)

    return dev.TABLES.get(key, make)


def field_for(table, expcoef, coef_scale=1.0, lmax_use=-1, nmax_use=-1, precision="f64") -> dev.SphField:
    ec = np.asarray(expcoef, dtype=np.float64) if not isinstance(expcoef, torch.Tensor) else expcoef
    if isinstance(ec, torch.Tensor):
        return table.prepare(ec, coef_scale, lmax_use, nmax_use, precision)
    key = (dev.fingerprint(ec), float(coef_scale), int(lmax_use), int(nmax_use), precision)
    return table.field_cache.get(key, lambda: table.prepare(ec, coef_scale, lmax_use, nmax_use, precision))


def _full_coef(expcoef, table, lmax_use, nmax_use):
    """Pad a truncated coefficient matrix to the table's full (rows, nmax)."""
    ec = np.asarray(expcoef, dtype=np.float64)
    full = np.zeros((table.nrow, table.nmax))
    rows = min(ec.shape[0], table.nrow)
    cols = min(ec.shape[1], table.nmax)
    full[:rows, :cols] = ec[:rows, :cols]
    return full


# ---------------------------------------------------------------- accumulation
def compute_coefficients_solitary(ParticleInstance, sph_file, model_file, verbose=0, no_odd=False, precision="f64"):
    """spheresl.compute_coefficients_solitary (spheresl.py:567-656): returns
    expcoef ((lmax+1)^2, nmax)."""
    table = table_from_files(sph_file, model_file)
    x, y, z, m = (dev.to_dev(a) for a in positions(ParticleInstance))
    ec = table.accumulate(x, y, z, m, no_odd=no_odd, precision=precision)
    return dev.fetch_many([ec])[0]


def compute_coefficients(PSPInput, sph_file, mod_file, verbose=1, no_odd=False, precision="f64"):
    """spheresl.compute_coefficients (spheresl.py:439-475): one GPU pass over
    all particles (the reference's process pool and object-array sum are not
    needed).  Returns an SL_Object."""
    out = SL_Object()
    out.time = getattr(PSPInput, "time", None)
    out.filename = getattr(PSPInput, "filename", None)
    out.comp = getattr(PSPInput, "comp", None)
    x, y, z, m = positions(PSPInput)
    out.nbodies = m.size
    out.sph_file = sph_file
    out.model_file = mod_file
    table = table_from_files(sph_file, mod_file)
    out.lmax = table.lmax
    out.nmax = table.nmax
    xd, yd, zd, md = (dev.to_dev(a) for a in (x, y, z, m))
    out.expcoef = dev.fetch_many([table.accumulate(xd, yd, zd, md, no_odd=no_odd, precision=precision)])[0]
    return out


def compute_coefficients_batched(snapshots, sph_file, mod_file, no_odd=False, autotune=True, chunk=None,
                                 threads=None, engine="deposit", stages=None):
    """Coefficients of many snapshots in one pass on the GPU (the series
    spheresl.compute_coefficients would produce one call at a time).

    ``snapshots``: a list of particle containers (holder-like or ``.data``),
    or a pair (xyzm, offsets) with xyzm an (N, 4) float32 array / CUDA tensor
    of x y z m and offsets the nsnap+1 snapshot boundaries.  Returns an array
    of shape (nsnap, (lmax+1)^2, nmax).

    engine="deposit": one persistent launch with FP32 per-particle arithmetic
    and shared-memory accumulation, FP64 sums across work items and FP64
    contraction (about 1e-7 of FP64).  engine="tensor": particles sorted by
    (snapshot, radial window), BF16 products of interpolation weights and
    angular basis values on the tensor cores with FP32 accumulation, FP64
    window sums and contraction (BF16 operands: about 1e-4 of FP64 on
    snapshots of 1e4 particles and more).  ``chunk``/``threads`` (deposit)
    or ``chunk``/``stages`` (tensor) fix the launch shape; otherwise it is
    autotuned (or a default with autotune=False)."""
    table = table_from_files(sph_file, mod_file)
    if isinstance(snapshots, tuple) and len(snapshots) == 2:
        xyzm, offsets = snapshots
        offsets = np.asarray(offsets, dtype=np.int64)
        if not isinstance(xyzm, torch.Tensor):
            xyzm = torch.from_numpy(np.ascontiguousarray(np.asarray(xyzm, dtype=np.float32)))
        xyzm = xyzm.to(dev.device(), dtype=torch.float32).contiguous()
    else:
        parts, counts = [], [0]
        for P in snapshots:
            x, y, z, m = positions(P)
            parts.append(np.stack([x, y, z, m], axis=1).astype(np.float32))
            counts.append(x.size)
        offsets = np.cumsum(counts).astype(np.int64)
        xyzm = torch.from_numpy(np.concatenate(parts, axis=0)).to(dev.device()).contiguous()
    if engine == "tensor":
        if chunk is None or stages is None:
            if autotune:
                from .. import autotune as at
                cfg, _ = at.sph_batched_tc_config(table, xyzm, offsets)
            else:
                cfg = {"chunk": 16384, "stages": 1, "ctas_per_sm": 0, "threads_per_particle": 1}
            chunk = cfg["chunk"] if chunk is None else chunk
            stages = cfg["stages"] if stages is None else stages
            ctas, split = cfg["ctas_per_sm"], cfg["threads_per_particle"]
        else:
            ctas, split = 0, 1
        out = table.accumulate_batched_tc(xyzm, offsets, no_odd=no_odd, chunk=chunk, stages=stages, ctas_per_sm=ctas,
                                          threads_per_particle=split)
        host = dev.to_host(out)
        dev.batched_tc_status()
        return host
    if engine != "deposit":
        raise ValueError(f"engine must be 'deposit' or 'tensor', not {engine!r}")
    if chunk is None or threads is None:
        if autotune:
            from .. import autotune as at
            cfg, _ = at.sph_batched_config(table, xyzm, offsets)
        else:
            cfg = {"chunk": 262144, "threads": 512}
        chunk = cfg["chunk"] if chunk is None else chunk
        threads = cfg["threads"] if threads is None else threads
    return dev.to_host(table.accumulate_batched(xyzm, offsets, no_odd=no_odd, chunk=chunk, threads=threads))


# ---------------------------------------------------------------- evaluation
def all_eval_particles(Particles, expcoef, sph_file, mod_file, verbose=0, L1=-1000, L2=1000, NO_ODD=False,
                       precision="f64"):
    """spheresl.all_eval_particles (spheresl.py:1240-1362): returns
    den0, den1, pot0, pot1, potr, pott, potp, rr."""
    table = table_from_files(sph_file, mod_file)
    field = field_for(table, expcoef, precision=precision)
    d = Particles.data
    a, b, c = (dev.to_dev(d[k]) for k in ("x", "y", "z"))
    outs = table.eval_points(field, a, b, c, _lib.XT_SPH_ALL_EVAL_PARTICLES, _lib.XT_COORD_CART, L1=L1, L2=L2,
                             no_odd=NO_ODD)
    return tuple(dev.to_host_many(list(outs)))


def eval_particles(ParticleInstance, expcoef, sph_file, mod_file, nprocs=-1, verbose=1, l1=0, l2=1000,
                   precision="f64"):
    """spheresl.eval_particles (spheresl.py:502-528)."""
    return all_eval_particles(ParticleInstance, expcoef, sph_file, mod_file, verbose, L1=l1, L2=l2,
                              precision=precision)


def _points(*vals):
    arrs = [np.atleast_1d(np.asarray(v, dtype=np.float64)) for v in vals]
    n = max(a.size for a in arrs)
    arrs = [np.broadcast_to(a, (n,)) if a.size != n else a for a in arrs]
    scalar = all(np.ndim(v) == 0 for v in vals)
    return arrs, scalar


def _point_eval(mode, r, costh, phi, expcoef, xi, p0, d0, cmap, scale, lmax, nmax, evtable, eftable, no_odd,
                trig_l, precision):
    table = table_from_arrays(xi, p0, d0, cmap, scale, evtable, eftable)
    lmax = table.lmax if lmax is None else int(lmax)
    nmax = table.nmax if nmax is None else int(nmax)
    lmax_use = lmax if lmax < table.lmax else table.lmax
    nmax_use = nmax if nmax < table.nmax else table.nmax
    coef = _full_coef(expcoef, table, lmax_use, nmax_use)
    field = field_for(table, coef, 1.0, lmax_use, nmax_use, precision)
    (ra, ca, pa), scalar = _points(r, costh, phi)
    outs = table.eval_points(field, dev.to_dev(ra), dev.to_dev(ca), dev.to_dev(pa), mode, _lib.XT_COORD_SPH,
                             no_odd=no_odd, lmax_use=lmax_use, trig_l=trig_l)
    return outs, scalar


def all_eval(r, costh, phi, expcoef, xi, p0, d0, cmap, scale, lmax, nmax, evtable, eftable, no_odd=False, verbose=0,
             precision="f64"):
    """spheresl.all_eval (spheresl.py:987-1102); r, costh, phi may be arrays.
    Returns den0, den1, pot0, pot1, potr, pott, potp."""
    outs, scalar = _point_eval(_lib.XT_SPH_ALL_EVAL, r, costh, phi, expcoef, xi, p0, d0, cmap, scale, lmax, nmax,
                               evtable, eftable, no_odd, False, precision)
    res = dev.to_host_many(list(outs[:7]))
    return tuple(float(v[0]) for v in res) if scalar else tuple(res)


def force_eval(r, costh, phi, expcoef, xi, p0, d0, cmap, scale, lmax, nmax, evtable, eftable, no_odd=False,
               verbose=0, correct_m=False, precision="f64"):
    """spheresl.force_eval (spheresl.py:1107-1234): returns potr, pott, potp,
    pot1, pot0.  By default the azimuthal factor of row (l, m) is cos(l phi) /
    sin(l phi) exactly as the reference computes it (spheresl.py:1173);
    ``correct_m=True`` uses cos(m phi) / sin(m phi) as ``all_eval`` does."""
    outs, scalar = _point_eval(_lib.XT_SPH_FORCE_EVAL, r, costh, phi, expcoef, xi, p0, d0, cmap, scale, lmax, nmax,
                               evtable, eftable, no_odd, not correct_m, precision)
    res = dev.to_host_many(list(outs[:5]))
    return tuple(float(v[0]) for v in res) if scalar else tuple(res)


def factorial_return(lmax):
    """spheresl.factorial_return (spheresl.py:823-863), host-side constants."""
    from scipy.special import gammaln
    f = np.zeros((lmax + 1, lmax + 1))
    for l in range(lmax + 1):
        for m in range(l + 1):
            f[l, m] = np.sqrt((0.5 * l + 0.25) / np.pi * np.exp(gammaln(1.0 + l - m) - gammaln(1.0 + l + m)))
            if m != 0:
                f[l, m] *= np.sqrt(2.0)
    return f


# ---------------------------------------------------------------- coefficient files
def sl_coefficients_to_file(f, SL_Object):
    """spheresl.sl_coefficients_to_file (spheresl.py:1390-1409): one dump at
    the current position of the open file."""
    from ..io import coefficients
    coefficients.sl_coefficients_to_file(f, SL_Object)


def save_sl_coefficients(outfile, SL_Object, verbose=0):
    """spheresl.save_sl_coefficients (spheresl.py:1414-1441): append a dump and
    bump the leading dump count."""
    from ..io import coefficients
    coefficients.save_sl_coefficients(outfile, SL_Object, verbose)


def restore_sl_coefficients(infile):
    """spheresl.restore_sl_coefficients (spheresl.py:1444-1467): (last dump,
    {round(time, 3): SL_Object})."""
    from ..io import coefficients
    return coefficients.restore_sl_coefficients(infile, SL_Object)


def extract_sl_coefficients(f):
    """spheresl.extract_sl_coefficients (spheresl.py:1471-1488)."""
    from ..io import coefficients
    return coefficients.extract_sl_coefficients(f, SL_Object)


# ---------------------------------------------------------------- EXP coefficient time series
def read_binary_sl_coefficients(coeffile):
    """spheresl.read_binary_sl_coefficients (spheresl.py:1636-1696): old-layout
    EXP SphereSL coefficients -> (times, coefs[t, lm, n])."""
    from ..io import outcoef
    return outcoef.read_old_spheresl(coeffile)


def compute_coefficients_series(files, comp, sph_file, mod_file, outfile=None, no_odd=False, precision="f64",
                                reader="psp"):
    """Coefficients of component `comp` in each snapshot file (PSP, or SPL
    main files with reader='spl'): (times, expcoef[t, (lmax+1)^2, nmax]), the
    next file read while the GPU accumulates the current one.  With
    `outfile`, also written as an EXP SphereSL coefficient file
    (exptool_gb300.io.outcoef.write_new_spheresl)."""
    from ..io import outcoef, series
    table = table_from_files(sph_file, mod_file)
    T, cs = series.coefficient_series(
        files, comp, lambda x, y, z, m: table.accumulate(x, y, z, m, no_odd=no_odd, precision=precision), reader)
    ec = series.stack_to_host(cs)
    if outfile is not None:
        outcoef.write_new_spheresl(outfile, T, ec)
    return T, ec
