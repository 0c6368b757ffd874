"""Import the exptool reference from a source tree with the minimal shims it
needs on numpy 2 / without matplotlib and PyYAML.

Used only by ``make_golden.py`` to run the reference and record golden
vectors; nothing at test time imports it.  No file of the reference tree is
modified and no bytecode is written into it.

Shims (each one names the reference line it works around):
1. stub modules for matplotlib (``exptool/utils/utils.py:62``,
   ``exptool/basis/eof.py:66-69``) and yaml (``eof.py:81``) — top-level imports
   only, never used on the hot path;
2. ``halo_methods.read_cached_table`` replaced by a reader of the identical
   layout that takes ``[0]`` of the one-element ``np.fromfile`` result, which
   numpy 2 refuses to assign to a scalar slot (``halo_methods.py:154``);
3. ``halo_methods.log = np.log`` (bare ``log`` at ``halo_methods.py:195``);
4. ``spheresl.xmin/xmax`` set to ``log(rmin)/log(rmax)`` before each cmap=2
   call (undefined module globals read at ``spheresl.py:128-130`` and siblings).
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

# root of the exptool source tree (the directory holding the ``exptool``
# package): EXPTOOL_REFERENCE, or the argument of load()
REF_ROOT = os.environ.get("EXPTOOL_REFERENCE", "")


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Stub(self.__name__ + "." + name)

    def __call__(self, *a, **k):
        return _Stub("call")


def load(root=None):
    """Import the reference from ``root`` (default: the EXPTOOL_REFERENCE
    environment variable) with the shims above; returns its modules."""
    root = root or REF_ROOT
    if not root or not os.path.isdir(os.path.join(root, "exptool")):
        raise RuntimeError("set EXPTOOL_REFERENCE (or pass --reference) to the exptool source tree root")
    sys.dont_write_bytecode = True
    if root not in sys.path:
        sys.path.insert(0, root)
    for name in ["matplotlib", "matplotlib.pyplot", "matplotlib.cm", "matplotlib.colors",
                 "matplotlib.colorbar", "yaml", "mpl_toolkits", "mpl_toolkits.mplot3d"]:
        sys.modules.setdefault(name, _Stub(name))
    import warnings
    warnings.filterwarnings("ignore", category=SyntaxWarning)
    from exptool.utils import halo_methods
    from exptool.basis import spheresl, eof, potential
    from exptool.utils import integrate
    from exptool.orbits import orbit
    from exptool.io import particle

    def read_cached_table(file, verbose=0, retall=True):
        with open(file, "rb") as f:
            a = np.fromfile(f, dtype=np.uint32, count=4)
            lmax, nmax, numr, cmap = (int(v) for v in a)
            b = np.fromfile(f, dtype="<f8", count=3)
            rmin, rmax, scale = (float(v) for v in b)
            ltable = np.zeros(lmax + 1)
            evtable = np.ones([lmax + 1, nmax])
            eftable = np.ones([lmax + 1, nmax, numr])
            for l in range(lmax + 1):
                ltable[l] = np.fromfile(f, dtype=np.uint32, count=1)[0]
                evtable[l, 0:nmax] = np.fromfile(f, dtype="f8", count=nmax)
                for n in range(nmax):
                    eftable[l, n, :] = np.fromfile(f, dtype="f8", count=numr)
        if retall:
            return lmax, nmax, numr, cmap, rmin, rmax, scale, ltable, evtable, eftable
        return ltable, evtable, eftable

    halo_methods.read_cached_table = read_cached_table
    halo_methods.log = np.log
    ns = types.SimpleNamespace(halo_methods=halo_methods, spheresl=spheresl, eof=eof,
                               potential=potential, integrate=integrate, orbit=orbit,
                               particle=particle)
    return ns


def set_log_bounds(ref, rmin, rmax):
    """Shim 4: the cmap=2 clamps read module globals xmin/xmax."""
    ref.spheresl.xmin = float(np.log(rmin))
    ref.spheresl.xmax = float(np.log(rmax))


def patch_eof_compute_coefficients(ref):
    """Shim 5: eof.compute_coefficients tests ``if nanvals > 0`` on an index
    array (eof.py:1194), which numpy 2 refuses for an empty array.  The
    replacement takes the function's own steps with that test written
    ``nanvals.size > 0``: the EOF_Object fields of eof.py:1207-1216 and
    :1250-1251, the tables through the reference's parse_eof / eof_params /
    set_table_params, and the coefficients from its single-process
    ``accumulate`` branch (eof.py:1236-1243)."""
    eof = ref.eof

    def compute_coefficients(PSPInput, eof_file, verbose=1, no_odd=False, nprocs_max=-1, VAR=False,
                             nanblock=False):
        d = PSPInput.data
        nanvals = np.where(np.isnan(d['x']) | np.isnan(d['y']) | np.isnan(d['z']))[0]
        if nanvals.size > 0 and not nanblock:
            d['x'][nanvals] = 0.
            d['y'][nanvals] = 0.
            d['z'][nanvals] = 0.
        out = eof.EOF_Object()
        out.time = PSPInput.time
        out.filename = PSPInput.filename
        out.comp = PSPInput.comp
        out.nbodies = d['m'].size
        out.eof_file = eof_file
        potC, rforceC, zforceC, densC, potS, rforceS, zforceS, densS = eof.parse_eof(eof_file)
        rmin, rmax, numx, numy, mmax, norder, ascale, hscale, cmap, dens = eof.eof_params(eof_file)
        XMIN, XMAX, dX, YMIN, YMAX, dY = eof.set_table_params(RMAX=rmax, RMIN=rmin, ASCALE=ascale, HSCALE=hscale,
                                                              NUMX=numx, NUMY=numy, CMAP=cmap)
        out.mmax = mmax
        out.nmax = norder
        out.cos, out.sin = eof.accumulate(PSPInput, potC, potS, mmax, norder, XMIN, dX, YMIN, dY, numx, numy, ascale,
                                          hscale, cmap, verbose=verbose, no_odd=no_odd)
        return out

    keep = eof.compute_coefficients
    eof.compute_coefficients = compute_coefficients
    return keep
