"""Halo (SL) + disc (EOF) field composition on the GPU, with the interface of
``exptool/basis/potential.py`` ``Fields``.

``prep_tables`` uploads both bases once; the coefficient-contracted fields are
prepared on first use and cached for the current coefficients, halofac and
truncation settings, so repeated force calls (orbit integration) only run the
per-point kernel.  ``total_coefficients`` reads the snapshot named by the
instance (or takes in-memory particle containers); ``get_fields`` is the
snapshot -> prepared Fields driver of the reference.
"""
from __future__ import annotations

import numpy as np

from .. import device as dev
from ..utils import halo_methods
from . import eof, spheresl


class Fields:
    """Field of a halo + disc system (potential.py:49-963)."""

    def __init__(self, infile, eof_file, sph_file, model_file, nhalo=1000000, transform=False, no_odd=False,
                 centering=False, mutual_center=False, verbose=1, precision="f64", halo_correct_m=False):
        self.filename = infile
        self.eof_file = eof_file
        self.sph_file = sph_file
        self.model_file = model_file
        self.nhalo = nhalo
        self.transform = transform
        self.no_odd = no_odd
        self.centering = centering
        self.mutual_center = mutual_center
        self.verbose = verbose
        self.halofac = 1.0
        self.precision = precision
        # The reference halo force (spheresl.force_eval) uses cos(l phi) for row
        # (l, m) (spheresl.py:1173); halo_correct_m=True uses cos(m phi).
        self.halo_correct_m = halo_correct_m
        self._fcache = {}

    # ------------------------------------------------------------ coefficients
    def total_coefficients(self, disk_particles=None, halo_particles=None, halo_total=None, ncenter=10000):
        """potential.Fields.total_coefficients (potential.py:98-252).

        Called without arguments, as in the reference: reads the components
        'star' (disc) and 'dark' (halo) of the snapshot ``self.filename`` with
        ``particle.Input`` (PSP or SPL by file name), sets ``self.time`` from
        the disc component and halofac = 1 (the reference divides the halo
        count by itself, :139-142).

        Added keywords: ``disk_particles`` and ``halo_particles`` take
        in-memory containers (``.data`` dicts or holders) instead of the file,
        and halofac = len(halo_particles) / halo_total when halo_total is
        given.

        With ``centering``: the mass-weighted centre of the ``ncenter`` disc
        particles nearest the origin (argsort of r) is taken off the disc, and
        off the halo either the same centre (``mutual_center``) or the centre
        of the halo particles at those same indices (the reference ranks the
        disc radii for the halo too, :196-205); then both bases are
        accumulated on the GPU."""
        if self.transform:
            raise NotImplementedError("transform=True needs the bar transform of exptool.analysis.pattern")
        if disk_particles is None and halo_particles is None:
            from ..io import particle
            disk_particles = particle.Input(self.filename, comp='star', verbose=self.verbose)
            halo_particles = particle.Input(self.filename, comp='dark', verbose=self.verbose)
        elif disk_particles is None or halo_particles is None:
            raise ValueError("total_coefficients: give both disk_particles and halo_particles, or neither "
                             "(then components 'star' and 'dark' of the snapshot self.filename are read)")
        from ..io.particle import holder, positions
        self.time = getattr(disk_particles, "time", None)
        dx, dy, dz, dm = positions(disk_particles)
        hx, hy, hz, hm = positions(halo_particles)
        self.halofac = float(hm.size) / float(halo_total) if halo_total else 1.0
        if self.centering:
            print('potential.Fields.total_coefficients: Computing centering (centering=True)')
            cp = ((dx * dx + dy * dy + dz * dz) ** 0.5).argsort()[0:ncenter]
            wd = np.sum(dm[cp])
            self.xcen_disk = np.sum(dx[cp] * dm[cp]) / wd
            self.ycen_disk = np.sum(dy[cp] * dm[cp]) / wd
            self.zcen_disk = np.sum(dz[cp] * dm[cp]) / wd
            if self.mutual_center:
                print('potential.Fields.total_coefficients: Using computed disk center for halo (mutual_center=True)')
                self.xcen_halo, self.ycen_halo, self.zcen_halo = self.xcen_disk, self.ycen_disk, self.zcen_disk
            else:
                wh = np.sum(hm[cp])
                self.xcen_halo = np.sum(hx[cp] * hm[cp]) / wh
                self.ycen_halo = np.sum(hy[cp] * hm[cp]) / wh
                self.zcen_halo = np.sum(hz[cp] * hm[cp]) / wh
            print('potential.Fields.total_coefficients: (x,y,z) = {0:6.5f},{1:6.5f},{2:6.5f}'
                  .format(float(self.xcen_disk), float(self.ycen_disk), float(self.zcen_disk)))
        else:
            self.xcen_disk = self.ycen_disk = self.zcen_disk = 0.
            self.xcen_halo = self.ycen_halo = self.zcen_halo = 0.

        def shifted(x, y, z, m, cx, cy, cz, src):
            h = holder()
            h.xpos, h.ypos, h.zpos, h.mass = x - cx, y - cy, z - cz, m
            h.time = getattr(src, "time", None)
            return h

        disk = shifted(dx, dy, dz, dm, self.xcen_disk, self.ycen_disk, self.zcen_disk, disk_particles)
        halo = shifted(hx, hy, hz, hm, self.xcen_halo, self.ycen_halo, self.zcen_halo, halo_particles)
        self.centered_particles = (disk, halo)
        self.EOF = eof.compute_coefficients(disk, self.eof_file, verbose=self.verbose, no_odd=self.no_odd)
        self.SL = spheresl.compute_coefficients(halo, self.sph_file, self.model_file, verbose=self.verbose,
                                                no_odd=self.no_odd)

    # ------------------------------------------------------------ tables
    def prep_tables(self):
        """Read and upload both bases (potential.py:257-294)."""
        self._read_tables()
        self._cyl = eof.table_from_file(self.EOF.eof_file)
        self._upload_halo()

    def _read_tables(self):
        """The host half of prep_tables: table arrays and parameters as
        instance attributes (what save_field writes)."""
        try:
            eof_file = self.EOF.eof_file
        except AttributeError:
            raise RuntimeError("potential.Fields.prep_tables: must first call total_coefficients.") from None
        self.potC, self.rforceC, self.zforceC, self.densC, self.potS, self.rforceS, self.zforceS, self.densS = \
            eof.parse_eof(eof_file)
        (self.rmindisk, self.rmaxdisk, self.numx, self.numy, self.mmax, self.norder, self.ascale, self.hscale,
         self.cmapdisk, self.densdisk) = eof.eof_params(eof_file)
        self.XMIN, self.XMAX, self.dX, self.YMIN, self.YMAX, self.dY = eof.set_table_params(
            RMAX=self.rmaxdisk, RMIN=self.rmindisk, ASCALE=self.ascale, HSCALE=self.hscale, NUMX=self.numx,
            NUMY=self.numy, CMAP=self.cmapdisk)
        self.disk_use_m = self.mmax
        self.disk_use_n = self.norder
        (self.lmaxhalo, self.nmaxhalo, self.numrhalo, self.cmaphalo, self.rminhalo, self.rmaxhalo, self.scalehalo,
         self.ltablehalo, self.evtablehalo, self.eftablehalo) = halo_methods.read_cached_table(self.SL.sph_file)
        self.xihalo, self.rarrhalo, self.p0halo, self.d0halo = halo_methods.init_table(
            self.SL.model_file, self.numrhalo, self.rminhalo, self.rmaxhalo, cmap=self.cmaphalo, scale=self.scalehalo)
        self.halo_use_l = self.lmaxhalo
        self.halo_use_n = self.nmaxhalo

    def _upload_halo(self):
        self._sph = dev.SphTable(self.lmaxhalo, self.nmaxhalo, self.numrhalo, self.cmaphalo, self.rminhalo,
                                 self.rmaxhalo, self.scalehalo, self.xihalo, self.p0halo, self.d0halo,
                                 self.evtablehalo, self.eftablehalo)
        self._fcache = {}

    def _upload_from_arrays(self):
        """Device tables from the instance's own arrays (a restored field)."""
        dens = bool(self.densdisk)
        self._cyl = eof.table_from_arrays(self.mmax, self.norder, self.numx, self.numy, self.cmapdisk, self.XMIN,
                                          self.dX, self.YMIN, self.dY, self.ascale, self.hscale, self.potC,
                                          self.rforceC, self.zforceC, self.potS, self.rforceS, self.zforceS,
                                          self.densC if dens else None, self.densS if dens else None)
        self._upload_halo()

    # ------------------------------------------------------------ persistence
    def save_field(self, filename=''):
        """potential.Fields.save_field (potential.py:738-963): the global, EOF
        and SL blocks of a prepared instance in one binary record, readable by
        ``restore_field``."""
        from ..io import coefficients
        if filename == '':
            print('potential.Fields.save_field: No filename specified.')
        if not hasattr(self, "potC"):
            self._read_tables()
        for k in ("xcen_disk", "ycen_disk", "zcen_disk", "xcen_halo", "ycen_halo", "zcen_halo"):
            if not hasattr(self, k):
                setattr(self, k, 0.0)
        with open(filename, "wb") as f:
            coefficients.field_record(self).tofile(f)

    # ------------------------------------------------------------ curves
    def rotation_curve(self, rvals=np.linspace(0.0001, 0.1, 100), mono=False, angle=0.):
        """potential.Fields.rotation_curve (potential.py:500-565): v_c from the
        radial forces at (x, y, z) = (r, angle, 0) -- the reference passes
        `angle` as the y coordinate -- all points in one GPU call."""
        if mono:
            keep = (self.halo_use_l, self.disk_use_m)
            self.halo_use_l, self.disk_use_m = 0, 0
        rv = np.asarray(rvals, dtype=np.float64)
        res = self.return_forces_cyl(rv, np.full_like(rv, angle), np.zeros_like(rv))
        disk_force, halo_force = np.asarray(res[0]), np.asarray(res[1])
        self.rvals = rvals
        self.disk_dpdr = -1. * disk_force
        self.halo_dpdr = -1. * halo_force
        self.total_dpdr = -1. * disk_force + -1. * halo_force
        self.disk_rotation = (rv * abs(disk_force)) ** 0.5
        self.halo_rotation = (rv * abs(halo_force)) ** 0.5
        self.total_rotation = (rv * (abs(halo_force) + abs(disk_force))) ** 0.5
        if mono:
            self.halo_use_l, self.disk_use_m = keep

    def resonance_positions(self, rvals=np.linspace(0.0001, 0.1, 100), mono=False):
        """potential.Fields.resonance_positions (potential.py:568-628): omega and
        kappa = sqrt(3 omega^2 + d omega/dr) (the reference's expression) from
        the radial forces along +x, derivative by an interpolating cubic spline."""
        from scipy.interpolate import UnivariateSpline
        if mono:
            keep = (self.halo_use_l, self.disk_use_m)
            self.halo_use_l, self.disk_use_m = 0, 0
        rv = np.asarray(rvals, dtype=np.float64)
        res = self.return_forces_cyl(rv, np.zeros_like(rv), np.zeros_like(rv))
        disk_force, halo_force = np.asarray(res[0]), np.asarray(res[1])
        self.rvals = rvals
        self.omega = ((abs(halo_force) + abs(disk_force)) / rv) ** 0.5
        spl = UnivariateSpline(rv, self.omega, k=3, s=0)
        ddphi = spl.derivative()(rv)
        self.kappa = (3. * self.omega ** 2. + ddphi) ** 0.5
        if mono:
            self.halo_use_l, self.disk_use_m = keep

    def set_field_parameters(self, no_odd=False, halo_l=-1, halo_n=-1, disk_m=-1, disk_n=-1):
        """potential.py:365-377."""
        self.no_odd = no_odd
        if halo_l > -1:
            self.halo_use_l = halo_l
        if halo_n > -1:
            self.halo_use_n = halo_n
        if disk_m > -1:
            self.disk_use_m = disk_m
        if disk_n > -1:
            self.disk_use_n = disk_n

    def reset_field_parameters(self):
        """potential.py:380-386."""
        self.no_odd = False
        self.halo_use_l = self.lmaxhalo
        self.halo_use_n = self.nmaxhalo
        self.disk_use_m = self.mmax
        self.disk_use_n = self.norder

    # ------------------------------------------------------------ device fields
    def device_fields(self, precision=None):
        """(SphField, CylField) for the current coefficients and settings."""
        if not hasattr(self, "_sph"):
            self.prep_tables()
        precision = self.precision if precision is None else precision
        ec = np.asarray(self.SL.expcoef, dtype=np.float64)
        key = (dev.fingerprint(ec, self.EOF.cos, self.EOF.sin), float(self.halofac), int(self.halo_use_l),
               int(self.halo_use_n), int(self.disk_use_m), int(self.disk_use_n), precision)
        if key not in self._fcache:
            lmax_use = min(int(self.halo_use_l), self.lmaxhalo)
            nmax_use = min(int(self.halo_use_n), self.nmaxhalo)
            sf = self._sph.prepare(ec, self.halofac, lmax_use, nmax_use, precision)
            cf = self._cyl.prepare(np.asarray(self.EOF.cos), np.asarray(self.EOF.sin), min(int(self.disk_use_m),
                                                                                          self.mmax),
                                   min(int(self.disk_use_n), self.norder), False, precision)
            self._fcache = {key: (sf, cf)}
        return self._fcache[key]

    def _halo_l(self):
        return min(int(self.halo_use_l), self.lmaxhalo)

    def _disk_m(self):
        return min(int(self.disk_use_m), self.mmax)

    def return_forces_cart(self, xval, yval, zval, rotpos=0.0):
        """potential.py:445-497: fxdisk, fxhalo, fydisk, fyhalo, fzdisk, fzhalo,
        diskp, halop+halop0.  Scalars or arrays (rotpos scalar or per point)."""
        sf, cf = self.device_fields()
        scalar = all(np.ndim(v) == 0 for v in (xval, yval, zval))
        x = np.atleast_1d(np.asarray(xval, dtype=np.float64))
        y = np.atleast_1d(np.asarray(yval, dtype=np.float64))
        z = np.atleast_1d(np.asarray(zval, dtype=np.float64))
        rot = None
        rs = 0.0
        if np.ndim(rotpos) == 0:
            rs = float(rotpos)
        else:
            rot = dev.to_dev(np.asarray(rotpos, dtype=np.float64))
        outs = dev.fields_forces(sf, cf, dev.to_dev(x), dev.to_dev(y), dev.to_dev(z), rotpos=rot, rotpos_scalar=rs,
                                 halo_l=self._halo_l(), disk_m=self._disk_m(), no_odd=self.no_odd,
                                 trig_l=not self.halo_correct_m)
        res = [dev.to_host(t) for t in outs]
        return tuple(float(v[0]) for v in res) if scalar else tuple(res)

    def return_forces_cyl(self, xval, yval, zval, rotpos=0.0):
        """potential.py:389-442: diskfr, frhalo, diskfp, -halofp, diskfz, fzhalo,
        -diskp, halop+halop0, with R = sqrt(x^2+y^2)+1e-10, r = sqrt(R^2+z^2)+1e-10."""
        if not hasattr(self, "_sph"):
            self.prep_tables()
        scalar = all(np.ndim(v) == 0 for v in (xval, yval, zval))
        x = np.atleast_1d(np.asarray(xval, dtype=np.float64))
        y = np.atleast_1d(np.asarray(yval, dtype=np.float64))
        z = np.atleast_1d(np.asarray(zval, dtype=np.float64))
        r2 = np.sqrt(x * x + y * y) + 1.0e-10
        r3 = np.sqrt(r2 * r2 + z * z) + 1.0e-10
        costh = z / r3
        phi = np.arctan2(y, x) + rotpos
        sf, cf = self.device_fields()
        from .. import _lib
        dfr, dfp, dfz, dp, dp0 = self._cyl.eval_points(cf, dev.to_dev(r2), dev.to_dev(z), dev.to_dev(phi),
                                                       _lib.XT_CYL_FORCE_EVAL, _lib.XT_COORD_CYL,
                                                       mmax_use=self._disk_m(), no_odd=self.no_odd)[:5]
        hfr, hft, hfp, hp, hp0 = self._sph.eval_points(sf, dev.to_dev(r3), dev.to_dev(costh), dev.to_dev(phi),
                                                       _lib.XT_SPH_FORCE_EVAL, _lib.XT_COORD_SPH, no_odd=self.no_odd,
                                                       lmax_use=self._halo_l(), trig_l=not self.halo_correct_m)[:5]
        dfr, dfp, dfz, dp, hfr, hft, hfp, hp, hp0 = (dev.to_host(t) for t in (dfr, dfp, dfz, dp, hfr, hft, hfp, hp,
                                                                             hp0))
        inner = r3 < np.min(self.xihalo)
        hfp = np.where(inner, 0.0, hfp)
        dfp = np.where(inner, 0.0, dfp)
        frhalo = -1.0 * (r2 * hfr + z * hft) / r3
        fzhalo = -1.0 * (z * hfr - r2 * hft) / r3
        res = (dfr, frhalo, dfp, -1.0 * hfp, dfz, fzhalo, -1.0 * dp, hp + hp0)
        return tuple(float(v[0]) for v in res) if scalar else res


def restore_field(filename=''):
    """potential.restore_field (potential.py:968-1042): a Fields instance
    from a ``save_field`` file, with its tables and coefficients, ready for
    force evaluation without the original cache files."""
    from ..io import coefficients
    r = coefficients.read_field_record(filename)
    infile, eof_file, sph_file, model_file = r["files"]
    nhalo, transform, no_odd, centering, mutual_center, verbose = (int(v) for v in r["flags"])
    F = Fields(infile, eof_file, sph_file, model_file, nhalo=nhalo, transform=transform, no_odd=no_odd,
               centering=centering, mutual_center=mutual_center, verbose=verbose)
    F.time = r["time"]
    F.numx, F.numy, F.mmax, F.norder, F.cmapdisk, F.densdisk = (int(v) for v in r["eof_i"])
    (F.rmindisk, F.rmaxdisk, F.ascale, F.hscale, F.XMIN, F.dX, F.YMIN, F.dY, F.xcen_disk, F.ycen_disk,
     F.zcen_disk) = r["eof_f"]
    shp = (F.mmax + 1, F.norder, F.numx + 1, F.numy + 1)
    F.EOF = eof.EOF_Object()
    F.EOF.cos = r["cos"].reshape(F.mmax + 1, F.norder)
    F.EOF.sin = r["sin"].reshape(F.mmax + 1, F.norder)
    for k in ("potC", "rforceC", "zforceC", "densC", "potS", "rforceS", "zforceS", "densS"):
        setattr(F, k, r[k].reshape(shp))
    F.halofac, F.rminhalo, F.rmaxhalo, F.scalehalo, F.xcen_halo, F.ycen_halo, F.zcen_halo = r["sl_f"]
    F.numrhalo, F.cmaphalo, F.lmaxhalo, F.nmaxhalo = (int(v) for v in r["sl_i"])
    F.xihalo, F.p0halo, F.d0halo = r["xi"], r["p0"], r["d0"]
    F.ltable = F.ltablehalo = r["ltable"]
    F.evtablehalo = r["ev"].reshape(F.lmaxhalo + 1, F.nmaxhalo)
    F.eftablehalo = r["ef"].reshape(F.lmaxhalo + 1, F.nmaxhalo, F.numrhalo)
    F.SL = spheresl.SL_Object()
    F.SL.expcoef = r["expcoef"].reshape((F.lmaxhalo + 1) ** 2, F.nmaxhalo)
    F.disk_use_m, F.disk_use_n = F.mmax, F.norder
    F.halo_use_l, F.halo_use_n = F.lmaxhalo, F.nmaxhalo
    F.SL.model_file, F.SL.sph_file = F.model_file, F.sph_file
    F.EOF.eof_file, F.EOF.mmax = F.eof_file, F.mmax
    F.halofac = float(F.halofac)
    F._upload_from_arrays()
    return F


def get_fields(simulation_directory, simulation_name, intime, eof_file, sph_file, model_file, bar_file='',
               nhalo=1000000, transform=True, fileprefix='OUT'):
    """potential.get_fields (potential.py:1243-1288): the Fields of snapshot
    ``simulation_directory + fileprefix + '.' + simulation_name + '.%05i' %
    intime``, centred on the disc (centering=True, mutual_center=True), with
    coefficients accumulated and tables prepared; returns (F, pattern speed,
    rotation frequency) = (F, 0, 0).  transform=True (the reference's
    default) rotates into the bar frame found from ``bar_file`` by
    exptool.analysis.pattern, which is outside this package:
    NotImplementedError."""
    infile = simulation_directory + fileprefix + '.' + simulation_name + '.%05i' % intime
    if transform:
        raise NotImplementedError("get_fields(transform=True) needs the bar pattern of exptool.analysis.pattern; "
                                  "pass transform=False")
    patt = 0.
    rotfreq = 0.
    F = Fields(infile, eof_file, sph_file, model_file, nhalo=nhalo, transform=transform, no_odd=False,
               centering=True, mutual_center=True)
    F.total_coefficients()
    F.prep_tables()
    return F, patt, rotfreq
