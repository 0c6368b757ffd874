"""Oracle: halo + disc field composition (``exptool/basis/potential.py``) and
the velocity-Verlet integrator (``exptool/utils/integrate.py``), vectorised
over orbits.  TEST INFRASTRUCTURE (see package docstring)."""
from __future__ import annotations

import numpy as np

from . import eof as oeof
from . import sl as osl


class FieldsOracle:
    """Tables and coefficients the way ``Fields.prep_tables`` holds them
    (``potential.py:257-294``)."""

    def __init__(self, sl_table, expcoef, eof_table, cos, sin, halofac=1.0):
        self.sl = sl_table
        self.expcoef = np.asarray(expcoef, dtype=np.float64)
        self.e = eof_table
        self.cos = np.asarray(cos, dtype=np.float64)
        self.sin = np.asarray(sin, dtype=np.float64)
        self.halofac = float(halofac)
        self.reset_field_parameters()

    def set_field_parameters(self, no_odd=False, halo_l=-1, halo_n=-1, disk_m=-1, disk_n=-1):
        """``Fields.set_field_parameters`` (``potential.py:365-377``)."""
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
        self.no_odd = False
        self.halo_use_l = self.sl["lmax"]
        self.halo_use_n = self.sl["nmax"]
        self.disk_use_m = self.e["mmax"]
        self.disk_use_n = self.e["norder"]

    def return_forces_cart(self, x, y, z, rotpos=0.0, correct_m=False):
        """``Fields.return_forces_cart`` (``potential.py:445-497``), vectorised:
        fxdisk, fxhalo, fydisk, fyhalo, fzdisk, fzhalo, diskp, halop+halop0."""
        x = np.atleast_1d(np.asarray(x, dtype=np.float64))
        y = np.atleast_1d(np.asarray(y, dtype=np.float64))
        z = np.atleast_1d(np.asarray(z, dtype=np.float64))
        r2 = (x * x + y * y) ** 0.5 + 1.0e-15
        r3 = (r2 * r2 + z * z) ** 0.5 + 1.0e-15
        costh = z / r3
        phi = np.arctan2(y, x) + rotpos
        e = self.e
        dfr, dfp, dfz, dp, dp0 = oeof.force_eval(
            r2, z, phi, self.cos, self.sin, e["potC"], e["rforceC"], e["zforceC"], e["potS"], e["rforceS"],
            e["zforceS"], rmin=e["XMIN"], dR=e["dX"], zmin=e["YMIN"], dZ=e["dY"], numx=e["numx"], numy=e["numy"],
            MMAX=self.disk_use_m, NMAX=self.disk_use_n, ASCALE=e["ascale"], HSCALE=e["hscale"], CMAP=e["cmap"],
            no_odd=self.no_odd, perturb=False)
        hfr, hft, hfp, hp, hp0 = osl.force_eval(r3, costh, phi, self.halofac * self.expcoef, self.sl,
                                                lmax=self.halo_use_l, nmax=self.halo_use_n, no_odd=self.no_odd,
                                                correct_m=correct_m)
        inner = r3 < np.min(self.sl["xi"])
        hfp = np.where(inner, 0.0, hfp)
        dfp = np.where(inner, 0.0, dfp)
        fxd = dfr * (x / r2) - dfp * (y / (r2 * r2))
        fxh = -1.0 * (hfr * (x / r3) - hft * (x * z / (r3 * r3 * r3))) + hfp * (y / (r2 * r2))
        fyd = dfr * (y / r2) + dfp * (x / (r2 * r2))
        fyh = -1.0 * (hfr * (y / r3) - hft * (y * z / (r3 * r3 * r3))) - hfp * (x / (r2 * r2))
        fzd = dfz
        fzh = -1.0 * (hfr * (z / r3) + hft * ((r2 * r2) / (r3 * r3 * r3)))
        return fxd, fxh, fyd, fyh, fzd, fzh, dp, hp + hp0


def leapfrog_integrate(F, nint, dt, initpos, initvel, rotfreq=0.0, no_odd=False, halo_l=-1, halo_n=-1,
                       disk_m=-1, disk_n=-1, force=False, ap_max=1000, apse=False, correct_m=False):
    """``integrate.leapfrog_integrate`` (``integrate.py:53-190``) for a batch of
    orbits (initpos, initvel: (N, 3)); returns a list of per-orbit dicts with
    the keys of the reference's ``Orbits``."""
    F.set_field_parameters(no_odd=no_odd, halo_l=halo_l, halo_n=halo_n, disk_m=disk_m, disk_n=disk_n)
    ip = np.atleast_2d(np.asarray(initpos, dtype=np.float64))
    iv = np.atleast_2d(np.asarray(initvel, dtype=np.float64))
    n = ip.shape[0]
    times = np.arange(0, nint, 1) * dt
    barpos = 2.0 * np.pi * rotfreq * times
    X = np.zeros((nint, n)); Y = np.zeros((nint, n)); Z = np.zeros((nint, n))
    VX = np.zeros((nint, n)); VY = np.zeros((nint, n)); VZ = np.zeros((nint, n))
    FX = np.zeros((nint, n)); FY = np.zeros((nint, n)); FZ = np.zeros((nint, n))
    PE = np.zeros((nint, n))
    X[0], Y[0], Z[0] = ip[:, 0], ip[:, 1], ip[:, 2]
    VX[0], VY[0], VZ[0] = iv[:, 0], iv[:, 1], iv[:, 2]

    def forces(k, rows):
        dfx, hfx, dfy, hfy, dfz, hfz, dp, hp = F.return_forces_cart(X[k, rows], Y[k, rows], Z[k, rows],
                                                                    rotpos=barpos[k], correct_m=correct_m)
        FX[k, rows] = dfx + hfx
        FY[k, rows] = dfy + hfy
        FZ[k, rows] = dfz + hfz
        PE[k, rows] = dp + hp

    forces(0, np.arange(n))
    n_aps = np.zeros(n, dtype=np.int64)
    nstep = np.full(n, 1, dtype=np.int64)
    active = np.ones(n, dtype=bool)
    step = 1
    while step < nint and np.any(active):
        rows = np.nonzero(active)[0]
        X[step, rows] = X[step - 1, rows] + (VX[step - 1, rows] * dt) + (0.5 * FX[step - 1, rows] * (dt ** 2.0))
        Y[step, rows] = Y[step - 1, rows] + (VY[step - 1, rows] * dt) + (0.5 * FY[step - 1, rows] * (dt ** 2.0))
        Z[step, rows] = Z[step - 1, rows] + (VZ[step - 1, rows] * dt) + (0.5 * FZ[step - 1, rows] * (dt ** 2.0))
        forces(step, rows)
        VX[step, rows] = VX[step - 1, rows] + (0.5 * (FX[step - 1, rows] + FX[step, rows]) * dt)
        VY[step, rows] = VY[step - 1, rows] + (0.5 * (FY[step - 1, rows] + FY[step, rows]) * dt)
        VZ[step, rows] = VZ[step - 1, rows] + (0.5 * (FZ[step - 1, rows] + FZ[step, rows]) * dt)
        if apse and step > 1:
            r0 = X[step - 2, rows] ** 2 + Y[step - 2, rows] ** 2
            r1 = X[step - 1, rows] ** 2 + Y[step - 1, rows] ** 2
            r2 = X[step, rows] ** 2 + Y[step, rows] ** 2
            n_aps[rows] += ((r1 > r0) & (r1 > r2)).astype(np.int64)
        nstep[rows] = step + 1
        active = active & (n_aps < ap_max)
        step += 1
    out = []
    for j in range(n):
        s = nstep[j]
        bp = barpos[:s]
        O = dict(T=times[:s], X=X[:s, j], Y=Y[:s, j], Z=Z[:s, j], VX=VX[:s, j], VY=VY[:s, j], VZ=VZ[:s, j],
                 P=PE[:s, j])
        if force:
            O.update(FX=FX[:s, j], FY=FY[:s, j], FZ=FZ[:s, j])
        if np.min(bp) < 0.0:
            O["TX"], O["TY"] = _transform(O["X"], O["Y"], bp)
            O["VTX"], O["VTY"] = _transform(O["VX"], O["VY"], bp)
        else:
            O["TX"], O["TY"] = _clock_transform(O["X"], O["Y"], bp)
            O["VTX"], O["VTY"] = _clock_transform(O["VX"], O["VY"], bp)
        out.append(O)
    return out


def _transform(x, y, th):
    """``integrate.transform`` (``integrate.py:34-38``)."""
    return np.cos(th) * x - np.sin(th) * y, np.sin(th) * x + np.cos(th) * y


def _clock_transform(x, y, th):
    """``integrate.clock_transform`` (``integrate.py:41-45``)."""
    return np.cos(th) * x + np.sin(th) * y, -1.0 * np.sin(th) * x + np.cos(th) * y


def compute_timestep(F, start_pos, start_vel, dyn_res=100.0):
    """``integrate.compute_timestep`` (``integrate.py:217-272``), including the
    reference's ``dfz*hfz`` product at :249,251."""
    eps = 1.0e-10
    vtot = np.sum(np.array(start_vel) ** 2.0) ** 0.5 + eps
    dfx, hfx, dfy, hfy, dfz, hfz, dp, hp = (float(v[0]) for v in F.return_forces_cart(*start_pos))
    dtr = np.sum(np.array(start_pos) * np.array([(dfx + hfx), (dfy + hfy), (dfz * hfz)]))
    atot = ((dfx + hfx) ** 2.0 + (dfy + hfy) ** 2.0 + (dfz * hfz) ** 2.0) ** 0.5 + eps
    ptot = np.abs(dp + hp)
    T = [1.0 / np.sqrt(vtot + eps), np.sqrt(vtot / (atot + eps)), ptot / (np.abs(dtr) + eps),
         np.sqrt(ptot / (atot * atot + eps))]
    return np.min(T) / dyn_res
