"""Velocity-Verlet ("leapfrog") orbit integration on the GPU, with the
interface of ``exptool/utils/integrate.py``.

``leapfrog_integrate`` integrates one orbit exactly as the reference does
(integrate.py:53-190) in a single kernel launch; ``leapfrog_ensemble`` is the
batched form: many independent orbits, one thread each, advanced in chunks of
steps that are captured once into a CUDA graph and replayed.  Forces come from
``Fields`` device fields (FP64, or FP32 with ``precision='f32'``); positions
and velocities are always updated in FP64.
"""
from __future__ import annotations

import numpy as np
import torch

from .. import device as dev
from ..orbits import orbit


def transform(xarray, yarray, thetas):
    """Counter-clockwise planar rotation (integrate.py:34-38)."""
    return np.cos(thetas) * xarray - np.sin(thetas) * yarray, np.sin(thetas) * xarray + np.cos(thetas) * yarray


def clock_transform(xarray, yarray, thetas):
    """Clockwise planar rotation (integrate.py:41-45)."""
    return np.cos(thetas) * xarray + np.sin(thetas) * yarray, -1.0 * np.sin(thetas) * xarray + np.cos(thetas) * yarray


def _new_state(initpos, initvel):
    ip = np.atleast_2d(np.asarray(initpos, dtype=np.float64))
    iv = np.atleast_2d(np.asarray(initvel, dtype=np.float64))
    n = ip.shape[0]
    host = np.zeros((len(dev.STATE_SLOTS), n))
    host[0:3] = ip.T
    host[3:6] = iv.T
    return dev.to_dev(host)


def leapfrog_integrate(FieldInstance, nint, dt, initpos, initvel, rotfreq=0., no_odd=False, halo_l=-1, halo_n=-1,
                       disk_m=-1, disk_n=-1, verbose=0, force=False, ap_max=1000, apse=False):
    """integrate.leapfrog_integrate (integrate.py:53-190): returns an
    ``orbit.Orbits`` dict of the steps taken."""
    F = FieldInstance
    F.set_field_parameters(no_odd=no_odd, halo_l=halo_l, halo_n=halo_n, disk_m=disk_m, disk_n=disk_n)
    sf, cf = F.device_fields()
    nint = int(nint)
    state = _new_state([initpos], [initvel])
    traj = torch.zeros((1, nint, 10), dtype=torch.float64, device=state.device)
    rotc = 2.0 * np.pi * rotfreq
    dev.leapfrog(sf, cf, state, 0, nint, nint, float(dt), rotc=rotc, apse=apse, ap_max=ap_max, traj=traj,
                 halo_l=F._halo_l(), disk_m=F._disk_m(), no_odd=F.no_odd, trig_l=not F.halo_correct_m)
    st = state.cpu().numpy()
    tr = traj[0].cpu().numpy()
    nstep = int(st[13, 0])
    times = np.arange(0, nint, 1) * dt
    barpos = 2.0 * np.pi * rotfreq * times
    O = orbit.Orbits()
    O["T"] = times[0:nstep]
    for k, key in enumerate(("X", "Y", "Z", "VX", "VY", "VZ", "P")):
        O[key] = tr[:nstep, k].copy()
    barpos = barpos[0:nstep]
    if force:
        O["FX"] = tr[:nstep, 7].copy()
        O["FY"] = tr[:nstep, 8].copy()
        O["FZ"] = tr[:nstep, 9].copy()
    if np.min(barpos) < 0.0:
        O["TX"], O["TY"] = transform(O["X"], O["Y"], barpos)
        O["VTX"], O["VTY"] = transform(O["VX"], O["VY"], barpos)
    else:
        O["TX"], O["TY"] = clock_transform(O["X"], O["Y"], barpos)
        O["VTX"], O["VTY"] = clock_transform(O["VX"], O["VY"], barpos)
    return O


def gen_init_step(xpos, vtan, z0=0.0, zvel0=0.):
    """integrate.py:196-214."""
    return [xpos, 0.0, z0], [0.0, vtan, zvel0]


def compute_timestep(FieldInstance, start_pos, start_vel, dyn_res=100., verbose=False):
    """integrate.compute_timestep (integrate.py:217-272), including the
    reference's ``dfz*hfz`` product (:249, :251)."""
    eps = 1.0e-10
    vtot = np.sum(np.array(start_vel) ** 2.) ** 0.5 + eps
    dfx, hfx, dfy, hfy, dfz, hfz, dp, hp = FieldInstance.return_forces_cart(start_pos[0], start_pos[1],
                                                                            start_pos[2])
    dtr = np.sum(np.array(start_pos) * np.array([(dfx + hfx), (dfy + hfy), (dfz * hfz)]))
    atot = ((dfx + hfx) ** 2. + (dfy + hfy) ** 2. + (dfz * hfz) ** 2.0) ** 0.5 + eps
    ptot = np.abs(dp + hp)
    T = {"dtd": 1.0 / np.sqrt(vtot + eps), "dtv": np.sqrt(vtot / (atot + eps)), "dta": ptot / (np.abs(dtr) + eps),
         "dtA": np.sqrt(ptot / (atot * atot + eps))}
    crit = [T[k] for k in T]
    if verbose:
        k = list(T.keys())[int(np.argmin(crit))]
        print("The chosen time criteria is {0:s}, dt={1:6.5f}".format(k, np.min(crit) / dyn_res))
    return np.min(crit) / dyn_res


class Ensemble:
    """Many independent orbits in a frozen ``Fields`` potential.

    State lives on the device as a (16, n) float64 tensor (see
    ``device.STATE_SLOTS``).  ``run`` advances all orbits through steps
    [0, nint) in launches of ``chunk`` steps; with ``graph=True`` the launch
    sequence is captured once as a CUDA graph and replayed.
    """

    def __init__(self, FieldInstance, initpos, initvel, nint, dt, rotfreq=0.0, precision=None, chunk=50,
                 apse=False, ap_max=1000):
        self.F = FieldInstance
        self.precision = FieldInstance.precision if precision is None else precision
        self.sf, self.cf = FieldInstance.device_fields(self.precision)
        self.init = _new_state(initpos, initvel)
        self.state = self.init.clone()
        self.nint, self.dt, self.rotc = int(nint), float(dt), 2.0 * np.pi * float(rotfreq)
        self.chunk = max(1, int(chunk))
        self.apse, self.ap_max = apse, ap_max
        self.graph = None

    def _launch_all(self):
        F = self.F
        step = 0
        while step < self.nint:
            n = self.chunk if step > 0 else min(self.chunk, self.nint)
            dev.leapfrog(self.sf, self.cf, self.state, step, n, self.nint, self.dt, rotc=self.rotc, apse=self.apse,
                         ap_max=self.ap_max, halo_l=F._halo_l(), disk_m=F._disk_m(), no_odd=F.no_odd,
                         trig_l=not F.halo_correct_m)
            step += n

    def launches_per_run(self):
        return (self.nint + self.chunk - 1) // self.chunk

    def reset(self):
        self.state.copy_(self.init)

    def run(self, graph=True):
        """Integrate all orbits from the initial state through nint steps."""
        self.reset()
        if not graph:
            self._launch_all()
            return self.state
        if self.graph is None:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._launch_all()          # warm-up outside capture (lazy module loading)
            torch.cuda.current_stream().wait_stream(s)
            self.reset()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g):
                self._launch_all()
            self.graph = g
            self.reset()
        self.graph.replay()
        return self.state

    def energy_drift(self):
        """Per-orbit max |E(t) - E0| / |E0| over the run (E = v^2/2 + Phi)."""
        st = self.state
        return (st[15] / st[14].abs()).cpu().numpy()


def leapfrog_ensemble(FieldInstance, nint, dt, initpos, initvel, rotfreq=0.0, precision=None, chunk=50, graph=True,
                      apse=False, ap_max=1000):
    """Integrate an ensemble of orbits; returns the final state as a dict of
    NumPy arrays (x y z vx vy vz fx fy fz pot ... nstep e0 edev)."""
    ens = Ensemble(FieldInstance, initpos, initvel, nint, dt, rotfreq, precision, chunk, apse, ap_max)
    st = ens.run(graph=graph).cpu().numpy()
    return {k: st[i] for i, k in enumerate(dev.STATE_SLOTS)}
