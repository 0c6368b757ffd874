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
    sequence is captured once as a CUDA graph and replayed.  With ``sort``
    (default) the orbits are reordered by disc table cell before every chunk,
    so that neighbouring threads gather from the same cells (xt_orbit_sort),
    and put back in their order at the end: the same results bit for bit.
    """

    def __init__(self, FieldInstance, initpos, initvel, nint, dt, rotfreq=0.0, precision=None, chunk=50,
                 apse=False, ap_max=1000, sort=True):
        self.F = FieldInstance
        self.precision = FieldInstance.precision if precision is None else precision
        self.sf, self.cf = FieldInstance.device_fields(self.precision)
        self.init = _new_state(initpos, initvel)
        self.state = self.init.clone()
        self.nint, self.dt, self.rotc = int(nint), float(dt), 2.0 * np.pi * float(rotfreq)
        self.chunk = max(1, int(chunk))
        self.apse, self.ap_max = apse, ap_max
        self.graph = None
        self.sort = bool(sort)
        if self.sort:
            n = int(self.state.shape[1])
            self._buf = [torch.empty_like(self.state), torch.empty_like(self.state)]
            self._ord = [torch.empty(n, dtype=torch.int64, device=self.state.device) for _ in range(2)]
            self._iota = torch.arange(n, dtype=torch.int64, device=self.state.device)
            self._ws = torch.empty(max(1, dev.orbit_sort_workspace(self.cf, n)), dtype=torch.uint8,
                                   device=self.state.device)

    def _launch_all(self):
        F = self.F
        cur = self.state
        if self.sort:
            k = 0
            self._buf[0].copy_(self.state)
            self._ord[0].copy_(self._iota)
        step = 0
        while step < self.nint:
            n = self.chunk if step > 0 else min(self.chunk, self.nint)
            if self.sort:
                dev.orbit_sort(self.cf, self._buf[k], self._buf[1 - k], self._ord[k], self._ord[1 - k], self._ws)
                k = 1 - k
                cur = self._buf[k]
            dev.leapfrog(self.sf, self.cf, cur, step, n, self.nint, self.dt, rotc=self.rotc, apse=self.apse,
                         ap_max=self.ap_max, halo_l=F._halo_l(), disk_m=F._disk_m(), no_odd=F.no_odd,
                         trig_l=not F.halo_correct_m)
            step += n
        if self.sort:
            dev.orbit_unsort(cur, self.state, self._ord[k])

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
                      apse=False, ap_max=1000, sort=True):
    """Integrate an ensemble of orbits; returns the final state as a dict of
    NumPy arrays (x y z vx vy vz fx fy fz pot ... nstep e0 edev)."""
    ens = Ensemble(FieldInstance, initpos, initvel, nint, dt, rotfreq, precision, chunk, apse, ap_max, sort)
    st = ens.run(graph=graph).cpu().numpy()
    return {k: st[i] for i, k in enumerate(dev.STATE_SLOTS)}


# ---------------------------------------------------------------- orbit grids
def compute_timesteps(FieldInstance, start_pos, start_vel, dyn_res=100.):
    """compute_timestep for many starting points in one force call: (n,)
    step sizes, elementwise the reference's criteria (integrate.py:217-272)."""
    eps = 1.0e-10
    pos = np.atleast_2d(np.asarray(start_pos, dtype=np.float64))
    vel = np.atleast_2d(np.asarray(start_vel, dtype=np.float64))
    vtot = np.sum(vel ** 2., axis=1) ** 0.5 + eps
    dfx, hfx, dfy, hfy, dfz, hfz, dp, hp = (np.asarray(v) for v in
                                            FieldInstance.return_forces_cart(pos[:, 0], pos[:, 1], pos[:, 2]))
    acc = np.stack([dfx + hfx, dfy + hfy, dfz * hfz], axis=1)
    dtr = np.sum(pos * acc, axis=1)
    atot = np.sum(acc ** 2., axis=1) ** 0.5 + eps
    ptot = np.abs(dp + hp)
    crit = np.stack([1.0 / np.sqrt(vtot + eps), np.sqrt(vtot / (atot + eps)), ptot / (np.abs(dtr) + eps),
                     np.sqrt(ptot / (atot * atot + eps))], axis=1)
    return np.min(crit, axis=1) / dyn_res


def _grid_orbits(F, pos, vel, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max):
    """All orbits of a grid in one launch, each with the step
    max(compute_timestep, dt): trajectories (n, nint, 10), steps taken (n,),
    step sizes (n,)."""
    # the reference computes each orbit's step before its leapfrog_integrate
    # call sets the field parameters, so the first orbit's step uses the
    # parameters the instance had on entry
    dt0 = compute_timesteps(F, pos[:1], vel[:1], dyn_res=dyn_res)
    F.set_field_parameters(no_odd=no_odd, halo_l=halo_l, disk_m=disk_m)
    rest = compute_timesteps(F, pos[1:], vel[1:], dyn_res=dyn_res) if pos.shape[0] > 1 else np.zeros(0)
    dts = np.maximum(np.concatenate([dt0, rest]), dt)
    sf, cf = F.device_fields()
    nint = int(nint)
    state = _new_state(pos, vel)
    n = state.shape[1]
    traj = torch.zeros((n, nint, 10), dtype=torch.float64, device=state.device)
    dev.leapfrog(sf, cf, state, 0, nint, nint, 0.0, rotc=2.0 * np.pi * rotfreq, apse=False, ap_max=ap_max,
                 traj=traj, halo_l=F._halo_l(), disk_m=F._disk_m(), no_odd=F.no_odd, trig_l=not F.halo_correct_m,
                 dts=dev.to_dev(dts))
    return dev.to_host(traj), dev.to_host(state[13]).astype(np.int64), dts


def _orbit_rows(tr, nstep, dtime, nint, rotfreq, keys):
    """Rows of one orbit in the integrate_grid layout, zero-padded to nint:
    the Orbits fields of leapfrog_integrate (integrate.py:163-188)."""
    times = np.arange(0, nint, 1) * dtime
    barpos = 2.0 * np.pi * rotfreq * times[:nstep]
    X, Y = tr[:nstep, 0], tr[:nstep, 1]
    VX, VY = tr[:nstep, 3], tr[:nstep, 4]
    if np.min(barpos) < 0.0:
        TX, TY = transform(X, Y, barpos)
    else:
        TX, TY = clock_transform(X, Y, barpos)
    val = {"X": X, "Y": Y, "Z": tr[:nstep, 2], "TX": TX, "TY": TY, "VX": VX, "VY": VY, "VZ": tr[:nstep, 5],
           "T": times[:nstep]}
    out = np.zeros((len(keys), nint))
    for i, k in enumerate(keys):
        out[i, :nstep] = val[k]
    return out


_KEYS_2D = ("X", "Y", "TX", "TY", "VX", "VY", "T")
_KEYS_3D = ("X", "Y", "Z", "TX", "TY", "VX", "VY", "VZ", "T")


def integrate_grid(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, verbose):
    """integrate.integrate_grid (integrate.py:848-884): orbits launched from
    (rad, 0, 0) with velocity (0, vel, 0), step max(compute_timestep, dt);
    array [rads, vels, 7 (X Y TX TY VX VY T), nint].  All orbits in one launch."""
    rads, vels = np.asarray(rads, dtype=np.float64), np.asarray(vels, dtype=np.float64)
    R, V = np.meshgrid(rads, vels, indexing="ij")
    pos = np.stack([R.ravel(), np.zeros(R.size), np.zeros(R.size)], axis=1)
    vel = np.stack([np.zeros(R.size), V.ravel(), np.zeros(R.size)], axis=1)
    return _grid(F, pos, vel, (rads.size, vels.size), nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max,
                 _KEYS_2D)


def integrate_grid_launchy(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, verbose):
    """integrate.integrate_grid_launchy (integrate.py:886-922): launched from
    (0, rad, 0) with velocity (0, vel, 0)."""
    rads, vels = np.asarray(rads, dtype=np.float64), np.asarray(vels, dtype=np.float64)
    R, V = np.meshgrid(rads, vels, indexing="ij")
    pos = np.stack([np.zeros(R.size), R.ravel(), np.zeros(R.size)], axis=1)
    vel = np.stack([np.zeros(R.size), V.ravel(), np.zeros(R.size)], axis=1)
    return _grid(F, pos, vel, (rads.size, vels.size), nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max,
                 _KEYS_2D)


def _grid3(rads, vels, zs, vzs, launch):
    G = np.meshgrid(np.asarray(rads, dtype=np.float64), np.asarray(vels, dtype=np.float64),
                    np.asarray(zs, dtype=np.float64), np.asarray(vzs, dtype=np.float64), indexing="ij")
    R, V, Z, VZ = (g.ravel() for g in G)
    zero = np.zeros(R.size)
    pos = np.stack([R, zero, Z] if launch == "x" else [zero, R, Z], axis=1)
    vel = np.stack([zero, V, VZ], axis=1)
    return pos, vel, G[0].shape


def integrate_grid_3D(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, zs, vzs, verbose):
    """integrate.integrate_grid_3D (integrate.py:760-802): launched from
    (rad, 0, z) with velocity (0, vel, vz); array [rads, vels, zs, vzs, 9
    (X Y Z TX TY VX VY VZ T), nint]."""
    if zs is None or vzs is None:
        print('ERROR: 3D orbit specified, but no z or vz values passed!')
        return None
    pos, vel, shape = _grid3(rads, vels, zs, vzs, "x")
    return _grid(F, pos, vel, shape, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, _KEYS_3D)


def integrate_grid_3D_launchy(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, zs, vzs,
                              verbose):
    """integrate.integrate_grid_3D_launchy (integrate.py:804-846): launched
    from (0, rad, z)."""
    if zs is None or vzs is None:
        print('ERROR: 3D orbit specified, but no z or vz values passed!')
        return None
    pos, vel, shape = _grid3(rads, vels, zs, vzs, "y")
    return _grid(F, pos, vel, shape, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, _KEYS_3D)


def _grid(F, pos, vel, shape, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, keys):
    nint = int(nint)
    tr, nstep, dts = _grid_orbits(F, pos, vel, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max)
    out = np.zeros((pos.shape[0], len(keys), nint))
    for i in range(pos.shape[0]):
        out[i] = _orbit_rows(tr[i], int(nstep[i]), dts[i], nint, rotfreq, keys)
    return out.reshape(tuple(shape) + (len(keys), nint))


def redistribute_arrays(rads, divisions):
    """integrate.redistribute_arrays (integrate.py:440-466): split rads into
    `divisions` contiguous chunks."""
    return np.array_split(np.asarray(rads), divisions)


def re_form_orbit_arrays(array):
    """integrate.re_form_orbit_arrays (integrate.py:469-487): concatenate
    per-chunk grids along the radius axis as float32."""
    return np.concatenate([np.asarray(a) for a in array], axis=0).astype("f4")


def re_form_orbit_arrays_3D(array):
    """integrate.re_form_orbit_arrays_3D (integrate.py:490-509)."""
    return re_form_orbit_arrays(array)


def do_integrate_multi(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, verbose=0,
                       nprocs=-1, threedee=False, zs=None, vzs=None, launch='x'):
    """integrate.do_integrate_multi (integrate.py:290-335): the whole grid in
    one GPU launch (nprocs is accepted and unused); float32 orbit array as
    the reference's re_form_orbit_arrays returns."""
    if threedee:
        if (zs is None) or (vzs is None):
            print('ERROR: 3D orbit specified, but no z or vz values passed!')
            return None
        fn = integrate_grid_3D if launch == 'x' else integrate_grid_3D_launchy
        arr = fn(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, zs, vzs, verbose)
        return re_form_orbit_arrays_3D([arr])
    fn = integrate_grid if launch == 'x' else integrate_grid_launchy
    arr = fn(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, disk_m, dyn_res, ap_max, verbose)
    return re_form_orbit_arrays([arr])


# ---------------------------------------------------------------- orbit text files
def _orbit_line(head, rows):
    """One line as the reference's print calls write it: every token followed
    by a space, then a newline (integrate.py:513-536)."""
    toks = [str(v) for v in head]
    for row in rows:
        toks.extend(str(v) for v in row)
    return "".join(t + " " for t in toks) + "\n"


def print_orbit_array(f, OrbitArray):
    """integrate.print_orbit_array (integrate.py:513-536): per orbit, nsteps,
    R_0, V_0, dT, then the X, Y, TX, TY, VX, VY rows."""
    nsteps = OrbitArray.shape[-1]
    for rad in range(0, OrbitArray.shape[0]):
        for vel in range(0, OrbitArray.shape[1]):
            O = OrbitArray[rad, vel]
            f.write(_orbit_line((nsteps, O[0, 0], O[5, 0], O[-1, 1]), [O[k] for k in range(6)]))


def print_orbit_array_3D(f, OrbitArray):
    """integrate.print_orbit_array_3D (integrate.py:539-568)."""
    nsteps = OrbitArray.shape[-1]
    for rad in range(0, OrbitArray.shape[0]):
        for vel in range(0, OrbitArray.shape[1]):
            for z in range(0, OrbitArray.shape[2]):
                for vz in range(0, OrbitArray.shape[3]):
                    O = OrbitArray[rad, vel, z, vz]
                    f.write(_orbit_line((nsteps, O[0, 0], O[6, 0], O[2, 0], O[7, 0], O[-1, 1]),
                                        [O[k] for k in range(8)]))


def _read_lines(infile, head, keys):
    D = {k: {} for k in head + keys}
    with open(infile, "r") as f:
        for linenum, line in enumerate(f):
            d = [float(q) for q in line.split()]
            npoints = int(d[0])
            for i, k in enumerate(head):
                D[k][linenum] = d[1 + i]
            o = 1 + len(head)
            for i, k in enumerate(keys):
                D[k][linenum] = d[o + i * npoints:o + (i + 1) * npoints]
    return D


def read_integrations(infile):
    """integrate.read_integrations (integrate.py:970-998)."""
    return _read_lines(infile, ["R_0", "V_0", "dT"], ["X", "Y", "TX", "TY", "VX", "VY"])


def read_integrations_3D(infile):
    """integrate.read_integrations_3D (integrate.py:1001-1038)."""
    return _read_lines(infile, ["R_0", "V_0", "Z_0", "VZ_0", "dT"], ["X", "Y", "Z", "TX", "TY", "VX", "VY", "VZ"])


# ---------------------------------------------------------------- snapshot -> orbit grid driver
def run_time_mod(simulation_directory, simulation_name, eof_file, sph_file, model_file, intime, rads, vels, nint, dt,
                 no_odd, halo_l, max_m, dyn_res, ap_max, verbose, nprocs=-1, omegap=-1., orbitfile='',
                 transform=False, save_field=True, field_file_name='', field_file=None, bar_file='', fileprefix='OUT',
                 threedee=False, zs=None, vzs=None, launch='x'):
    """integrate.run_time_mod (integrate.py:638-758): the Fields of snapshot
    ``intime`` (potential.get_fields, or potential.restore_field of
    ``field_file_name`` when ``field_file`` is given, as the reference reads
    the name rather than the argument), optionally saved with save_field
    (default name 'field_file' in the working directory), then an orbit grid
    by do_integrate_multi written with print_orbit_array(_3D) to
    ``orbitfile`` or ``simulation_directory + 'omap_<intime>.txt'``
    ('omap_3D_<intime>.txt' in 3D).  The grid rotates with frequency
    -|omegap| / 2 pi when omegap >= 0, else 0.  transform=True (bar frame,
    exptool.analysis.pattern) is outside this package: NotImplementedError
    (after the reference's own missing-bar-file message and return)."""
    from ..basis import potential
    if verbose:
        print('exptool.integrate.run_time: in directory {}, run {} at output {}, with transform={}'
              .format(simulation_directory, simulation_name, intime, transform))
    if transform:
        if bar_file == '':
            print('error - no bar file supplied for transform')
            return
        raise NotImplementedError("run_time_mod(transform=True) needs the bar pattern of exptool.analysis.pattern")
    patt = 0.
    if field_file is None:
        F, patt, rotfreq = potential.get_fields(simulation_directory, simulation_name, intime, eof_file, sph_file,
                                                model_file, transform=transform, bar_file=bar_file,
                                                fileprefix=fileprefix)
        if save_field:
            if str(field_file_name) != '':
                F.save_field(str(field_file_name))
            else:
                print('saving field file with default name (field_file) to local directory')
                F.save_field('field_file')
    else:
        print('field file supplied! File name:')
        print(field_file_name)
        F = potential.restore_field(str(field_file_name))
    if omegap >= 0.:
        patt = omegap
    rotfreq = -1. * abs(patt / (2. * np.pi))
    if not threedee:
        print('launching from ', launch, ' axis')
        OrbitArray = do_integrate_multi(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, max_m, dyn_res, ap_max,
                                        verbose=verbose, nprocs=nprocs, launch=launch)
        if orbitfile == '':
            print('Saving 2D orbit')
            orbitfile = simulation_directory + 'omap_' + str(intime) + '.txt'
        with open(orbitfile, 'w') as f:
            print_orbit_array(f, OrbitArray)
        return
    if (zs is None) or (vzs is None):
        print('ERROR: 3D orbit specified, but no z or vz values passed!')
        return
    OrbitArray = do_integrate_multi(rads, vels, F, nint, dt, rotfreq, no_odd, halo_l, max_m, dyn_res, ap_max,
                                    verbose=verbose, nprocs=nprocs, threedee=threedee, zs=zs, vzs=vzs, launch=launch)
    if orbitfile == '':
        print('Saving 3D orbit')
        orbitfile = simulation_directory + 'omap_3D_' + str(intime) + '.txt'
    with open(orbitfile, 'w') as f:
        print_orbit_array_3D(f, OrbitArray)
