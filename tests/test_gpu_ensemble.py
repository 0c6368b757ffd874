"""Orbit ensembles (``integrate.Ensemble`` / ``leapfrog_ensemble``) on the GPU.

The ensemble advances many orbits with the same ``xt_leapfrog`` kernel that
``leapfrog_integrate`` uses for one orbit (integrate.py:53-190), in chunks of
steps, optionally captured once into a CUDA graph and replayed.  Checked here:
- FP64 final states and energies against the reference's own orbits (golden
  ``fields.npz``, made by exptool's leapfrog_integrate) at <= 1e-9, the
  single-orbit golden bar;
- each ensemble orbit equal bit for bit to a single-orbit integration;
- graph replay equal bit for bit to direct launches, also after ``reset`` and a
  second replay, with nint not a multiple of the chunk;
- FP32 forces with FP64 kick/drift within a stated bound of FP64;
- ``energy_drift`` equal to max |E(t) - E0| / |E0| over the golden trajectory.
"""
import numpy as np
import pytest

from tests.test_gpu_golden import make_fields, rel

pytestmark = pytest.mark.gpu

GOLDEN_ORBITS = [([1.0, 0.0, 0.05], [0.0, 0.55, 0.02], 0.0, False, 1000, False),
                 ([0.3, -1.2, 0.0], [0.4, 0.1, 0.0], 0.2, True, 1000, False),
                 ([2.5, 0.5, -0.1], [-0.1, -0.4, 0.05], -0.15, False, 1, True)]


def _random_orbits(n, seed):
    rng = np.random.default_rng(seed)
    R = rng.uniform(0.2, 4.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    z = rng.normal(0.0, 0.05, n)
    vc = 0.6 / np.sqrt(1.0 + 0.2 * R)
    vR = rng.normal(0.0, 0.1, n) * vc
    vp = vc * (1.0 + rng.normal(0.0, 0.1, n))
    vz = rng.normal(0.0, 0.05, n)
    c, s = np.cos(ph), np.sin(ph)
    pos = np.stack([R * c, R * s, z], axis=1)
    vel = np.stack([vR * c - vp * s, vR * s + vp * c, vz], axis=1)
    return pos, vel


def test_ensemble_matches_golden_orbits():
    """Each golden orbit as a one-orbit ensemble (its own rotation and apse
    settings), direct and graph-replayed: final state = the reference's last
    row, energy drift = the one of the reference trajectory."""
    from exptool_gb300.utils import integrate
    F, g = make_fields()
    for k, (ip, iv, rf, _force, apmax, apse) in enumerate(GOLDEN_ORBITS):
        F.reset_field_parameters()
        nint = g[f"orbit{k}_T"].size
        for graph in (False, True):
            st = integrate.leapfrog_ensemble(F, 60, 0.02, [ip], [iv], rotfreq=rf, precision="f64", chunk=7,
                                             graph=graph, apse=apse, ap_max=apmax)
            nstep = int(st["nstep"][0])
            assert nstep == nint, (k, nstep, nint)
            for key, gk in (("x", "X"), ("y", "Y"), ("z", "Z"), ("vx", "VX"), ("vy", "VY"), ("vz", "VZ"),
                            ("pot", "P")):
                ref = g[f"orbit{k}_{gk}"]
                d = abs(st[key][0] - ref[nstep - 1]) / max(np.max(np.abs(ref)), 1e-300)
                assert d <= 1e-9, (k, graph, key, d)
            E = 0.5 * (g[f"orbit{k}_VX"] ** 2 + g[f"orbit{k}_VY"] ** 2 + g[f"orbit{k}_VZ"] ** 2) + g[f"orbit{k}_P"]
            drift_ref = np.max(np.abs(E - E[0])) / abs(E[0])
            drift = st["edev"][0] / abs(st["e0"][0])
            assert abs(drift - drift_ref) <= 1e-9, (k, drift, drift_ref)


def test_ensemble_equals_single_orbit_integration():
    """Orbits integrated together (chunks of 7, nint = 60) equal, bit for bit,
    the same orbits integrated one at a time by leapfrog_integrate."""
    from exptool_gb300.utils import integrate
    F, _ = make_fields()
    pos, vel = _random_orbits(6, 11)
    st = integrate.leapfrog_ensemble(F, 60, 0.02, pos, vel, rotfreq=0.1, precision="f64", chunk=7, graph=True)
    for i in range(pos.shape[0]):
        F.reset_field_parameters()
        O = integrate.leapfrog_integrate(F, 60, 0.02, pos[i], vel[i], rotfreq=0.1)
        for key, ok in (("x", "X"), ("y", "Y"), ("z", "Z"), ("vx", "VX"), ("vy", "VY"), ("vz", "VZ"),
                        ("pot", "P")):
            assert st[key][i] == O[ok][-1], (i, key, st[key][i], O[ok][-1])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_graph_replay_is_bit_identical(precision):
    """graph=True (capture, replay) == graph=False (direct launches), and a
    second replay after reset() reproduces the first, with nint = 203 not a
    multiple of chunk = 20 (the last launch asks for more steps than remain)."""
    import torch
    from exptool_gb300.utils import integrate
    F, _ = make_fields()
    pos, vel = _random_orbits(4096, 5)
    ens = integrate.Ensemble(F, pos, vel, 203, 0.01, rotfreq=0.05, precision=precision, chunk=20)
    assert ens.launches_per_run() == 11
    direct = ens.run(graph=False).clone()
    first = ens.run(graph=True).clone()
    ens.reset()
    assert torch.equal(ens.state, ens.init)
    second = ens.run(graph=True).clone()
    torch.cuda.synchronize()
    assert torch.equal(direct, first)
    assert torch.equal(first, second)
    assert bool((first[13] == 203).all())          # every orbit took all steps


def test_fp32_force_within_bound_of_fp64():
    """FP32 forces with FP64 kick/drift stay within 1e-5 (positions,
    velocities, normwise over the ensemble) of the FP64 ensemble after 400
    steps, and both conserve energy to the same order."""
    from exptool_gb300.utils import integrate
    F, _ = make_fields()
    pos, vel = _random_orbits(2048, 9)
    s64 = integrate.leapfrog_ensemble(F, 400, 0.01, pos, vel, precision="f64", chunk=50)
    s32 = integrate.leapfrog_ensemble(F, 400, 0.01, pos, vel, precision="f32", chunk=50)
    for key in ("x", "y", "z", "vx", "vy", "vz"):
        assert rel(s32[key], s64[key]) <= 1e-5, (key, rel(s32[key], s64[key]))
    d64 = s64["edev"] / np.abs(s64["e0"])
    d32 = s32["edev"] / np.abs(s32["e0"])
    assert np.max(np.abs(d32 - d64)) <= 1e-5, np.max(np.abs(d32 - d64))


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_cell_sorted_ensemble_is_bit_identical(precision):
    """Orbits reordered by disc table cell before every chunk (the default,
    xt_orbit_sort) end in the same states, bit for bit, as the unsorted
    ensemble, with and without graph replay; one reordering step is a
    permutation other than the identity that moves whole state columns, and
    xt_orbit_unsort inverts it."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.utils import integrate
    F, _ = make_fields()
    pos, vel = _random_orbits(5000, 7)
    plain = integrate.Ensemble(F, pos, vel, 150, 0.01, rotfreq=0.05, precision=precision, chunk=40, sort=False)
    a = plain.run(graph=False).clone()
    ens = integrate.Ensemble(F, pos, vel, 150, 0.01, rotfreq=0.05, precision=precision, chunk=40, sort=True)
    b = ens.run(graph=False).clone()
    c = ens.run(graph=True).clone()
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert torch.equal(a, c)
    # one reordering step on its own
    n = ens.state.shape[1]
    out = torch.empty_like(ens.state)
    order = torch.empty(n, dtype=torch.int64, device="cuda")
    dev.orbit_sort(ens.cf, ens.state, out, ens._iota, order, ens._ws)
    back = torch.empty_like(ens.state)
    dev.orbit_unsort(out, back, order)
    torch.cuda.synchronize()
    assert torch.equal(torch.sort(order).values, ens._iota)
    assert not torch.equal(order, ens._iota)
    assert torch.equal(back, ens.state)
    assert torch.equal(out, ens.state[:, order])
