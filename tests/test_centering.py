"""Fields.total_coefficients centring against the reference (centres and
the centred particles it hands to the accumulators; no GPU: the
accumulators are replaced by recorders, as when the fixture was made)."""
import os

import numpy as np

from tests.conftest import GOLDEN


class _Data:
    def __init__(self, x, y, z, m, time=None):
        self.data = {"x": x, "y": y, "z": z, "m": m}
        self.time = time


def _inputs():
    from exptool_gb300.tables.samplers import disc_sample, hernquist_sample
    rng = np.random.default_rng(41)
    dx, dy, dz, dm = disc_sample(12000, seed=42)
    dm = dm * rng.uniform(0.5, 1.5, dm.size)
    dx, dy, dz = dx + 0.03, dy - 0.02, dz + 0.01
    hx, hy, hz, hm = hernquist_sample(15000, seed=43)
    hx = hx - 0.05
    return _Data(dx, dy, dz, dm, 1.5), _Data(hx, hy, hz, hm)


def test_centering_matches_reference(monkeypatch):
    from exptool_gb300.basis import eof, potential, spheresl
    g = np.load(os.path.join(GOLDEN, "centering.npz"))
    seen = {}

    def rec(key):
        def f(P, *a, **k):
            seen[key] = np.stack([P.xpos, P.ypos, P.zpos, P.mass])
            return eof.EOF_Object() if key == "disk" else spheresl.SL_Object()
        return f

    monkeypatch.setattr(potential.eof, "compute_coefficients", rec("disk"))
    monkeypatch.setattr(potential.spheresl, "compute_coefficients", rec("halo"))
    for mutual, tag in ((False, "separate"), (True, "mutual")):
        disk, halo = _inputs()
        F = potential.Fields("fake", "eof", "sph", "mod", centering=True, mutual_center=mutual, verbose=0)
        F.total_coefficients(disk, halo)
        got = np.array([F.xcen_disk, F.ycen_disk, F.zcen_disk, F.xcen_halo, F.ycen_halo, F.zcen_halo, F.halofac,
                        F.time])
        assert np.array_equal(got, g[tag + "_centers"]), (got, g[tag + "_centers"])
        for key in ("disk", "halo"):
            a = seen[key]
            assert np.array_equal(a[:, :16], g[f"{tag}_{key}_first"])
            sums = np.array([a.sum(axis=1), (a ** 2).sum(axis=1)])
            assert np.allclose(sums, g[f"{tag}_{key}_sums"], rtol=1e-13, atol=0)
