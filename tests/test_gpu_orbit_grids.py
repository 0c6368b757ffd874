"""Orbit grids (integrate.integrate_grid, _launchy, _3D, do_integrate_multi)
in one GPU launch against the reference's orbit-by-orbit grids."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.test_gpu_golden import make_fields

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_orbit_grids_match_reference():
    from exptool_gb300.utils import integrate
    g = np.load(os.path.join(GOLDEN, "orbit_grids.npz"))
    F, _ = make_fields()
    rads, vels = np.array([0.6, 1.4]), np.array([0.45, 0.7])
    out = integrate.integrate_grid(rads, vels, F, 30, 1e-4, 0.15, False, -1, -1, 100., 1000, 0)
    assert out.shape == g["grid"].shape and rel(out, g["grid"]) <= 1e-9
    F.reset_field_parameters()
    out = integrate.integrate_grid_launchy(rads, vels, F, 25, 0.01, -0.2, True, 2, 2, 50., 1000, 0)
    assert rel(out, g["grid_launchy"]) <= 1e-9
    F.reset_field_parameters()
    out = integrate.integrate_grid_3D(np.array([1.0]), np.array([0.5, 0.6]), F, 20, 1e-4, 0.0, False, -1, -1, 100.,
                                      1000, np.array([0.05, -0.1]), np.array([0.02]), 0)
    assert out.shape == g["grid_3d"].shape and rel(out, g["grid_3d"]) <= 1e-9
    F.reset_field_parameters()
    multi = integrate.do_integrate_multi(rads, vels, F, 30, 1e-4, 0.15, False, -1, -1, 100., 1000, nprocs=4)
    assert multi.dtype == np.float32 and np.allclose(multi, g["grid"].astype(np.float32), rtol=1e-6, atol=1e-7)
