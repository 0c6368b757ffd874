"""Orbit-array text files (integrate.print_orbit_array / read_integrations,
and the 3D forms) against text the reference printed (no GPU)."""
import io
import os

import numpy as np

from tests.conftest import GOLDEN


def test_print_orbit_array_matches_reference_text():
    from exptool_gb300.utils import integrate
    g = np.load(os.path.join(GOLDEN, "orbit_grids.npz"))
    buf = io.StringIO()
    integrate.print_orbit_array(buf, g["grid"])
    assert buf.getvalue() == str(g["grid_text"])
    buf = io.StringIO()
    integrate.print_orbit_array_3D(buf, g["grid_3d"])
    assert buf.getvalue() == str(g["grid_3d_text"])


def test_read_integrations_round_trip(tmp_path):
    from exptool_gb300.utils import integrate
    g = np.load(os.path.join(GOLDEN, "orbit_grids.npz"))
    p = tmp_path / "orbits.txt"
    p.write_text(str(g["grid_text"]))
    D = integrate.read_integrations(str(p))
    grid = g["grid"]
    k = 0
    for i in range(grid.shape[0]):
        for j in range(grid.shape[1]):
            assert D["R_0"][k] == grid[i, j, 0, 0] and D["V_0"][k] == grid[i, j, 5, 0]
            assert D["dT"][k] == grid[i, j, -1, 1]
            for c, key in enumerate(("X", "Y", "TX", "TY", "VX", "VY")):
                assert np.array_equal(np.array(D[key][k]), grid[i, j, c])
            k += 1
    p3 = tmp_path / "orbits3.txt"
    p3.write_text(str(g["grid_3d_text"]))
    D3 = integrate.read_integrations_3D(str(p3))
    g3 = g["grid_3d"].reshape(-1, 9, g["grid_3d"].shape[-1])
    for k in range(g3.shape[0]):
        assert D3["Z_0"][k] == g3[k, 2, 0] and D3["VZ_0"][k] == g3[k, 7, 0]
        for c, key in enumerate(("X", "Y", "Z", "TX", "TY", "VX", "VY", "VZ")):
            assert np.array_equal(np.array(D3[key][k]), g3[k, c])
