"""EXP coefficient time series (outcoef files) against the reference's own
readers (tests/golden/outcoef.npz, made by tests/golden/make_golden.py)."""
import os

import numpy as np

from tests.conftest import GOLDEN

FOLDER = os.path.join(GOLDEN, "outcoef")


def _g():
    return np.load(os.path.join(GOLDEN, "outcoef.npz"))


def test_outcoef_layouts_match_reference():
    from exptool_gb300.io import outcoef
    g = _g()
    for name in ("sl_new", "sl_old", "cyl_new", "cyl_old"):
        O = outcoef.OutCoef(os.path.join(FOLDER, name))
        assert O.basis == str(g[f"{name}/basis"])
        assert np.array_equal(O.T, g[f"{name}/T"]), name
        assert O.coefs.shape == g[f"{name}/coefs"].shape
        assert np.array_equal(O.coefs, g[f"{name}/coefs"]), name


def test_repackaging_matches_reference():
    from exptool_gb300.io import outcoef
    g = _g()
    S = outcoef.OutCoef(os.path.join(FOLDER, "sl_new"))
    S._repackage_spherical_coefficients()
    assert np.array_equal(S.C[2][1]["sin"][3], g["sl_new/C_2_1_sin_3"])
    assert np.array_equal(S.C[3][0]["cos"][4], g["sl_new/C_3_0_cos_4"])
    assert "sin" not in S.C[3][0]
    C = outcoef.OutCoef(os.path.join(FOLDER, "cyl_new"))
    C._repackage_cylindrical_coefficients()
    assert np.array_equal(C.C[4]["sin"][2], g["cyl_new/C_4_sin_2"])
    d = C._repackage_cylindrical_coefficients_compatibility()
    assert np.array_equal(np.array(sorted(d)), g["cyl_new/dict_times"])
    assert np.array_equal(d[0.75].cos, g["cyl_new/dict_cos_at_0.75"])
    assert d[0.75].mmax == 6 and d[0.75].nmax == 11


def test_basis_level_readers_match_reference():
    from exptool_gb300.basis import eof, spheresl
    g = _g()
    T, c = eof.read_binary_eof_coefficients(os.path.join(FOLDER, "cyl_old"))
    assert np.array_equal(T, g["eof_read_binary/T"]) and np.array_equal(c, g["eof_read_binary/coefs"])
    d = eof.read_binary_eof_coefficients_dict(os.path.join(FOLDER, "cyl_old"))
    assert np.array_equal(np.array(sorted(d)), g["eof_read_binary_dict/times"])
    assert np.array_equal(d[12.5].sin, g["eof_read_binary_dict/sin_at_12.5"])
    T, c = spheresl.read_binary_sl_coefficients(os.path.join(FOLDER, "sl_old"))
    assert np.array_equal(T, g["spheresl_read_binary/T"]) and np.array_equal(c, g["spheresl_read_binary/coefs"])


def test_writers_round_trip_and_cylcoefs(tmp_path):
    from exptool_gb300.io import outcoef
    rng = np.random.default_rng(3)
    T = np.linspace(0, 1, 4)
    cy = rng.normal(size=(4, 2, 3, 5))
    cy[:, 1, 0] = 0
    p = str(tmp_path / "cyl")
    outcoef.write_new_cylinder(p, T, cy)
    cc = outcoef.CylCoefs(p)
    assert cc.mmax == 3 and cc.norder == 5 and np.array_equal(cc.numt, T)
    cc.normalise()
    assert np.allclose(cc.CylNormCoefs[:, 0, 0, 0], 1.0)
    assert np.allclose(cc.total_order_amplitude() ** 2, cc.total_order_power())
