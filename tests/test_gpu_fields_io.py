"""A restored field evaluates forces like the reference's restored field, and
rotation_curve / resonance_positions match the reference (golden fixtures
from tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.test_coef_files import _field_instance

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_restore_field_forces(tmp_path, monkeypatch):
    from exptool_gb300.basis import potential
    g = np.load(os.path.join(GOLDEN, "coef_files.npz"))
    monkeypatch.chdir(GOLDEN)
    F = _field_instance()
    path = str(tmp_path / "field.bin")
    F.save_field(path)
    monkeypatch.chdir(tmp_path)          # the restored field needs no cache files
    G = potential.restore_field(path)
    px = np.array([0.7, -1.3, 2.2])
    py = np.array([0.4, 0.9, -0.6])
    pz = np.array([0.05, -0.2, 0.3])
    res = np.array([G.return_forces_cart(px[i], py[i], pz[i]) for i in range(3)])
    assert rel(res, g["restored_forces_cart"]) <= 1e-10
    vec = np.array(G.return_forces_cart(px, py, pz)).T
    assert rel(vec, g["restored_forces_cart"]) <= 1e-10


def test_rotation_curve_and_resonances(monkeypatch):
    g = np.load(os.path.join(GOLDEN, "coef_files.npz"))
    monkeypatch.chdir(GOLDEN)
    F = _field_instance()
    F.prep_tables()
    rv = np.linspace(0.05, 3.0, 12)
    F.rotation_curve(rvals=rv)
    for k in ("disk_rotation", "halo_rotation", "total_rotation", "disk_dpdr", "halo_dpdr", "total_dpdr"):
        assert rel(getattr(F, k), g["rc_" + k]) <= 1e-10, k
    F.rotation_curve(rvals=rv, mono=True, angle=0.3)
    assert rel(F.total_rotation, g["rc_mono_angle_total_rotation"]) <= 1e-10
    assert F.halo_use_l == F.lmaxhalo and F.disk_use_m == F.mmax      # restored after mono
    F.resonance_positions(rvals=rv)
    assert rel(F.omega, g["rp_omega"]) <= 1e-10
    assert rel(F.kappa, g["rp_kappa"]) <= 1e-8
