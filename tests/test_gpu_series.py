"""Coefficient time series straight from snapshot files: each file's
coefficients equal a per-file compute_coefficients call on the same
particles, and the written EXP coefficient files read back unchanged."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _snapshots(tmp_path, sampler, kind, nfile=3):
    from exptool_gb300.io import snapshot
    files, parts = [], []
    for i in range(nfile):
        x, y, z, m = sampler(2000 + 500 * i, seed=40 + i)
        comp = {"m": m, "x": x, "y": y, "z": z}
        for k in ("vx", "vy", "vz", "potE"):
            comp[k] = np.zeros_like(m)
        if kind == "psp":
            p = str(tmp_path / f"OUT.run.{i:05d}")
            snapshot.write_psp(p, 0.5 * i, {"halo": comp}, float_len=8 if i % 2 == 0 else 4)
        else:
            p = str(tmp_path / f"SPL.run.{i:05d}")
            snapshot.write_spl(p, 0.5 * i, {"halo": comp}, nsub=2, float_len=8)
        files.append(p)
        parts.append((x, y, z, m) if (kind == "spl" or i % 2 == 0) else
                     tuple(a.astype(np.float32).astype(np.float64) for a in (x, y, z, m)))
    return files, parts


@pytest.mark.parametrize("kind", ["psp", "spl"])
def test_sl_series_matches_per_file_calls(tmp_path, kind):
    from exptool_gb300.basis import spheresl
    from exptool_gb300.io import outcoef
    from exptool_gb300.io.particle import ParticleData
    from exptool_gb300.tables.samplers import hernquist_sample
    cache, model = os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model")
    files, parts = _snapshots(tmp_path, hernquist_sample, kind)
    out = str(tmp_path / "outcoef.halo")
    T, ec = spheresl.compute_coefficients_series(files, "halo", cache, model, outfile=out, reader=kind)
    assert np.array_equal(T, 0.5 * np.arange(len(files)))
    for i, p in enumerate(parts):
        ref = spheresl.compute_coefficients_solitary(ParticleData(*p), cache, model)
        assert np.max(np.abs(ec[i] - ref)) <= 1e-12 * np.max(np.abs(ref)), i
    O = outcoef.OutCoef(out)
    assert O.basis == "SphereSL" and np.array_equal(O.T, T) and np.array_equal(O.coefs, ec)


def test_eof_series_matches_per_file_calls(tmp_path):
    from exptool_gb300.basis import eof
    from exptool_gb300.io import outcoef
    from exptool_gb300.io.particle import ParticleData
    from exptool_gb300.tables.samplers import disc_sample
    path = os.path.join(GOLDEN, "eof_c1.cache")
    files, parts = _snapshots(tmp_path, disc_sample, "psp")
    out = str(tmp_path / "outcoef.star")
    T, c = eof.compute_coefficients_series(files, "halo", path, outfile=out)
    for i, p in enumerate(parts):
        E = eof.compute_coefficients(ParticleData(*p), path, verbose=0)
        assert np.max(np.abs(c[i, 0] - E.cos)) <= 1e-12 * np.max(np.abs(E.cos)), i
        assert np.max(np.abs(c[i, 1] - E.sin)) <= 1e-12 * np.max(np.abs(E.cos)), i
    O = outcoef.OutCoef(out)
    assert O.basis == "Cylinder" and np.array_equal(O.coefs, c)
