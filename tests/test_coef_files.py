"""Coefficient and field files against files written by the reference
(tests/golden/coef_files.npz, made by tests/golden/make_golden.py): byte
equality of what this package writes, and restoring reference-written files.
Host-side I/O only; no GPU."""
import hashlib
import os

import numpy as np

from tests.conftest import GOLDEN


def _golden():
    return np.load(os.path.join(GOLDEN, "coef_files.npz"))


def _sl_objects():
    from exptool_gb300.basis import spheresl
    sl = np.load(os.path.join(GOLDEN, "sl_c2.npz"))
    objs = []
    for t, ec in ((0.5, sl["expcoef"]), (1.25, sl["expcoef_noodd"])):
        o = spheresl.SL_Object()
        o.filename, o.comp, o.nbodies, o.sph_file, o.model_file = ("OUT.run0.00010", "dark", 207, "sl_c2.cache",
                                                                   "sl_c2.model")
        o.lmax, o.nmax, o.time, o.expcoef = 4, 6, t, ec
        objs.append(o)
    return objs


def _eof_objects():
    from exptool_gb300.basis import eof
    e1 = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    objs = []
    for t, c, s in ((0.5, e1["cos"], e1["sin"]), (1.25, 2.0 * e1["cos"], -e1["sin"])):
        o = eof.EOF_Object()
        o.filename, o.comp, o.nbodies, o.eof_file, o.mmax, o.nmax = "OUT.run0.00010", "star", 3000, "eof_c1.cache", 3, 3
        o.time, o.cos, o.sin = t, c, s
        objs.append(o)
    return objs


def test_sl_coefficient_file_bytes_and_restore(tmp_path):
    from exptool_gb300.basis import spheresl
    g = _golden()
    path = str(tmp_path / "sl.coef")
    for o in _sl_objects():
        spheresl.save_sl_coefficients(path, o)
    assert open(path, "rb").read() == g["sl_bytes"].tobytes()
    ref_path = str(tmp_path / "ref_sl.coef")
    g["sl_bytes"].tofile(ref_path)
    last, dumps = spheresl.restore_sl_coefficients(ref_path)
    assert sorted(dumps.keys()) == list(g["sl_restored_times"])
    objs = _sl_objects()
    for o in objs:
        d = dumps[np.round(np.float32(o.time), 3)]
        assert np.array_equal(d.expcoef, o.expcoef)
        assert d.lmax == 4 and d.nmax == 6 and d.nbodies == 207
        assert d.sph_file == b"sl_c2.cache" and d.comp == b"dark"
    assert np.array_equal(last.expcoef, objs[-1].expcoef)


def test_eof_coefficient_file_bytes_and_restore(tmp_path):
    from exptool_gb300.basis import eof
    g = _golden()
    path = str(tmp_path / "eof.coef")
    for o in _eof_objects():
        eof.save_eof_coefficients(path, o)
    assert open(path, "rb").read() == g["eof_bytes"].tobytes()
    ref_path = str(tmp_path / "ref_eof.coef")
    g["eof_bytes"].tofile(ref_path)
    last, dumps = eof.restore_eof_coefficients(ref_path)
    assert list(dumps.keys()) == list(g["eof_restored_times"])
    for o, d in zip(_eof_objects(), dumps.values()):
        assert np.array_equal(d.cos, o.cos) and np.array_equal(d.sin, o.sin)
        assert d.mmax == 3 and d.nmax == 3 and d.eof_file == b"eof_c1.cache"
    # a truncated trailing dump is skipped, as the reference does
    trunc = str(tmp_path / "trunc.coef")
    g["eof_bytes"][:-40].tofile(trunc)
    last, dumps = eof.restore_eof_coefficients(trunc)
    assert len(dumps) == 1 and np.array_equal(last.cos, _eof_objects()[0].cos)


def _field_instance():
    from exptool_gb300.basis import eof, potential, spheresl
    sl = np.load(os.path.join(GOLDEN, "sl_c2.npz"))
    e1 = np.load(os.path.join(GOLDEN, "eof_c1.npz"))
    F = potential.Fields("OUT.run0.00010", "eof_c1.cache", "sl_c2.cache", "sl_c2.model", verbose=0)
    F.EOF = eof.EOF_Object()
    F.EOF.eof_file, F.EOF.cos, F.EOF.sin = "eof_c1.cache", e1["cos"], e1["sin"]
    F.SL = spheresl.SL_Object()
    F.SL.sph_file, F.SL.model_file, F.SL.expcoef = "sl_c2.cache", "sl_c2.model", sl["expcoef"]
    F.halofac = 0.75
    F.time = 2.5
    return F


def test_save_field_matches_reference_bytes(tmp_path, monkeypatch):
    g = _golden()
    monkeypatch.chdir(GOLDEN)
    F = _field_instance()
    path = str(tmp_path / "field.bin")
    F.save_field(path)
    raw = open(path, "rb").read()
    assert len(raw) == int(g["field_size"])
    assert hashlib.sha256(raw).digest() == g["field_sha256"].tobytes()
