"""Snapshot file -> Fields -> orbit grid, against the reference run on the
same snapshot (tests/golden/run_time.npz, made by make_golden.py run_time):
- ``Fields.total_coefficients()`` with no arguments reads components 'star'
  and 'dark' of its own snapshot (potential.py:98-252), with and without
  centring: time, halofac and centres equal, coefficients <= 1e-10;
- ``potential.get_fields`` (potential.py:1243-1288);
- ``integrate.run_time_mod`` (integrate.py:638-758): the saved field equal in
  size and header, its coefficients <= 1e-10; the orbit text file with the
  same layout (lines, tokens per line, step counts) and every number within
  two float32 units in the last place of the reference's (the orbit array is
  float32 and printed by repr, so values computed to 1e-10 agree to the last
  printed digit except near a float32 rounding boundary).
The snapshot is rebuilt from seeds with platform-independent arithmetic
(tests/golden/run_time_input.py) and its SHA-256 checked against the one the
reference read.
"""
import hashlib
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN
from tests.golden import run_time_input
from tests.test_gpu_golden import block_rel, rel

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture
def run_dir(tmp_path):
    d = str(tmp_path) + "/"
    run_time_input.write_snapshot(d + "OUT.run0.00003")
    return d


def _golden():
    return np.load(os.path.join(GOLDEN, "run_time.npz"))


def _tables():
    return (os.path.join(GOLDEN, "eof_c1.cache"), os.path.join(GOLDEN, "sl_c2.cache"),
            os.path.join(GOLDEN, "sl_c2.model"))


def _check_coefficients(F, g, tag):
    assert rel(F.EOF.cos, g[tag + "_cos"]) <= TOL
    assert rel(F.EOF.sin[1:], g[tag + "_sin"][1:]) <= TOL
    assert block_rel(np.asarray(F.SL.expcoef), g[tag + "_expcoef"], 4) <= TOL


def test_snapshot_is_the_one_the_reference_read(run_dir):
    h = hashlib.sha256(open(run_dir + "OUT.run0.00003", "rb").read()).hexdigest()
    assert h == str(_golden()["snapshot_sha256"])


@pytest.mark.parametrize("tag,centering", [("plain", False), ("separate", True)])
def test_total_coefficients_reads_its_snapshot(run_dir, tag, centering):
    from exptool_gb300.basis import potential
    g = _golden()
    eof_path, cache, model = _tables()
    F = potential.Fields(run_dir + "OUT.run0.00003", eof_path, cache, model, centering=centering,
                         mutual_center=False, verbose=0)
    F.total_coefficients()
    meta = np.array([F.time, F.halofac, F.xcen_disk, F.ycen_disk, F.zcen_disk, F.xcen_halo, F.ycen_halo,
                     F.zcen_halo], dtype=np.float64)
    # centres: NumPy sums, whose order may differ between platforms
    assert np.allclose(meta, g[tag + "_meta"], rtol=1e-13, atol=1e-16), (meta, g[tag + "_meta"])
    _check_coefficients(F, g, tag)


def test_total_coefficients_argument_checks():
    from exptool_gb300.basis import potential
    F = potential.Fields("none", *_tables(), verbose=0)
    with pytest.raises(ValueError):
        F.total_coefficients(disk_particles=object())
    F.transform = True
    with pytest.raises(NotImplementedError):
        F.total_coefficients()


def test_get_fields(run_dir):
    from exptool_gb300.basis import potential
    g = _golden()
    F, patt, rotfreq = potential.get_fields(run_dir, "run0", 3, *_tables(), transform=False)
    meta = np.array([patt, rotfreq, F.time, F.halofac, F.xcen_disk, F.ycen_disk, F.zcen_disk, F.xcen_halo,
                     F.ycen_halo, F.zcen_halo])
    assert np.allclose(meta, g["get_fields_meta"], rtol=1e-13, atol=1e-16), (meta, g["get_fields_meta"])
    _check_coefficients(F, g, "get_fields")
    with pytest.raises(NotImplementedError):
        potential.get_fields(run_dir, "run0", 3, *_tables())      # transform=True by default


def _tokens(text):
    return [line.split(" ") for line in text.split("\n")]


def _compare_orbit_text(text, ref_text, ulps=None, rtol=None):
    """Same lines and tokens per line, same step counts; numbers within
    `ulps` float32 units in the last place, or within rtol of each line's
    largest magnitude.  Returns the fraction of byte-identical tokens."""
    mine, ref = _tokens(text), _tokens(ref_text)
    assert [len(r) for r in mine] == [len(r) for r in ref]
    same = total = 0
    for a, b in zip(mine, ref):
        assert a[0] == b[0] and a[-1] == b[-1] == ""           # step count; trailing space before newline
        fa = np.array([float(t) for t in a[1:-1]], dtype=np.float32)
        fb = np.array([float(t) for t in b[1:-1]], dtype=np.float32)
        if ulps is not None:
            ulp = np.spacing(np.maximum(np.abs(fa), np.abs(fb)))
            assert np.all(np.abs(fa - fb) <= ulps * ulp), np.max(np.abs(fa - fb) / ulp)
        else:
            assert np.all(np.abs(fa - fb) <= rtol * max(np.max(np.abs(fb), initial=0.0), 1e-30))
        same += sum(x == y for x, y in zip(a, b))
        total += len(a)
    return same / max(total, 1)


def test_run_time_mod(run_dir):
    from exptool_gb300.io import coefficients
    from exptool_gb300.utils import integrate
    g = _golden()
    G = run_time_input.GRID
    integrate.run_time_mod(run_dir, "run0", *_tables(), 3, G["rads"], G["vels"], G["nint"], G["dt"], False, -1,
                           -1, 100., 1000, 0, nprocs=2, omegap=G["omegap"], orbitfile=run_dir + "omap.txt",
                           save_field=True, field_file_name=run_dir + "field.dat")
    # saved field: same size and header, coefficients to the parity bar
    assert os.path.getsize(run_dir + "field.dat") == int(g["field_size"])
    rec = coefficients.read_field_record(run_dir + "field.dat")
    for k in ("eof_i", "sl_i", "flags", "time"):
        assert np.array_equal(np.asarray(rec[k]), g["field_" + k]), k
    for k in ("eof_f", "sl_f"):
        assert np.allclose(np.asarray(rec[k]), g["field_" + k], rtol=2 ** -22, atol=0), k
    assert rel(rec["cos"], g["field_cos"]) <= TOL
    assert rel(rec["expcoef"], g["field_expcoef"]) <= TOL
    names = [os.path.basename(bytes(v).decode().rstrip("\x00")) for v in rec["files"]]
    assert names == list(g["field_files"])
    # orbit text: identical layout, numbers within two float32 ulps, almost all byte-equal
    frac = _compare_orbit_text(open(run_dir + "omap.txt").read(), str(g["omap_text"]), ulps=2)
    assert frac >= 0.99, frac


def test_run_time_mod_restored_field(run_dir):
    """field_file given: the field is restored from field_file_name (the
    reference reads the name, not the argument) and the grid agrees with the
    one from the snapshot to 1e-5 (the field file stores the table
    parameters as float32, as the reference's does)."""
    from exptool_gb300.utils import integrate
    G = run_time_input.GRID
    args = (run_dir, "run0", *_tables(), 3, G["rads"], G["vels"], G["nint"], G["dt"], False, -1, -1, 100., 1000, 0)
    integrate.run_time_mod(*args, omegap=G["omegap"], orbitfile=run_dir + "a.txt", save_field=True,
                           field_file_name=run_dir + "field.dat")
    integrate.run_time_mod(*args, omegap=G["omegap"], orbitfile=run_dir + "b.txt", field_file=True,
                           field_file_name=run_dir + "field.dat")
    _compare_orbit_text(open(run_dir + "b.txt").read(), open(run_dir + "a.txt").read(), rtol=1e-5)
