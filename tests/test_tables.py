"""Table generators and host-side table readers (no GPU)."""
import os

import numpy as np

from exptool_gb300.basis import eof as geof
from exptool_gb300.tables.eof_builder import EOFTables
from exptool_gb300.tables.models import TruncatedHernquist
from exptool_gb300.tables.samplers import disc_cylindrical, hernquist_sample
from exptool_gb300.tables.sl_solver import SLBasis
from exptool_gb300.utils import halo_methods
from oracle import eof as oeof
from oracle import sl as osl
from tests.conftest import GOLDEN


def test_hernquist_sl_eigenvalues():
    b = SLBasis(TruncatedHernquist(), 2, 5, 1e-3, 100.0, nfine=8001)
    # the l = 0, n = 0 function is the background itself: mu = 1, u = const
    assert abs(b.ev[0, 0] - 1.0) < 1e-4
    u = b.u[0, 0]
    assert np.ptp(u) / np.mean(u) < 2e-3
    # Hernquist-Ostriker ladder mu_nl ~ (n+l)(n+l+1)/2 + ... for the lowest modes
    assert np.allclose(b.ev[0, :4], [1, 3, 6, 10], rtol=1e-2)
    assert np.all(np.diff(b.ev, axis=1) > 0)


def test_sl_greens_function_monopole():
    b = SLBasis(TruncatedHernquist(), 0, 24, 1e-3, 100.0, nfine=8001)
    pot, _ = b.pot_and_dpot(0, np.array([0.7, 3.0]))
    # sum_n Phi_n(r) Phi_n(r') -> 1/r_> for l = 0
    assert abs(np.sum(pot[:, 0] * pot[:, 1]) - 1.0 / 3.0) < 5e-3


def test_samplers_deterministic():
    a = hernquist_sample(1000, 3)
    b = hernquist_sample(1000, 3)
    assert all(np.array_equal(u, v) for u, v in zip(a, b))
    r = np.sqrt(a[0] ** 2 + a[1] ** 2 + a[2] ** 2)
    assert r.max() < 100.0 and abs(a[3].sum() - 1.0) < 1e-12
    R, z, phi = disc_cylindrical(2000, 1)
    assert R.max() < 20.0 and np.abs(z).max() < 2.0


def test_host_readers_match_oracle():
    for cmap in (0, 1, 2):
        cache = os.path.join(GOLDEN, f"sl_c{cmap}.cache")
        model = os.path.join(GOLDEN, f"sl_c{cmap}.model")
        got = halo_methods.read_cached_table(cache)
        ref = osl.read_cached_table(cache)
        for g, r in zip(got, ref):
            assert np.array_equal(np.asarray(g), np.asarray(r))
        xi, r, p0, d0 = halo_methods.init_table(model, got[2], got[4], got[5], got[3], got[6])
        t = osl.load_table(cache, model)
        assert np.array_equal(xi, t["xi"]) and np.array_equal(p0, t["p0"]) and np.array_equal(d0, t["d0"])
    for tag in ("c1", "c0"):
        path = os.path.join(GOLDEN, f"eof_{tag}.cache")
        for g, r in zip(geof.parse_eof(path), oeof.parse_eof(path)):
            assert np.array_equal(g, r)
        assert tuple(geof.eof_params(path)) == tuple(oeof.eof_params(path))


def test_eof_builder_roundtrip(tmp_path):
    t = EOFTables(mmax=2, norder=3, numx=10, numy=10, lmax_sph=8, nmax_sph=6, nsample=5000, engine="numpy")
    p = str(tmp_path / "eof.cache")
    t.write(p, dens=True)
    tabs = geof.parse_eof(p)
    assert np.array_equal(tabs[0], t.pot) and np.array_equal(tabs[1], t.rforce)
    assert np.array_equal(tabs[5][1:], t.rforce[1:]) and not np.any(tabs[4][0])
    assert os.path.getsize(p) == 76 + 8 * 4 * 3 * 121 * (3 + 2)


def test_truncated_cache_rejected(tmp_path):
    src = os.path.join(GOLDEN, "sl_c2.cache")
    bad = tmp_path / "bad.cache"
    bad.write_bytes(open(src, "rb").read()[:1000])
    try:
        halo_methods.read_cached_table(str(bad))
    except ValueError as e:
        assert "truncated" in str(e)
    else:
        raise AssertionError("truncated cache accepted")
