"""Accuracy of the double-float functions of the FP64 binning (table-driven
log, asinh, and the z map of compatibility.z_to_y at hscale 1) against NumPy's
FP64, through xt_df_eval.  Double-float carries about 2^-47 relative per
operation; the bounds below (2e-14 to 3e-14) leave a few units of that for the
short chains of operations, and are three orders of magnitude inside what the
1e-10 parity bar of the binning's cell offsets needs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eval(fn, x):
    import torch
    from exptool_gb300 import _lib, device as dev
    xd = dev.to_dev(np.ascontiguousarray(x, dtype=np.float64))
    out = torch.empty_like(xd)
    _lib.check(_lib.load().xt_df_eval(int(fn), dev.dptr(xd), dev.dptr(out), xd.numel(), dev.stream_ptr()),
               "xt_df_eval")
    return dev.to_host(out)


def _rel(got, ref):
    return np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)


def _as_pair(x):
    """The input as the kernel sees it: rounded to a float pair (hi, lo),
    about 2^-48 relative; the functions are judged on that value."""
    h = x.astype(np.float32).astype(np.float64)
    return h + (x - h).astype(np.float32).astype(np.float64)


def test_log_table_driven():
    rng = np.random.default_rng(3)
    x = np.concatenate([
        10.0 ** rng.uniform(-30, 30, 200000),
        1.0 + rng.uniform(-1e-3, 1e-3, 20000),                     # near 1: small logs
        1.0 + np.arange(129) / 128.0,                              # the table points
        (1.0 + np.arange(128) / 128.0 + 1.0 / 256.0),              # half-way between them
        2.0 ** np.arange(-120, 121).astype(np.float64),            # powers of two
        np.nextafter(2.0 ** np.arange(-100, 101), 0.0),            # just below them
    ])
    got = _eval(0, x)
    ref = np.log(_as_pair(x))
    far = np.abs(ref) > 1e-3
    assert np.max(np.abs(got - ref)[far] / np.abs(ref[far])) <= 2e-14
    assert np.max(_rel(got[~far], ref[~far])) <= 2e-13         # near 1, relative to a small log
    assert got[np.flatnonzero(x == 1.0)[0]] == 0.0


def test_asinh_series_log_and_large():
    rng = np.random.default_rng(4)
    x = np.concatenate([
        10.0 ** rng.uniform(-12, 6, 200000),
        rng.uniform(0.0, 0.0625, 20000),                           # the series branch
        0.0625 + np.array([-1e-12, 0.0, 1e-12]),                   # the series/log1p boundary
        rng.uniform(0.0625, 0.4, 20000),                           # the log1p branch
        0.4 + np.array([-1e-12, 0.0, 1e-12]),                      # the log1p/log boundary
        16777216.0 * np.array([0.999999, 1.0, 1.000001]),          # the log/large boundary
        10.0 ** rng.uniform(7, 28, 1000),
        np.array([0.0]),
    ])
    got = _eval(1, x)
    ref = np.arcsinh(_as_pair(x))
    nz = x > 0
    assert np.max(_rel(got[nz], ref[nz])) <= 3e-14
    assert got[~nz][0] == 0.0


def test_z_map():
    rng = np.random.default_rng(5)
    mag = np.concatenate([10.0 ** rng.uniform(-12, 4, 200000), [1e-8, 0.336, 0.3355, 0.3365]])
    z = np.concatenate([mag, -mag, [0.0]])
    got = _eval(2, z)
    zr = _as_pair(z)
    ref = (zr / (np.abs(zr) + 1.0e-8)) * np.arcsinh(np.abs(zr))
    nz = z != 0
    assert np.max(_rel(got[nz], ref[nz])) <= 3e-14
    assert got[~nz][0] == 0.0
    assert np.all(np.sign(got[nz]) == np.sign(z[nz]))
