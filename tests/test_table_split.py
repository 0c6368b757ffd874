"""The fused EOF paths read each FP64 table entry t as hi = FP32 rounding of t
plus a 16-bit remainder k = round((t - hi) / 2^(e-38)), e the exponent of hi
(`lo16_encode` / `lo16_decode` in csrc/xt_df.cuh).  This restates that
encoding in NumPy and checks, on the golden EOF tables and on edge values,
that |k| <= 2^14 (it fits 16 bits) and that hi + k 2^(e-38) is t to 2^-39
relative, the bound the fused FP64 path's error budget rests on."""
import os

import numpy as np

from tests.conftest import GOLDEN

SHIFT = 38


def lo16_encode(t):
    t = np.asarray(t, dtype=np.float64)
    hi = t.astype(np.float32)
    hb = (hi.view(np.uint32) >> 23) & 0xFF                # biased exponent of hi
    ok = (hb >= SHIFT + 1) & (hb != 0xFF)
    r = t - hi.astype(np.float64)                          # exact
    k = np.where(ok, np.rint(np.ldexp(r, (127 + SHIFT - hb.astype(np.int64)))), 0.0)
    return hi, k


def lo16_decode(hi, k):
    hb = (hi.view(np.uint32) >> 23) & 0xFF
    scale_bits = np.maximum(hb.astype(np.int64) - SHIFT, 0).astype(np.uint32) << 23
    scale = scale_bits.view(np.float32)
    lo = (k.astype(np.float32) * scale).astype(np.float32)   # exact: |k| < 2^24
    return hi, lo


def check(t):
    hi, k = lo16_encode(t)
    assert np.all(np.abs(k) <= 2 ** 14)
    h, lo = lo16_decode(hi, k)
    back = h.astype(np.float64) + lo.astype(np.float64)
    big = np.abs(hi) >= 2.0 ** -88
    err = np.abs(back - t)
    assert np.all(err[big] <= 2.0 ** -39 * np.abs(t[big]))
    # below 2^-88 the remainder is dropped: the error is hi's rounding alone
    assert np.all(err[~big] <= 2.0 ** -149 + 2.0 ** -24 * np.abs(t[~big]))
    return float(np.max(err[big] / np.abs(t[big]))) if big.any() else 0.0


def test_golden_tables():
    from exptool_gb300.basis import eof
    for tag in ("c1", "c0"):
        tabs = eof.parse_eof(os.path.join(GOLDEN, f"eof_{tag}.cache"))
        worst = max(check(np.asarray(a, dtype=np.float64).ravel()) for a in tabs if a is not None)
        assert worst <= 2.0 ** -39


def test_edge_values():
    rng = np.random.default_rng(7)
    t = np.concatenate([
        rng.standard_normal(100000) * 10.0 ** rng.uniform(-30, 30, 100000),
        [0.0, -0.0, 1.0, -1.0, 2.0 ** -88, 2.0 ** -89, 1e-300, 3.4e38],
        # values just below powers of two, where hi rounds up to the next binade
        np.nextafter(2.0 ** np.arange(-60, 60), 0.0),
        2.0 ** np.arange(-60, 60) * (1 + 2.0 ** -25),
    ])
    check(t)
