"""The fused EOF paths read each FP64 table entry t as hi = FP32 rounding of t
plus a 16-bit remainder k = round((t - hi) / 2^(e-38)), e the exponent of hi
(`lo16_encode` / `lo16_unscaled` in csrc/xt_df.cuh: the kernels form
k 2^e and fold the 2^-38 into the other factor of each product).  This
restates that encoding in NumPy and checks, on the golden EOF tables and on
edge values, that |k| <= 2^14 (it fits 16 bits) and that hi + k 2^(e-38) is t
to 2^-39 relative for 2^-88 <= |hi| < 2^113, the bound the fused FP64 path's
error budget rests on; outside that range no remainder is stored."""
import os

import numpy as np

from tests.conftest import GOLDEN

SHIFT = 38


def lo16_encode(t):
    t = np.asarray(t, dtype=np.float64)
    hi = t.astype(np.float32)
    hb = (hi.view(np.uint32) >> 23) & 0xFF                # biased exponent of hi
    ok = (hb >= SHIFT + 1) & (hb < 127 + 113)
    r = t - hi.astype(np.float64)                          # exact
    k = np.where(ok, np.rint(np.ldexp(r, (127 + SHIFT - hb.astype(np.int64)))), 0.0)
    return hi, k


def lo16_decode(hi, k):
    """k 2^e (the device's unscaled remainder, exact) times 2^-38."""
    pow2 = (hi.view(np.uint32) & np.uint32(0x7F800000)).view(np.float32)   # 2^e, 0 for zero/subnormal hi
    unscaled = (k.astype(np.float32) * pow2).astype(np.float32)
    lo = unscaled.astype(np.float64) * 2.0 ** -SHIFT
    return hi, lo


def check(t):
    hi, k = lo16_encode(t)
    assert np.all(np.abs(k) <= 2 ** 14)
    h, lo = lo16_decode(hi, k)
    with np.errstate(invalid="ignore", over="ignore"):
        back = h.astype(np.float64) + lo
    big = (np.abs(hi) >= 2.0 ** -88) & (np.abs(hi) < 2.0 ** 113)
    err = np.abs(back - t)
    assert np.all(err[big] <= 2.0 ** -39 * np.abs(t[big]))
    # outside [2^-88, 2^113) the remainder is dropped: the error is hi's rounding alone
    fin = ~big & np.isfinite(hi)
    assert np.all(err[fin] <= 2.0 ** -149 + 2.0 ** -24 * np.abs(t[fin]))
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
        # either side of 2^113, above which no remainder is stored
        [2.0 ** 112 * 1.7, -(2.0 ** 112) * 1.9, 2.0 ** 113 * (1 + 2.0 ** -30), 2.0 ** 120 / 3],
        # values just below powers of two, where hi rounds up to the next binade
        np.nextafter(2.0 ** np.arange(-60, 60), 0.0),
        2.0 ** np.arange(-60, 60) * (1 + 2.0 ** -25),
    ])
    check(t)
