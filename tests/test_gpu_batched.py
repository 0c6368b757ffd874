"""Batched (many-snapshot, one persistent launch) spherical accumulation:
mixed precision against the FP64 single-snapshot path, per snapshot, and
against the oracle on small snapshots; the autotuner's choice is cached.

Tolerances of the mixed (FP32 per particle) path: normwise over all rows
max|dc|/max|c| <= 2e-6 (FP32 rounding of each particle's contribution,
relative to the largest, monopole, coefficient), and <= 5e-4 within each l
block (the odd-l blocks of a spherical sample are at noise level, so the same
absolute error is large relative to them)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def norm_err(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def block_err(a, b, lmax):
    worst, row = 0.0, 0
    for l in range(lmax + 1):
        blk = slice(row, row + 2 * l + 1)
        s = np.max(np.abs(b[blk]))
        worst = max(worst, np.max(np.abs(a[blk] - b[blk])) / s if s > 0 else 0.0)
        row += 2 * l + 1
    return worst


@pytest.fixture(scope="module")
def l6_table(tmp_path_factory):
    from exptool_gb300.tables.sl_solver import make_hernquist_sl
    d = str(tmp_path_factory.mktemp("sl6"))
    return make_hernquist_sl(d, lmax=6, nmax=20, numr=2000, rmin=1e-3, rmax=100.0, cmap=2, tag="l6n20")


def test_batched_vs_fp64_per_snapshot(l6_table, tmp_path, monkeypatch):
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import spheresl
    from exptool_gb300.tables.samplers import hernquist_sample
    from oracle import sl as osl
    monkeypatch.setenv("XT_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    cache, model = l6_table
    sizes = [10000, 3000, 250000, 77777, 1, 0, 120000, 40000]
    snaps = [hernquist_sample(n, 500 + i) for i, n in enumerate(sizes)]

    class H:
        def __init__(self, x, y, z, m):
            self.xpos, self.ypos, self.zpos, self.mass = x, y, z, m

    got = spheresl.compute_coefficients_batched([H(*s) for s in snaps], cache, model)
    assert got.shape == (len(sizes), 49, 20)
    assert os.path.exists(tmp_path / "tune.json")
    table = spheresl.table_from_files(cache, model)
    for i, (x, y, z, m) in enumerate(snaps):
        # FP64 reference on the same (FP32-rounded) inputs
        xf, yf, zf, mf = (a.astype(np.float32).astype(np.float64) for a in (x, y, z, m))
        if xf.size == 0:
            assert not np.any(got[i])
            continue
        ref = dev.to_host(table.accumulate(*(dev.to_dev(a) for a in (xf, yf, zf, mf))))
        assert norm_err(got[i], ref) < 2e-6, (i, norm_err(got[i], ref))
        assert block_err(got[i], ref, 6) < 5e-4, (i, block_err(got[i], ref, 6))
    # oracle on a small snapshot
    t = osl.load_table(cache, model)
    x, y, z, m = (a.astype(np.float32).astype(np.float64) for a in snaps[1])
    assert norm_err(got[1], osl.compute_coefficients_solitary(x, y, z, m, t)) < 2e-6
    # explicit launch shapes give the same sums up to FP32 rounding
    again = spheresl.compute_coefficients_batched([H(*s) for s in snaps], cache, model, chunk=4096, threads=256)
    for i in range(len(sizes)):
        if sizes[i]:
            assert norm_err(again[i], got[i]) < 2e-6
    assert torch.cuda.is_available()
