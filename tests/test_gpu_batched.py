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


def test_batched_tensor_core_vs_fp64_and_oracle(l6_table, tmp_path, monkeypatch):
    """Tensor-core engine (tcgen05, BF16 operands, FP32 accumulation in tensor
    memory, FP64 window sums and contraction) against the FP64 single-snapshot
    path on the same FP32-rounded particles, and against the oracle on a small
    snapshot.  BF16 rounds each operand to 2^-9 relative, so one particle's
    contribution carries up to ~4e-3 relative error: normwise <= 5e-3 for any
    snapshot, and <= 5e-4 for snapshots of 1e4 particles or more, where the
    independent roundings average out.  Empty and one-particle snapshots,
    work items of several K-tiles, every stage count and repeated calls
    (the operand tiles keep the last call's contents) are covered; the
    kernels' error flag stays clear."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import spheresl
    from exptool_gb300.tables.samplers import hernquist_sample
    from oracle import sl as osl
    monkeypatch.setenv("XT_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    cache, model = l6_table
    sizes = [10000, 3000, 250000, 77777, 1, 0, 120000, 40000]
    snaps = [hernquist_sample(n, 700 + i) for i, n in enumerate(sizes)]
    xyzm = np.concatenate([np.stack(s, axis=1) for s in snaps], axis=0).astype(np.float32)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    table = spheresl.table_from_files(cache, model)
    xd = torch.from_numpy(xyzm).cuda().contiguous()
    refs = []
    for i in range(len(sizes)):
        blk = xd[int(offs[i]):int(offs[i + 1])].double()
        refs.append(dev.to_host(table.accumulate(*(blk[:, k].contiguous() for k in range(4)))) if sizes[i] else None)
    # residency: fewer operand stages never fit fewer CTAs on an SM
    for sp in (1, 2):
        res = [table.batched_tc_residency(st, sp) for st in (1, 2, 3)]
        assert res[0] >= res[1] >= res[2] >= 1, (sp, res)
    results = []
    for chunk, stages, ctas, sp in ((16384, 2, 0, 1), (512, 3, 0, 1), (128, 2, 1, 1), (4096, 1, 0, 1), (4096, 1, 2, 1),
                                    (4096, 1, 0, 2), (512, 2, 1, 2)):
        got = dev.to_host(table.accumulate_batched_tc(xd, offs, chunk=chunk, stages=stages, ctas_per_sm=ctas,
                                                      threads_per_particle=sp))
        dev.batched_tc_status()
        results.append(got)
        for i, n in enumerate(sizes):
            if n == 0:
                assert not np.any(got[i]), (chunk, i)
                continue
            e = norm_err(got[i], refs[i])
            assert e <= 5e-3, (chunk, stages, ctas, sp, i, e)
            if n >= 10000:
                assert e <= 5e-4, (chunk, stages, ctas, sp, i, e)
    # the same sums whatever the work-item size or launch width, to FP32 summation
    # order (slots inside a bucket come from shared-memory atomics, so the order of
    # the particles within a work item may differ between calls)
    for i, n in enumerate(sizes):
        if n >= 10000:
            assert norm_err(results[1][i], results[0][i]) <= 1e-5
            assert norm_err(results[4][i], results[3][i]) <= 1e-5
            assert norm_err(results[5][i], results[3][i]) <= 1e-5      # two threads per particle
            assert norm_err(results[6][i], results[3][i]) <= 1e-5
    # against the oracle on a small snapshot (FP32-rounded inputs)
    t = osl.load_table(cache, model)
    x, y, z, m = (xyzm[offs[1]:offs[2], k].astype(np.float64) for k in range(4))
    assert norm_err(results[0][1], osl.compute_coefficients_solitary(x, y, z, m, t)) <= 5e-3
    # the public entry point with autotuned item size and stages; no_odd zeroes odd-l rows
    pub = spheresl.compute_coefficients_batched((xyzm, offs), cache, model, engine="tensor")
    assert norm_err(pub[2], refs[2]) <= 5e-4
    assert os.path.exists(tmp_path / "tune.json")
    odd = spheresl.compute_coefficients_batched((xyzm, offs), cache, model, engine="tensor", no_odd=True,
                                                autotune=False)
    for l in (1, 3, 5):
        assert not np.any(odd[:, l * l:(l + 1) * (l + 1)])
    assert norm_err(odd[2][0:1], refs[2][0:1]) <= 5e-4


@pytest.mark.parametrize("lmax,nmax,cmap", [(4, 10, 1), (8, 12, 2)])
def test_batched_tensor_core_other_tables(tmp_path_factory, lmax, nmax, cmap):
    """The tensor-core engine on the other instantiations of its tile (lmax 4:
    N = 32; lmax 8: N = 96) and on the rational radial map (cmap 1), with one
    and two threads per particle and one or two stages, against the FP64
    single-snapshot path on the same FP32-rounded particles (the BF16 bounds of
    the lmax 6 test).  Two threads per particle order the rows by the parity
    of m; the rows come back to their places through the permutation table."""
    import torch
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import spheresl
    from exptool_gb300.tables.samplers import hernquist_sample
    from exptool_gb300.tables.sl_solver import make_hernquist_sl
    d = str(tmp_path_factory.mktemp(f"sl{lmax}c{cmap}"))
    cache, model = make_hernquist_sl(d, lmax=lmax, nmax=nmax, numr=1200, rmin=1e-3, rmax=100.0, cmap=cmap,
                                     tag=f"l{lmax}c{cmap}")
    sizes = [30000, 700, 52000]
    snaps = [hernquist_sample(n, 900 + i) for i, n in enumerate(sizes)]
    xyzm = np.concatenate([np.stack(s, axis=1) for s in snaps], axis=0).astype(np.float32)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    table = spheresl.table_from_files(cache, model)
    xd = torch.from_numpy(xyzm).cuda().contiguous()
    refs = []
    for i in range(len(sizes)):
        blk = xd[int(offs[i]):int(offs[i + 1])].double()
        refs.append(dev.to_host(table.accumulate(*(blk[:, k].contiguous() for k in range(4)))))
    got = {}
    for sp in (1, 2):
        for stages in (1, 2):
            out = dev.to_host(table.accumulate_batched_tc(xd, offs, chunk=8192, stages=stages,
                                                          threads_per_particle=sp))
            dev.batched_tc_status()
            got[sp, stages] = out
            for i, n in enumerate(sizes):
                e = norm_err(out[i], refs[i])
                assert e <= (5e-4 if n >= 10000 else 5e-3), (lmax, cmap, sp, stages, i, e)
    for i, n in enumerate(sizes):
        if n >= 10000:
            assert norm_err(got[2, 1][i], got[1, 1][i]) <= 1e-5, (lmax, i)
