"""The allocation-free spherical accumulation entry point.

xt_sph_accumulate_noalloc exists for callers that cannot allocate device
memory for a workspace (a framework that owns all device memory through its
own pool, a latency-critical loop, a C/cgo/Fortran binding without a device
allocator).  It keeps its deposit grid in a static device array of the
library.  This file checks, through the C ABI, that two calls in a row agree
with the workspace-taking entry point and that tables beyond the array's
limit are refused with a clear error.  It is collected last so that a run that
stops at the first failure has already run every other test.
"""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL = 1e-10   # normwise relative, per l block: FP64 atomics reorder the sums


def _block_rel(a, b, lmax):
    worst, row = 0.0, 0
    for l in range(lmax + 1):
        blk = slice(row, row + 2 * l + 1)
        s = np.max(np.abs(b[blk]))
        d = np.max(np.abs(a[blk] - b[blk]))
        worst = max(worst, d / s if s > 0 else d)
        row += 2 * l + 1
    return worst


def test_noalloc_matches_workspace_entry_point_twice():
    import torch
    from exptool_gb300 import _lib
    from exptool_gb300.basis import spheresl
    from exptool_gb300.tables.samplers import hernquist_sample

    lib = _lib.load()
    cache, model = os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model")
    table = spheresl.table_from_files(cache, model)
    x, y, z, m = (torch.from_numpy(a).cuda() for a in hernquist_sample(50000, 11))
    stream = torch.cuda.current_stream().cuda_stream
    shape = (table.nrow, table.nmax)
    ref = torch.empty(shape, dtype=torch.float64, device="cuda")
    ws = torch.empty(lib.xt_sph_accumulate_workspace(table.handle), dtype=torch.uint8, device="cuda")
    rc = lib.xt_sph_accumulate(table.handle, x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(), x.numel(), 0,
                               _lib.XT_F64, ref.data_ptr(), ws.data_ptr(), ws.numel(), stream)
    assert rc == 0, lib.xt_last_error()
    outs = []
    for _ in range(2):
        out = torch.full(shape, np.nan, dtype=torch.float64, device="cuda")
        rc = lib.xt_sph_accumulate_noalloc(table.handle, x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(),
                                           x.numel(), 0, _lib.XT_F64, out.data_ptr(), stream)
        assert rc == 0, lib.xt_last_error()
        outs.append(out)
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    for out in outs:
        o = out.cpu().numpy()
        assert np.all(np.isfinite(o))
        assert _block_rel(o, r, table.lmax) <= TOL


def test_noalloc_rejects_tables_beyond_the_static_grid():
    from exptool_gb300 import _lib
    from exptool_gb300 import device as dev

    lib = _lib.load()
    lmax, nmax, numr = 8, 2, 4000             # (lmax+1)^2 * numr = 324000 > 262144
    xi = np.log(np.geomspace(1e-3, 1e2, numr))
    big = dev.SphTable(lmax, nmax, numr, 2, 1e-3, 1e2, 1.0, xi, np.ones(numr), np.ones(numr),
                       np.ones((lmax + 1, nmax)), np.ones((lmax + 1, nmax, numr)))
    import torch
    out = torch.zeros(((lmax + 1) ** 2, nmax), dtype=torch.float64, device="cuda")
    rc = lib.xt_sph_accumulate_noalloc(big.handle, None, None, None, None, 0, 0, _lib.XT_F64, out.data_ptr(), None)
    assert rc == -1
    msg = lib.xt_last_error().decode()
    assert "exceeds the static grid" in msg and "262144" in msg
