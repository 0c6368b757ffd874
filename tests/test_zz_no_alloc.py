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


def _accumulate_pair(lib, table, x, y, z, m, precision, stream):
    """(workspace entry point result, allocation-free result) as host arrays."""
    import torch
    from exptool_gb300 import _lib
    shape = (table.nrow, table.nmax)
    ref = torch.empty(shape, dtype=torch.float64, device="cuda")
    ws = torch.empty(max(1, lib.xt_sph_accumulate_workspace(table.handle)), dtype=torch.uint8, device="cuda")
    n = x.numel() if x is not None else 0
    ptr = (lambda t: t.data_ptr() if t is not None else None)
    rc = lib.xt_sph_accumulate(table.handle, ptr(x), ptr(y), ptr(z), ptr(m), n, 0, precision, ref.data_ptr(),
                               ws.data_ptr(), ws.numel(), stream)
    assert rc == 0, lib.xt_last_error()
    out = torch.full(shape, np.nan, dtype=torch.float64, device="cuda")
    rc = lib.xt_sph_accumulate_noalloc(table.handle, ptr(x), ptr(y), ptr(z), ptr(m), n, 0, precision,
                                       out.data_ptr(), stream)
    assert rc == 0, lib.xt_last_error()
    torch.cuda.synchronize()
    return ref.cpu().numpy(), out.cpu().numpy()


def test_noalloc_mixed_precision_empty_call_and_smaller_table():
    """The FP32 deposit path agrees with xt_sph_accumulate at XT_F32; a call
    with no particles after a non-empty one returns zeros; and a smaller table
    after a larger one returns its own sums (each call clears the part of the
    shared array it uses, so the larger call's leftovers stay out)."""
    import torch
    from exptool_gb300 import _lib
    from exptool_gb300 import device as dev
    from exptool_gb300.basis import spheresl
    from exptool_gb300.tables.samplers import hernquist_sample
    from exptool_gb300.utils import halo_methods

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    cache, model = os.path.join(GOLDEN, "sl_c2.cache"), os.path.join(GOLDEN, "sl_c2.model")
    table = spheresl.table_from_files(cache, model)
    x, y, z, m = (torch.from_numpy(a).cuda() for a in hernquist_sample(40000, 12))
    # FP32 per-particle arithmetic on both entry points
    ref, out = _accumulate_pair(lib, table, x, y, z, m, _lib.XT_F32, stream)
    assert np.all(np.isfinite(out))
    assert _block_rel(out, ref, table.lmax) <= 1e-5
    # n = 0 right after a non-empty call: zeros, not the previous sums
    ref0, out0 = _accumulate_pair(lib, table, None, None, None, None, _lib.XT_F64, stream)
    assert not np.any(ref0) and not np.any(out0)
    # a larger table, then a smaller one (lmax 2 of the same basis)
    ref_big, out_big = _accumulate_pair(lib, table, x, y, z, m, _lib.XT_F64, stream)
    assert _block_rel(out_big, ref_big, table.lmax) <= TOL
    lmax, nmax, numr, cmap, rmin, rmax, scale, _, ev, ef = halo_methods.read_cached_table(cache)
    xi, _, p0, d0 = halo_methods.init_table(model, numr, rmin, rmax, cmap=cmap, scale=scale)
    small = dev.SphTable(2, nmax, numr, cmap, rmin, rmax, scale, xi, p0, d0, ev[:3], ef[:3])
    assert small.nrow * numr < table.nrow * numr
    ref_s, out_s = _accumulate_pair(lib, small, x, y, z, m, _lib.XT_F64, stream)
    assert np.all(np.isfinite(out_s))
    assert _block_rel(out_s, ref_s, 2) <= TOL
    # and the small table's sums are the leading rows of the large table's
    assert _block_rel(out_s, out_big[:small.nrow], 2) <= TOL
